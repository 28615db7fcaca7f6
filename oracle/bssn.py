"""Vacuum BSSN right-hand side, projection, Sommerfeld faces, RK4 and constraints.

A NumPy restatement of the reference equations (uwplasma/JAX_BSSN):
  inverse metric by explicit Cholesky       JAX_BSSN/bssn/tensor_algebra.py:20-71
  determinant (closed-form 3x3)             JAX_BSSN/bssn/tensor_algebra.py:74-96
  Christoffel symbols                       JAX_BSSN/bssn/tensor_algebra.py:148-193
  trace / trace-free part                   JAX_BSSN/bssn/tensor_algebra.py:337-381
  dt gamma_tilde, dt W                      JAX_BSSN/bssn/spatial_metric.py:17-106
  shift derivatives / advection / gauge     JAX_BSSN/bssn/shift_and_lapse.py:14-132
  W^2 R_ij and W^2 D_i D_j alpha            JAX_BSSN/bssn/geometry.py:21-186
  dt K, dt A_tilde                          JAX_BSSN/bssn/extrinsic_curvature.py:31-224
  dt Gamma_tilde                            JAX_BSSN/bssn/conformal_connection.py:19-162
  momentum constraint and its derivative    JAX_BSSN/bssn/constraints.py:22-213
  Hamiltonian and auxiliary constraints     JAX_BSSN/bssn/constraints.py:271-412
  Sommerfeld replacement                    JAX_BSSN/evolution/boundaries.py:20-171
  RHS assembly, projection, RK4             JAX_BSSN/evolution/time_evolve.py:30-217

Geometric quantities shared by several equations (inverse metric, metric
derivatives, Christoffel symbols, gauge gradients) are computed once per state.
With kappa == 0 the constraint-damping term is kappa/2*alpha*(...) == 0 and is
skipped, which is exact for finite data.
"""

import numpy as np

from .state import BSSNVariables
from .stencils import D1, D2, D1_upwind, kreiss_oliger, SOMMERFELD

W_FLOOR = 1.0e-12
E = np.einsum


# ----------------------------------------------------------------------------
# pointwise tensor algebra
# ----------------------------------------------------------------------------

def inverse_metric(g):
    """SPD inverse via the explicit Cholesky factor L L^T (tensor_algebra.py:20-71)."""
    g00, g01, g02, g11, g12, g22 = g[0, 0], g[0, 1], g[0, 2], g[1, 1], g[1, 2], g[2, 2]
    l00 = np.sqrt(g00)
    l10 = g01 / l00
    l20 = g02 / l00
    l11 = np.sqrt(g11 - l10 * l10)
    l21 = (g12 - l20 * l10) / l11
    l22 = np.sqrt(g22 - l20 * l20 - l21 * l21)
    m00 = 1.0 / l00
    m10 = -l10 / (l00 * l11)
    m11 = 1.0 / l11
    m20 = (l10 * l21 - l20 * l11) / (l00 * l11 * l22)
    m21 = -l21 / (l11 * l22)
    m22 = 1.0 / l22
    i00 = m00 * m00 + m10 * m10 + m20 * m20
    i01 = m10 * m11 + m20 * m21
    i02 = m20 * m22
    i11 = m11 * m11 + m21 * m21
    i12 = m21 * m22
    i22 = m22 * m22
    return np.stack((np.stack((i00, i01, i02)), np.stack((i01, i11, i12)),
                     np.stack((i02, i12, i22))))


def determinant(g):
    """Closed-form 3x3 determinant, the six Sarrus products in a fixed order."""
    return (g[0, 0] * g[1, 1] * g[2, 2] + g[0, 1] * g[1, 2] * g[2, 0]
            + g[0, 2] * g[1, 0] * g[2, 1] - g[0, 2] * g[1, 1] * g[2, 0]
            - g[0, 0] * g[1, 2] * g[2, 1] - g[0, 1] * g[1, 0] * g[2, 2])


def trace_free(T, g, ginv):
    return T - 1.0 / 3.0 * g * E('ij...,ij...->...', ginv, T)


def christoffel_first(dg):
    """Gamma_ijk = (d_k g_ij + d_j g_ik - d_i g_jk)/2 with dg[k,i,j] = d_k g_ij."""
    return 0.5 * (E('kij...->ijk...', dg) + E('jik...->ijk...', dg) - E('ijk...->ijk...', dg))


def christoffel_second(ginv, chr1):
    return E('im...,mjk...->ijk...', ginv, chr1)


# ----------------------------------------------------------------------------
# shared per-state geometry
# ----------------------------------------------------------------------------

class Geometry:
    """Quantities several equations share, computed once per state."""

    def __init__(self, v, p):
        self.p = p
        self.g = np.asarray(v.conformal_metric)
        self.W = np.asarray(v.conformal_factor)
        self.A = np.asarray(v.traceless_K)
        self.K = np.asarray(v.trace_K)
        self.G = np.asarray(v.conformal_connection)
        self.alpha = np.asarray(v.lapse)
        self.beta = np.asarray(v.shift)
        self.ginv = inverse_metric(self.g)
        self.dg = np.stack([D1(self.g, d, p) for d in range(3)])        # [k,i,j]
        self.chr1 = christoffel_first(self.dg)
        self.chr2 = christoffel_second(self.ginv, self.chr1)
        self.dW = np.stack([D1(self.W, d, p) for d in range(3)])
        self.dalpha = np.stack([D1(self.alpha, d, p) for d in range(3)])
        self.dK = np.stack([D1(self.K, d, p) for d in range(3)])
        # dbeta[i, j] = d_j beta^i (shift_and_lapse.py:14-40)
        self.dbeta = np.stack([np.stack([D1(self.beta[i], j, p) for j in range(3)])
                               for i in range(3)])
        self.div_beta = E('ii...->...', self.dbeta)

    def advect(self, f):
        """beta^i d_i f with sign-selected upwind stencils (shift_and_lapse.py:43-63)."""
        terms = [self.beta[d] * D1_upwind(f, self.beta[d], d, self.p) for d in range(3)]
        return sum(terms)

    def hessian(self, f, df):
        """Second derivatives [i,j] = d_j d_i f, D2 on the diagonal."""
        out = np.zeros((3, 3) + f.shape)
        for i in range(3):
            for j in range(3):
                out[i, j] = D2(f, j, self.p) if i == j else D1(df[i], j, self.p)
        return out


# ----------------------------------------------------------------------------
# curvature sources
# ----------------------------------------------------------------------------

def w2_lapse_hessian(geo):
    """W^2 D_i D_j alpha without inverse powers of W (geometry.py:122-186)."""
    hess = geo.hessian(geo.alpha, geo.dalpha)
    conformal = hess - E('kij...,k...->ij...', geo.chr2, geo.dalpha)
    gradient = (E('i...,j...->ij...', geo.dW, geo.dalpha) + E('j...,i...->ij...', geo.dW, geo.dalpha)
                - E('ij...,mn...,m...,n...->ij...', geo.g, geo.ginv, geo.dW, geo.dalpha))
    return geo.W ** 2 * conformal + geo.W * gradient


def w2_ricci(geo):
    """W^2 R_ij (geometry.py:21-119)."""
    p, g, ginv = geo.p, geo.g, geo.ginv
    term1 = np.zeros_like(g)
    for m in range(3):
        for n in range(3):
            second = D2(g, n, p) if m == n else D1(geo.dg[m], n, p)
            term1 = term1 - 0.5 * (ginv[m, n] * second)
    dG = np.stack([D1(geo.G, d, p) for d in range(3)])               # [d, i] = d_d Gamma^i
    term2 = (E('mi...,jm...->ij...', g, dG) + E('mj...,im...->ij...', g, dG)) / 2.0
    term3 = (E('m...,ijm...->ij...', geo.G, geo.chr1) + E('m...,jim...->ij...', geo.G, geo.chr1)) / 2.0
    term4 = (E('mn...,kmi...,jkn...->ij...', ginv, geo.chr2, geo.chr1)
             + E('mn...,kmj...,ikn...->ij...', ginv, geo.chr2, geo.chr1))
    term5 = E('mn...,kim...,kjn...->ij...', ginv, geo.chr2, geo.chr1)
    ricci = term1 + term2 + term3 + term4 + term5
    ddW = geo.hessian(geo.W, geo.dW)
    DDW = ddW - E('kij...,k...->ij...', geo.chr2, geo.dW)
    lap = E('mn...,mn...->...', ginv, DDW)
    grad2 = E('mn...,m...,n...->...', ginv, geo.dW, geo.dW)
    return geo.W ** 2 * ricci + (geo.W * (DDW + g * lap) - 2.0 * g * grad2)


def momentum_constraint(geo):
    """M_i (constraints.py:22-97)."""
    p = geo.p
    Wf = np.maximum(geo.W, W_FLOOR)
    Bup = E('jk...,ik...->ij...', geo.ginv, geo.A)
    dBup = np.stack([D1(Bup, d, p) for d in range(3)])
    dA = np.stack([D1(geo.A, d, p) for d in range(3)])
    first = E('jij...->i...', dBup)
    second = -0.5 * E('jk...,ijk...->i...', geo.ginv, dA)
    third = -3 * E('ij...,j...->i...', Bup, geo.dW) / Wf
    fourth = -2.0 / 3.0 * geo.dK
    return first + second + third + fourth


def momentum_constraint_derivative(geo):
    """(M_i, d_l M_i) by the product rule, layout dM[i, l] (constraints.py:100-213)."""
    p = geo.p
    Wf = np.maximum(geo.W, W_FLOOR)
    B = E('jk...,ik...->ij...', geo.ginv, geo.A)
    BW = B / Wf
    M = momentum_constraint(geo)
    dB = np.stack([D1(B, d, p) for d in range(3)])
    dA = np.stack([D1(geo.A, d, p) for d in range(3)])
    dginv = np.stack([D1(geo.ginv, d, p) for d in range(3)])
    dBW = np.stack([D1(BW, d, p) for d in range(3)])
    dW, dK = geo.dW, geo.dK
    shape = geo.K.shape
    d2B = np.zeros((3, 3) + B.shape)
    d2A = np.zeros((3, 3) + geo.A.shape)
    d2W = np.zeros((3, 3) + shape)
    d2K = np.zeros((3, 3) + shape)
    for l in range(3):
        for inner in range(3):
            if l == inner:
                d2B[l, inner] = D2(B, l, p)
                d2A[l, inner] = D2(geo.A, l, p)
                d2W[l, inner] = D2(geo.W, l, p)
                d2K[l, inner] = D2(geo.K, l, p)
            else:
                d2B[l, inner] = D1(dB[inner], l, p)
                d2A[l, inner] = D1(dA[inner], l, p)
                d2W[l, inner] = D1(dW[inner], l, p)
                d2K[l, inner] = D1(dK[inner], l, p)
    dM = np.zeros((3, 3) + shape)
    for i in range(3):
        for l in range(3):
            div = np.zeros(shape)
            conf = np.zeros(shape)
            for j in range(3):
                div = div + d2B[l, j, i, j]
                conf = conf + (dBW[l, i, j] * dW[j] + BW[i, j] * d2W[l, j])
            metric = E('jk...,jk...->...', dginv[l], dA[i])
            metric2 = E('jk...,jk...->...', geo.ginv, d2A[l, i])
            dM[i, l] = div - 0.5 * metric - 0.5 * metric2 - 3.0 * conf - 2.0 / 3.0 * d2K[l, i]
    return M, dM


# ----------------------------------------------------------------------------
# evolution equations
# ----------------------------------------------------------------------------

def rhs_conformal_metric(geo):
    g = geo.g
    out = (geo.advect(g) + E('mi...,mj...->ij...', g, geo.dbeta) + E('mj...,mi...->ij...', g, geo.dbeta)
           + -2.0 / 3.0 * g * geo.div_beta + -2.0 * geo.alpha * geo.A)
    return out + kreiss_oliger(g, geo.p)


def rhs_conformal_factor(geo):
    W = geo.W
    out = (geo.advect(W) + 1.0 / 3.0 * geo.alpha * W * geo.K + -(1.0 / 3.0) * W * geo.div_beta)
    return out + kreiss_oliger(W, geo.p)


def rhs_trace_K(geo, hessian_alpha, matter=None):
    alpha, K, A, ginv = geo.alpha, geo.K, geo.A, geo.ginv
    out = (-E('ij...,ij...->...', ginv, hessian_alpha)
           + alpha * E('ij...,kl...,ik...,jl...->...', ginv, ginv, A, A)
           + alpha * K ** 2 / 3.0 + geo.advect(K))
    if matter is not None:
        # + 4 pi alpha (rho + W^2 gt^ij S_ij) (extrinsic_curvature.py:78-87)
        rho, _, S = matter
        Wf = np.maximum(geo.W, W_FLOOR)
        stress_trace = E('ij...,ij...->...', Wf ** 2 * ginv, S)
        out = out + 4.0 * np.pi * alpha * (rho + stress_trace)
    return out + kreiss_oliger(K, geo.p)


def rhs_traceless_A(geo, hessian_alpha, matter=None):
    p, alpha, K, A, g, ginv = geo.p, geo.alpha, geo.K, geo.A, geo.g, geo.ginv
    first = alpha * K * A
    second = -2 * alpha * E('ik...,kl...,lj...->ij...', A, ginv, A)
    source = alpha * w2_ricci(geo) - hessian_alpha
    if matter is not None:
        # - 8 pi alpha W^2 S_ij inside the trace-free part (extrinsic_curvature.py:164-175)
        Wf = np.maximum(geo.W, W_FLOOR)
        source = source - 8.0 * np.pi * alpha * Wf ** 2 * matter[2]
    third = trace_free(source, g, ginv)
    fourth = geo.advect(A)
    fifth = E('mi...,mj...->ij...', A, geo.dbeta) + E('mj...,mi...->ij...', A, geo.dbeta)
    sixth = -2.0 / 3.0 * A * geo.div_beta
    out = first + second + third + fourth + fifth + sixth
    if p.kappa != 0:
        M, dM = momentum_constraint_derivative(geo)
        if matter is not None:
            # M_i - 8 pi S_i and its derivative (constraints.py:233-259)
            S_i = matter[1]
            dS = np.stack([np.stack([D1(S_i[i], l, p) for l in range(3)]) for i in range(3)])
            M = M - 8.0 * np.pi * S_i
            dM = dM - 8.0 * np.pi * dS
        DjMi = dM - E('kij...,k...->ij...', geo.chr2, M)
        out = out + p.kappa / 2 * alpha * (DjMi + np.swapaxes(DjMi, 0, 1))
    return out + kreiss_oliger(A, p)


def rhs_conformal_connection_with_matter(geo, matter):
    """Vacuum RHS - 16 pi alpha gt^ij S_j (conformal_connection.py:166-178)."""
    return rhs_conformal_connection(geo) + -16.0 * np.pi * geo.alpha * E('ij...,j...->i...', geo.ginv, matter[1])


def rhs_conformal_connection(geo):
    p, alpha, ginv, G = geo.p, geo.alpha, geo.ginv, geo.G
    Wf = np.maximum(geo.W, W_FLOOR)
    Araised = E('ik...,jl...,kl...->ij...', ginv, ginv, geo.A)
    first = -4 / 3 * alpha * E('ij...,j...->i...', ginv, geo.dK)
    second = 2 * alpha * E('ijk...,jk...->i...', geo.chr2, Araised)
    third = -6 * alpha / Wf * E('ij...,j...->i...', Araised, geo.dW)
    fourth = -2 * E('ij...,j...->i...', Araised, geo.dalpha)
    fifth = geo.advect(G)
    sixth = 2.0 / 3.0 * G * geo.div_beta
    seventh = -E('m...,im...->i...', G, geo.dbeta)
    d2beta = np.zeros((3, 3, 3) + geo.K.shape)                         # [i,m,n] = d_m d_n beta^i
    for i in range(3):
        for m in range(3):
            for n in range(3):
                d2beta[i, m, n] = (D2(geo.beta[i], m, p) if m == n
                                   else D1(geo.dbeta[i, n], m, p))
    eighth = E('mn...,imn...->i...', ginv, d2beta)
    grad_div = np.zeros((3,) + geo.K.shape)
    for m in range(3):
        for n in range(3):
            grad_div[m] = grad_div[m] + (D2(geo.beta[n], m, p) if m == n
                                         else D1(geo.dbeta[n, n], m, p))
    ninth = 1.0 / 3.0 * E('im...,m...->i...', ginv, grad_div)
    out = first + second + third + fourth + fifth + sixth + seventh + eighth + ninth
    return out + kreiss_oliger(G, p)


def rhs_lapse(geo):
    alpha, K = geo.alpha, geo.K
    slicing = -np.power(alpha, 2) * K if geo.p.gauge == 0 else -2.0 * alpha * K
    return slicing + geo.advect(alpha) + kreiss_oliger(alpha, geo.p)


def rhs_shift(geo):
    p = geo.p
    if p.zero_shift != 0:
        return 0.0 * geo.beta
    out = p.g * geo.G + geo.advect(geo.beta) + -p.eta * geo.beta
    return out + kreiss_oliger(geo.beta, p)


# ----------------------------------------------------------------------------
# Sommerfeld faces (boundaries.py:20-171)
# ----------------------------------------------------------------------------

def coordinates(shape, p):
    mins = (p.x_min, p.y_min, p.z_min)
    axes = [np.asarray(mins[d], dtype=np.float64) + np.asarray(p.dx, dtype=np.float64)
            * (np.arange(shape[d], dtype=np.float64) + 0.0) for d in range(3)]
    return (axes[0][:, None, None], axes[1][None, :, None], axes[2][None, None, :])


def sommerfeld_mask(shape, p):
    codes = (p.xl_bc, p.xr_bc, p.yl_bc, p.yr_bc, p.zl_bc, p.zr_bc)
    start = p.guard_cells
    counts = shape if p.owned_shape is None else p.owned_shape
    idx = (np.arange(shape[0])[:, None, None], np.arange(shape[1])[None, :, None],
           np.arange(shape[2])[None, None, :])
    mask = np.zeros(shape, dtype=bool)
    owned = np.ones(shape, dtype=bool)
    for d in range(3):
        end = start + counts[d]
        lower = codes[2 * d] == SOMMERFELD and bool(p.owned_faces[2 * d])
        upper = codes[2 * d + 1] == SOMMERFELD and bool(p.owned_faces[2 * d + 1])
        if p.owned_shape is not None:
            lower = lower and counts[d] > 1
            upper = upper and counts[d] > 1
        mask = mask | (lower & (idx[d] == start)) | (upper & (idx[d] == end - 1))
        owned = owned & (idx[d] >= start) & (idx[d] < end)
    return mask & owned


def sommerfeld(field, rhs, asymptote, p):
    shape = field.shape[-3:]
    X, Y, Z = coordinates(shape, p)
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    rs = np.where(r > 0.0, r, 1.0)
    radial = (X * D1(field, 0, p) + Y * D1(field, 1, p) + Z * D1(field, 2, p)) / rs
    value = -(radial + (field - asymptote) / rs)
    return np.where(sommerfeld_mask(shape, p), value, rhs)


def has_sommerfeld(p):
    return any(int(c) == SOMMERFELD for c in (p.xl_bc, p.xr_bc, p.yl_bc, p.yr_bc, p.zl_bc, p.zr_bc))


def apply_sommerfeld(v, rhs, p):
    if not has_sommerfeld(p):
        return rhs
    flat = np.eye(3)[:, :, None, None, None]
    asymptotes = (flat, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0)
    return BSSNVariables(*(sommerfeld(np.asarray(f), r, a, p)
                           for f, r, a in zip(v, rhs, asymptotes)))


# ----------------------------------------------------------------------------
# assembly, projection and RK4 (time_evolve.py)
# ----------------------------------------------------------------------------

def compute_rhs(v, p, matter=None):
    """compute_bssn_rhs (time_evolve.py:41-57); with matter = (rho, S_i, S_ij),
    compute_bssn_rhs_with_matter (time_evolve.py:60-91): sources enter the bulk
    equations before the Sommerfeld faces are imposed."""
    geo = Geometry(v, p)
    hessian_alpha = w2_lapse_hessian(geo)
    if matter is not None:
        matter = tuple(np.asarray(m) for m in matter)
    rhs = BSSNVariables(
        conformal_metric=rhs_conformal_metric(geo),
        conformal_factor=rhs_conformal_factor(geo),
        traceless_K=rhs_traceless_A(geo, hessian_alpha, matter),
        trace_K=rhs_trace_K(geo, hessian_alpha, matter),
        conformal_connection=(rhs_conformal_connection(geo) if matter is None
                              else rhs_conformal_connection_with_matter(geo, matter)),
        lapse=rhs_lapse(geo),
        shift=rhs_shift(geo),
    )
    return apply_sommerfeld(v, rhs, p)


def project(v):
    """det(gamma_tilde) -> 1, then A_tilde -> trace-free (time_evolve.py:94-141)."""
    g = np.asarray(v.conformal_metric)
    g = g * inv_cbrt(determinant(g))
    A = trace_free(np.asarray(v.traceless_K), g, inverse_metric(g))
    return BSSNVariables(g, np.asarray(v.conformal_factor), A, np.asarray(v.trace_K),
                         np.asarray(v.conformal_connection), np.asarray(v.lapse), np.asarray(v.shift))


def _axpy(v, k, scale):
    return BSSNVariables(*(a + scale * b for a, b in zip(v, k)))


def rk4_step(v, p, rhs=compute_rhs):
    dt = p.dt
    v = project(v)
    k1 = rhs(v, p)
    k2 = rhs(project(_axpy(v, k1, 0.5 * dt)), p)
    k3 = rhs(project(_axpy(v, k2, 0.5 * dt)), p)
    k4 = rhs(project(_axpy(v, k3, dt)), p)
    total = BSSNVariables(*(a + 2 * b + 2 * c + d for a, b, c, d in zip(k1, k2, k3, k4)))
    return project(_axpy(v, total, dt / 6.0))


# ----------------------------------------------------------------------------
# constraints (constraints.py:271-412) and norms (diagnostics/constraints.py)
# ----------------------------------------------------------------------------

def constraints(v, p):
    """(H, M_i, det-1, tr A, Gamma_i - gamma^jk Gamma^i_jk)."""
    geo = Geometry(v, p)
    ginv = geo.ginv
    ricci_scalar = E('ij...,ij...->...', ginv, w2_ricci(geo))
    A2 = E('ik...,jl...,ij...,kl...->...', ginv, ginv, geo.A, geo.A)
    H = ricci_scalar + 2 / 3 * geo.K ** 2 - A2
    M = momentum_constraint(geo)
    det = determinant(geo.g) - 1.0
    trA = E('ij...,ij...->...', ginv, geo.A)
    gamma = geo.G - E('jk...,ijk...->i...', ginv, geo.chr2)
    return H, M, det, trA, gamma


def constraint_norms(v, p):
    """RMS and max-abs per constraint over all points (diagnostics/constraints.py:9-36)."""
    names = ("hamiltonian", "momentum", "det_gamma", "trace_A", "gamma")
    out = {}
    for name, field in zip(names, constraints(v, p)):
        out[name + "_l2"] = float(np.sqrt(np.mean(field ** 2)))
        out[name + "_linf"] = float(np.max(np.abs(field)))
    return out


# ----------------------------------------------------------------------------
# correctly rounded x^(-1/3)
# ----------------------------------------------------------------------------

def _split(a):
    c = 134217729.0 * a
    hi = c - (c - a)
    return hi, a - hi


def _two_prod(a, b):
    """Dekker's exact product a*b = p + e (no FMA needed)."""
    p = a * b
    ah, al = _split(a)
    bh, bl = _split(b)
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def _two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


# The double nearest -1/3 exceeds -1/3 by this much; pow(x, -1.0/3.0) is
# x^(-1/3) * x^POW_THIRD_OFFSET.
POW_THIRD_OFFSET = float(__import__("fractions").Fraction(-1.0 / 3.0) + __import__("fractions").Fraction(1, 3))


def _above_midpoint(xi, mu):
    """Is pow(1+xi, -1/3 + offset) above the midpoint 1 + mu?  Exact for
    |xi| < 2^-28: y* > m <=> x m^3 - 1 < 3*offset*ln x, where
    x m^3 - 1 = (xi + 3mu) + 3mu(mu + xi) + mu^2(mu + 3xi) + ...; the first
    term is a multiple of 2^-54 that is either zero or larger than the rest."""
    a1 = xi + 3.0 * mu
    ph, pl = _two_prod(3.0 * mu, mu + xi)
    a3 = mu * mu * (mu + 3.0 * xi)
    f = 3.0 * POW_THIRD_OFFSET * (xi - 0.5 * xi * xi)
    second = ((ph - f) + (pl + a3)) < 0.0
    return np.where(a1 != 0.0, a1 < 0.0, second)


def inv_cbrt(x):
    """Correctly rounded pow(x, -1.0/3.0), as libm evaluates ``det ** (-1/3)``.

    Near x = 1 (every projected metric's determinant) the result is chosen
    by exact midpoint tests -- values such as 1 - 3*2^-53 have cube roots
    within 2^-106 of a rounding midpoint.  Elsewhere one Newton step for
    y^-3 = x carried in double-double, plus the tiny correction for the
    double exponent differing from -1/3, is rounded once.  NumPy's SIMD power
    can differ from libm's in the last bit, so it only supplies the guess.
    """
    x = np.asarray(x, dtype=np.float64)
    with np.errstate(all="ignore"):
        y = np.power(x, -1.0 / 3.0)
        y2h, y2l = _two_prod(y, y)
        y3h, y3l = _two_prod(y2h, y)
        y3l = y3l + y2l * y
        xyh, xyl = _two_prod(x, y3h)
        xyl = xyl + x * y3l
        rh, rl = _two_sum(np.ones_like(x), -xyh)
        r = rh + (rl - xyl)
        c = y * (r * (1.0 / 3.0) + POW_THIRD_OFFSET * np.log(x))
        out = y + c
        xi = x - 1.0
        near = np.abs(xi) < 2.0 ** -28
        if np.any(near):
            xn = xi[near]
            yn = 1.0 - xn * (1.0 / 3.0)
            for _ in range(4):
                up = np.nextafter(yn, 2.0)
                go_up = _above_midpoint(xn, (yn - 1.0) + 0.5 * (up - yn))
                dn = np.nextafter(yn, 0.0)
                go_dn = ~go_up & ~_above_midpoint(xn, (yn - 1.0) - 0.5 * (yn - dn))
                yn = np.where(go_up, up, np.where(go_dn, dn, yn))
            out = np.array(out, copy=True)
            out[near] = yn
    good = np.isfinite(x) & (x > 0)
    return np.where(good, out, np.power(x, -1.0 / 3.0))
