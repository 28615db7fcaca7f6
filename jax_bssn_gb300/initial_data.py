"""Initial data and parameter sets for the benchmark and parity workloads.

Host-side NumPy set-up code (run once per evolution, not on the hot path).

* gauge wave: the exact harmonic-slicing gauge wave on a periodic box, the
  same analytic state the reference tests evolve
  (tests/initial_data.py:147-205 of uwplasma/JAX_BSSN);
* linear plus-polarised wave in Gauss coordinates with its analytic conformal
  connection (demos/gravitational_waves/linear_wave.py:36-56);
* linearised Teukolsky quadrupole wave: the even-parity m = 0 solution of
  Teukolsky, Phys. Rev. D 26, 745 (1982), as a time-symmetric standing wave
  built from F(x) = a x exp(-x^2/w^2).  The reference ships no such data; it is
  restated here from the published solution.  Each term c_k F^(n)/r^k of the
  radial functions A, B, C combines the outgoing and ingoing parts with the
  parity (-1)^k (odd powers of 1/r take the difference F(t-r) - F(t+r), even
  powers the sum), which is the combination regular at r = 0.  At t = 0 and for
  odd F only the terms noted below survive, and K_ij = 0.
"""

from __future__ import annotations

import math

import numpy as np

from .bssn.variables import BSSNParameters, BSSNVariables

SOMMERFELD = 1


# ----------------------------------------------------------------------------
# coordinates
# ----------------------------------------------------------------------------

def periodic_axis(n: int, length: float = 1.0) -> np.ndarray:
    """Endpoint-excluded periodic samples on [-L/2, L/2)."""
    return np.linspace(-length / 2.0, length / 2.0, n, endpoint=False)


def vertex_axis(n: int, dx: float) -> np.ndarray:
    """Vertex-centred samples symmetric about zero: (i - (n-1)/2) dx."""
    return (np.arange(n, dtype=np.float64) - (n - 1) / 2.0) * dx


def mesh(x, y=None, z=None):
    y = x if y is None else y
    z = x if z is None else z
    return np.meshgrid(x, y, z, indexing="ij")


# ----------------------------------------------------------------------------
# small tensor helpers (host)
# ----------------------------------------------------------------------------

def _inverse_sym(g):
    """Adjugate inverse of a field of symmetric 3x3 matrices (3,3,...)."""
    a, b, c = g[0, 0], g[0, 1], g[0, 2]
    d, e, f = g[1, 1], g[1, 2], g[2, 2]
    det = a * (d * f - e * e) - b * (b * f - e * c) + c * (b * e - d * c)
    inv = np.empty_like(g)
    inv[0, 0] = (d * f - e * e) / det
    inv[0, 1] = inv[1, 0] = (c * e - b * f) / det
    inv[0, 2] = inv[2, 0] = (b * e - c * d) / det
    inv[1, 1] = (a * f - c * c) / det
    inv[1, 2] = inv[2, 1] = (b * c - a * e) / det
    inv[2, 2] = (a * d - b * b) / det
    return inv, det


# Platform-independent elementary functions.  NumPy's exp and pow may differ
# by an ulp between CPU builds (x86-64 and Arm use different vector
# libraries); the functions below use only IEEE-rounded +, -, *, /, rint and
# ldexp in a fixed order, so the initial data they build are the same bits on
# every host -- which lets parity pins made on one machine be checked on
# another.  Accuracy is within a few ulp of the exact values.

_LN2_HI = 0.693145751953125            # 16 significant bits: k * _LN2_HI is exact for |k| < 2^37
_LN2_LO = 1.4286068203094173e-06       # ln 2 - _LN2_HI
_INV_LN2 = 1.4426950408889634


def _exp_portable(x):
    """exp(x) by Cody-Waite reduction x = k ln 2 + r, |r| <= ln 2 / 2, and the
    degree-20 Taylor polynomial of exp(r) in Horner form."""
    x = np.asarray(x, dtype=np.float64)
    k = np.rint(x * _INV_LN2)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    acc = np.ones_like(r)
    for n in range(20, 0, -1):
        acc = 1.0 + (r / float(n)) * acc
    return np.ldexp(acc, k.astype(np.int64))


def _power_near_one(x, exponent, terms=24):
    """x ** exponent for |x - 1| < 0.01 by the binomial series in Horner form."""
    x = np.asarray(x, dtype=np.float64)
    e = x - 1.0
    if np.max(np.abs(e)) >= 0.01:
        raise ValueError("_power_near_one needs |x - 1| < 0.01")
    coef = [1.0]
    for k in range(1, terms + 1):
        coef.append(coef[-1] * (exponent - (k - 1)) / k)
    acc = np.full_like(e, coef[terms])
    for k in range(terms - 1, -1, -1):
        acc = coef[k] + e * acc
    return acc


def _d1_closed(f, axis, dx, closed):
    """Fourth-order centred derivative; one-sided 5-point closures at both
    ends when ``closed`` (otherwise periodic)."""
    s = lambda k: np.roll(f, -k, axis=axis)  # noqa: E731
    out = (2.0 / 3.0 * (s(1) - s(-1)) - 1.0 / 12.0 * (s(2) - s(-2))) / dx
    if closed:
        m = np.moveaxis(f, axis, -1)
        o = np.moveaxis(out, axis, -1)
        o[..., 0] = (-25 / 12 * m[..., 0] + 4 * m[..., 1] - 3 * m[..., 2] + 4 / 3 * m[..., 3] - 1 / 4 * m[..., 4]) / dx
        o[..., 1] = (-1 / 4 * m[..., 0] - 5 / 6 * m[..., 1] + 3 / 2 * m[..., 2] - 1 / 2 * m[..., 3] + 1 / 12 * m[..., 4]) / dx
        o[..., -2] = (-1 / 12 * m[..., -5] + 1 / 2 * m[..., -4] - 3 / 2 * m[..., -3] + 5 / 6 * m[..., -2] + 1 / 4 * m[..., -1]) / dx
        o[..., -1] = (1 / 4 * m[..., -5] - 4 / 3 * m[..., -4] + 3 * m[..., -3] - 4 * m[..., -2] + 25 / 12 * m[..., -1]) / dx
    return out


def _ordered_sum(terms):
    acc = None
    for t in terms:
        acc = t if acc is None else acc + t
    return acc


def discrete_connection(conformal_metric, dx, closed):
    """Gamma^i = g^mn Gamma^i_mn from discrete D4 derivatives of gt (sums in a
    fixed order, so the result does not depend on the host's BLAS/einsum)."""
    dg = np.stack([_d1_closed(conformal_metric, 2 + d, dx, closed) for d in range(3)])  # [k,i,j]
    gi, _ = _inverse_sym(conformal_metric)
    R3 = range(3)
    c1 = [[[0.5 * ((dg[k, i, j] + dg[j, i, k]) - dg[i, j, k]) for k in R3] for j in R3] for i in R3]
    c2 = [[[_ordered_sum(gi[i, m] * c1[m][j][k] for m in R3) for k in R3] for j in R3] for i in R3]
    return np.stack([_ordered_sum(gi[m, n] * c2[i][m][n] for m in R3 for n in R3) for i in R3])


def bssn_from_adm(gamma, Kij, alpha, beta, connection=None, dx=None, closed=False):
    """Physical (gamma_ij, K_ij) -> BSSN W-formulation variables.  Metrics
    within 1% of unit determinant use the portable power series for
    det^(-1/6), so the result is host-independent."""
    gi, det = _inverse_sym(gamma)
    if np.max(np.abs(det - 1.0)) < 0.01:
        W = _power_near_one(det, -1.0 / 6.0)
    else:
        W = det ** (-1.0 / 6.0)
    gt = W * W * gamma
    K = _ordered_sum(gi[i, j] * Kij[i, j] for i in range(3) for j in range(3))
    At = W * W * (Kij - gamma * K / 3.0)
    if connection is None:
        connection = discrete_connection(gt, dx, closed)
    return BSSNVariables(gt, W, At, K, connection, alpha, beta)


# ----------------------------------------------------------------------------
# gauge wave (periodic)
# ----------------------------------------------------------------------------

def gauge_wave_state(X, Y, Z, t=0.0, amplitude=0.1, wavelength=1.0) -> BSSNVariables:
    """Exact harmonic gauge wave ds^2 = -H dt^2 + H dx^2 + dy^2 + dz^2,
    H = 1 - A sin(2 pi (x - t)/lambda), in BSSN variables."""
    shape = X.shape
    phase = 2.0 * np.pi * (X - t) / wavelength
    H = 1.0 - amplitude * np.sin(phase)
    W = np.power(H, -1.0 / 6.0)
    gt = np.zeros((3, 3) + shape)
    gt[0, 0] = H * W ** 2
    gt[1, 1] = W ** 2
    gt[2, 2] = W ** 2
    Kxx = -(np.pi * amplitude / wavelength) * np.cos(phase) / np.sqrt(H)
    # K = W^2 gt^xx K_xx ; At_xx = W^2 (K_xx - gamma_xx K/3)
    gtinv_xx = 1.0 / gt[0, 0]
    K = W ** 2 * gtinv_xx * Kxx
    At = np.zeros((3, 3) + shape)
    At[0, 0] = W ** 2 * (Kxx - gt[0, 0] * gtinv_xx * Kxx / 3.0)
    At[1, 1] = W ** 2 * (-gt[1, 1] * gtinv_xx * Kxx / 3.0)
    At[2, 2] = W ** 2 * (-gt[2, 2] * gtinv_xx * Kxx / 3.0)
    dHdx = -(2.0 * np.pi * amplitude / wavelength) * np.cos(phase)
    G = np.zeros((3,) + shape)
    G[0] = (2.0 / 3.0) * H ** (-5.0 / 3.0) * dHdx
    return BSSNVariables(gt, W, At, K, G, np.sqrt(H), np.zeros((3,) + shape))


def gauge_wave_config(n=32, amplitude=0.1, wavelength=1.0, cfl=0.25, nu=0.1):
    """3D periodic gauge wave on [-0.5, 0.5)^3, harmonic lapse, zero shift."""
    x = periodic_axis(n, 1.0)
    X, Y, Z = mesh(x)
    dx = 1.0 / n
    state = gauge_wave_state(X, Y, Z, 0.0, amplitude, wavelength)
    params = BSSNParameters(eta=0.0, kappa=0.0, nu=nu, g=0.0, dx=dx, dt=cfl * dx, zero_shift=1, gauge=0,
                            x_min=float(x[0]), y_min=float(x[0]), z_min=float(x[0]))
    return state, params


# ----------------------------------------------------------------------------
# linear plus-polarised wave (FMR demo data)
# ----------------------------------------------------------------------------

def linear_wave_state(X, Y, Z, amplitude=1.0e-8, wavelength=1.0) -> BSSNVariables:
    """h_+ = a sin(2 pi x/lambda) in Gauss coordinates with the analytic
    conformal connection Gamma^x = -d_x gt^xx (det gt = 1)."""
    k = 2.0 * np.pi / wavelength
    h = amplitude * np.sin(k * X) + 0.0 * Y + 0.0 * Z
    dh = k * amplitude * np.cos(k * X) + 0.0 * Y + 0.0 * Z
    W = (1.0 - h * h) ** (-1.0 / 6.0)
    shape = X.shape
    gt = np.zeros((3, 3) + shape)
    gt[0, 0] = W * W
    gt[1, 1] = (1.0 + h) * W * W
    gt[2, 2] = (1.0 - h) * W * W
    Kij = np.zeros((3, 3) + shape)
    Kij[1, 1] = dh / 2.0
    Kij[2, 2] = -dh / 2.0
    gi, _ = _inverse_sym(gt)
    trK = np.einsum("ij...,ij...->...", gi, Kij)
    At = W * W * (Kij - gt * trK / 3.0)
    K = W * W * trK
    G = np.zeros((3,) + shape)
    G[0] = 2.0 * h * dh / 3.0 * (1.0 - h * h) ** (-2.0 / 3.0)
    return BSSNVariables(gt, W, At, K, G, np.ones(shape), np.zeros((3,) + shape))


# ----------------------------------------------------------------------------
# linearised Teukolsky quadrupole wave
# ----------------------------------------------------------------------------

def _gauss_odd_derivatives(r, a, w):
    """F(x) = a x exp(-x^2/w^2) and its first four derivatives at x = r."""
    u = r / w
    u2 = u * u
    u3 = u2 * u
    u4 = u2 * u2
    u5 = u4 * u
    e = _exp_portable(-u2)
    F0 = a * r * e
    F1 = a * e * (1.0 - 2.0 * u2)
    F2 = a * e * (-6.0 * u + 4.0 * u3) / w
    F3 = a * e * (-6.0 + 24.0 * u2 - 8.0 * u4) / (w * w)
    F4 = a * e * (60.0 * u - 80.0 * u3 + 16.0 * u5) / (w * w * w)
    return F0, F1, F2, F3, F4


def teukolsky_radial(r, a, w):
    """Regular time-symmetric A, B, C at t = 0 (even-parity m = 0 wave).

    For odd F, the combinations are F^(n)(-r) - F^(n)(r) = -2 F^(n)(r) for odd
    powers of 1/r with even n, and F^(n)(-r) + F^(n)(r) = 2 F^(n)(r) for even
    powers with odd n; all others vanish.
    """
    F0, F1, F2, F3, F4 = _gauss_odd_derivatives(r, a, w)
    r2 = r * r
    r3 = r2 * r
    r4 = r2 * r2
    r5 = r4 * r
    A = 3.0 * (-2.0 * F2 / r3 + 3.0 * 2.0 * F1 / r4 + 3.0 * (-2.0) * F0 / r5)
    B = -(2.0 * F3 / r2 + 3.0 * (-2.0) * F2 / r3 + 6.0 * 2.0 * F1 / r4 + 6.0 * (-2.0) * F0 / r5)
    C = 0.25 * (-2.0 * F4 / r + 2.0 * 2.0 * F3 / r2 + 9.0 * (-2.0) * F2 / r3
                + 21.0 * 2.0 * F1 / r4 + 21.0 * (-2.0) * F0 / r5)
    return A, B, C


def teukolsky_metric(X, Y, Z, amplitude=1.0e-5, width=1.0):
    """Cartesian h_ij of the quadrupole wave at t = 0 (Teukolsky 1982, m = 0)."""
    r = np.sqrt(X * X + Y * Y + Z * Z)
    rho = np.sqrt(X * X + Y * Y)
    A, B, C = teukolsky_radial(r, amplitude, width)
    st = rho / r
    ct = Z / r
    safe = np.where(rho > 0, rho, 1.0)
    cp = np.where(rho > 0, X / safe, 1.0)
    sp = np.where(rho > 0, Y / safe, 0.0)
    s2 = st * st
    h_rr = A * (2.0 - 3.0 * s2)
    h_rt = B * (-3.0 * st * ct)
    h_tt = C * (3.0 * s2) + A * (-1.0)
    h_pp = C * (-3.0 * s2) + A * (3.0 * s2 - 1.0)
    rhat = np.stack([st * cp, st * sp, ct])
    that = np.stack([ct * cp, ct * sp, -st])
    phat = np.stack([-sp, cp, np.zeros_like(cp)])
    h = (h_rr * np.einsum("i...,j...->ij...", rhat, rhat)
         + h_rt * (np.einsum("i...,j...->ij...", rhat, that) + np.einsum("i...,j...->ij...", that, rhat))
         + h_tt * np.einsum("i...,j...->ij...", that, that)
         + h_pp * np.einsum("i...,j...->ij...", phat, phat))
    return h


def teukolsky_config(n=128, half_width=4.0, amplitude=1.0e-5, width=1.0, cfl=0.25,
                     eta=2.0, g=0.75, nu=0.02, kappa=0.0):
    """Linearised Teukolsky quadrupole wave on an n^3 vertex grid over
    [-half_width, half_width]^3: 1+log lapse, Gamma-driver shift, Sommerfeld faces."""
    dx = 2.0 * half_width / (n - 1)
    x = vertex_axis(n, dx)
    X, Y, Z = mesh(x)
    shape = X.shape
    gamma = np.eye(3)[:, :, None, None, None] + teukolsky_metric(X, Y, Z, amplitude, width)
    state = bssn_from_adm(gamma, np.zeros((3, 3) + shape), np.ones(shape), np.zeros((3,) + shape),
                          dx=dx, closed=True)
    params = BSSNParameters(eta=eta, kappa=kappa, nu=nu, g=g, dx=dx, dt=cfl * dx, zero_shift=0, gauge=1,
                            xl_bc=SOMMERFELD, xr_bc=SOMMERFELD, yl_bc=SOMMERFELD, yr_bc=SOMMERFELD,
                            zl_bc=SOMMERFELD, zr_bc=SOMMERFELD,
                            x_min=float(x[0]), y_min=float(x[0]), z_min=float(x[0]))
    return state, params


def random_smooth_state(shape, seed=0, amplitude=0.05, shift=True) -> BSSNVariables:
    """A smooth, generic, periodic state (all components non-trivial) for
    parity tests that must exercise every term of the RHS."""
    rng = np.random.default_rng(seed)
    axes = [np.linspace(0.0, 2.0 * np.pi, n, endpoint=False) for n in shape]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")

    def field():
        c = rng.normal(size=6)
        return c[0] * np.sin(X + c[1]) + c[2] * np.cos(2.0 * Y + c[3]) + c[4] * np.sin(Z + X + c[5])

    g = np.zeros((3, 3) + tuple(shape))
    A = np.zeros((3, 3) + tuple(shape))
    for i in range(3):
        for j in range(i, 3):
            g[i, j] = g[j, i] = (1.0 if i == j else 0.0) + amplitude * field()
            A[i, j] = A[j, i] = amplitude * field()
    W = 1.0 + amplitude * field()
    K = amplitude * field()
    alpha = 1.0 + amplitude * field()
    G = np.stack([amplitude * field() for _ in range(3)])
    beta = np.stack([amplitude * field() for _ in range(3)]) if shift else np.zeros((3,) + tuple(shape))
    return BSSNVariables(g, W, A, K, G, alpha, beta)


def cfl_timestep(dx, cfl):
    return cfl * dx


__all__ = [name for name in dir() if not name.startswith("_") and name not in ("annotations", "math", "np")]


def brill_lindquist_plane_state(masses=(0.5, 0.5), separation=2.0, num_radial_points=256, r_max=8.0):
    """Two time-symmetric punctures on the z axis as a compact axisymmetric
    Cartoon state (Nrho+4, 1, 2 Nrho).

    Zero-momentum Bowen-York data: the Hamiltonian constraint is solved by the
    Brill-Lindquist conformal factor psi = 1 + sum_i m_i / (2 |x - x_i|)
    exactly (JAX_BSSN tests/test_bowen_york.py:113-127), A_ij = 0.  As in
    bowen_york_plane_data (demos/axisymmetric_blackhole_collision/
    axisymmetric_blackhole_collision.py:59-136): cell-centred rho = (i+1/2) dx,
    z = -r_max + (k+1/2) dx, dx = r_max / Nrho, W = psi^-2, pre-collapsed lapse
    alpha = W, flat conformal metric, K = Gamma = beta = 0, four parity ghosts.
    """
    n = int(num_radial_points)
    dx = r_max / n
    rho = (np.arange(n, dtype=np.float64) + 0.5) * dx
    z = -r_max + (np.arange(2 * n, dtype=np.float64) + 0.5) * dx
    R, Z = np.meshgrid(rho, z, indexing="ij")
    psi = np.ones_like(R)
    for m, zc in zip(masses, (-separation / 2.0, separation / 2.0)):
        psi = psi + m / (2.0 * np.sqrt(R * R + (Z - zc) ** 2))
    W = 1.0 / (psi * psi)
    full = np.concatenate((W[3::-1], W), axis=0)[:, None, :]       # even parity ghosts
    shape = full.shape
    g = np.broadcast_to(np.eye(3)[:, :, None, None, None], (3, 3) + shape).copy()
    zeros = np.zeros(shape)
    return BSSNVariables(g, full.copy(), np.zeros((3, 3) + shape), zeros.copy(), np.zeros((3,) + shape),
                         full.copy(), np.zeros((3,) + shape)), dx


def brill_lindquist_config(masses=(0.5, 0.5), separation=2.0, num_radial_points=256, r_max=8.0, cfl=0.2,
                           eta=2.0, g=0.75, nu=0.02, kappa=0.002):
    """The axisymmetric head-on configuration: compact state plus the demo's
    parameters (1+log lapse, Gamma-driver, Sommerfeld x-right and z faces,
    x_min = -3.5 dx, y_min = -4 dx, z_min = -r_max + dx/2, dt = cfl dx)."""
    state, dx = brill_lindquist_plane_state(masses, separation, num_radial_points, r_max)
    params = BSSNParameters(eta=eta, kappa=kappa, nu=nu, g=g, dx=dx, dt=cfl * dx, zero_shift=0, gauge=1,
                            xl_bc=0, xr_bc=SOMMERFELD, yl_bc=0, yr_bc=0, zl_bc=SOMMERFELD, zr_bc=SOMMERFELD,
                            x_min=-3.5 * dx, y_min=-4.0 * dx, z_min=-r_max + 0.5 * dx, mad_q=1.0)
    return state, params


FMR_LINEAR_WAVE_PATCHES = (((32, 32, 32), (64, 64, 64), None), ((20, 20, 20), (44, 44, 44), 1))


def fmr_linear_wave_hierarchy(root=96, patches=FMR_LINEAR_WAVE_PATCHES):
    """Nested 2:1 hierarchy: level 1 over root samples [32, 64] (65^3 active),
    level 2 over level-1 samples [20, 44] (49^3 active), MAD weights on."""
    from .fmr import FMRHierarchySpec, FMRPatchSpec
    scale = root / 96.0
    specs = []
    for lo, hi, parent in patches:
        lo = tuple(int(round(v * scale)) for v in lo)
        hi = tuple(int(round(v * scale)) for v in hi)
        specs.append(FMRPatchSpec(lo, hi, parent=parent))
    return FMRHierarchySpec(tuple(specs), use_mad=True)


def fmr_linear_wave_root(root=96, half_width=8.0, wavelength=4.0, cfl=0.25, levels=3):
    """Root parameters of the nested linear-wave run: periodic [-half_width,
    half_width)^3 with dx = 2 half_width / root, harmonic lapse, zero shift,
    no damping or dissipation (demos/gravitational_waves/linear_wave.py:116-122),
    dt = cfl * dx_finest."""
    dx = 2.0 * half_width / root
    dt = cfl * dx / 2 ** (levels - 1)
    return BSSNParameters(eta=0.0, kappa=0.0, nu=0.0, g=0.0, dx=dx, dt=dt, zero_shift=1, gauge=0,
                          x_min=-half_width, y_min=-half_width, z_min=-half_width)


def linear_wave_callback(amplitude=1.0e-8, wavelength=4.0):
    """Initial-data callback for ``initialize_tiled_fmr``: the plus-polarised
    linear wave on a patch's owned samples (linear_wave.py:36-56)."""
    def initial(coordinates, local_params):
        X, Y, Z = np.broadcast_arrays(*coordinates)
        return linear_wave_state(X, Y, Z, amplitude, wavelength)
    return initial
