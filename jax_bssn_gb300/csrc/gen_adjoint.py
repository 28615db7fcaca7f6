"""Generator of the pointwise BSSN algebra and its reverse sweep (adjoint).

    python jax_bssn_gb300/csrc/gen_adjoint.py      # rewrites bssn_adjoint_point.cuh

The right-hand side of the BSSN equations is, at every grid point, a fixed
algebraic function F of the 21 state values and of their first and second
finite-difference derivatives; the advection terms beta^i d_i u and the
Kreiss-Oliger dissipation are linear stencils and are handled by the adjoint
kernels directly.  This file restates F once (the equations of
JAX_BSSN/bssn/spatial_metric.py:17-106, geometry.py:21-186,
extrinsic_curvature.py:31-224, conformal_connection.py:19-162 and
shift_and_lapse.py:65-132, for kappa = 0 and no matter) on a small tracing
type, records it as a straight-line program, and emits

  rhs_point_forward   F itself (used to check the restatement against the
                      production RHS kernels),
  rhs_point_vjp       the vector-Jacobian product  sum_f kbar_f dF_f/dx  for
                      every input x: the reverse sweep of the program,
                      accumulated in program order reversed (reverse-mode
                      automatic differentiation written out as code),
  project_point_vjp   the same for the algebraic projection
                      (JAX_BSSN/evolution/time_evolve.py:94-141).

The tracing type also evaluates on NumPy arrays, which is how the CPU tests
check the restatement against the oracle and the reverse sweep against finite
differences without a GPU.
"""

from __future__ import annotations

import math
from pathlib import Path

HERE = Path(__file__).resolve().parent
TARGET = HERE / "bssn_adjoint_point.cuh"

SYM = ((0, 1, 2), (1, 3, 4), (2, 4, 5))      # sym(i, j) -> upper-triangle slot
PAIRS = ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))


# ----------------------------------------------------------------------------
# straight-line program
# ----------------------------------------------------------------------------

class Program:
    """Nodes in creation order: (op, args, payload).  ops: in, param, const,
    add, sub, mul, div, neg, sqrt, powc (x ** c), maxc (max(x, c))."""

    COMMUTATIVE = ("add", "mul")

    def __init__(self):
        self.nodes = []
        self.consts = {}
        self.memo = {}      # (op, args, payload) -> node: identical expressions are one node
        self.inputs = []    # (name, node)
        self.params = []    # (name, node)

    def _new(self, op, args=(), payload=None):
        args = tuple(args)
        if op in self.COMMUTATIVE:
            args = tuple(sorted(args))
        key = (op, args, payload)
        if op not in ("in", "param") and key in self.memo:
            return self.memo[key]
        self.nodes.append((op, args, payload))
        n = len(self.nodes) - 1
        if op not in ("in", "param"):
            self.memo[key] = n
        return n

    def input(self, name):
        n = self._new("in", (), name)
        self.inputs.append((name, n))
        return V(self, n)

    def param(self, name):
        n = self._new("param", (), name)
        self.params.append((name, n))
        return V(self, n)

    def const(self, c):
        c = float(c)
        if c not in self.consts:
            self.consts[c] = self._new("const", (), c)
        return V(self, self.consts[c])

    def is_const(self, n, value=None):
        op, _, payload = self.nodes[n]
        return op == "const" and (value is None or payload == value)


class V:
    """A traced value; arithmetic appends nodes (with constant folding)."""

    __slots__ = ("P", "n")

    def __init__(self, P, n):
        self.P, self.n = P, n

    def _lift(self, o):
        return o if isinstance(o, V) else self.P.const(o)

    def _val(self):
        op, _, payload = self.P.nodes[self.n]
        return payload if op == "const" else None

    def __add__(self, o):
        o = self._lift(o)
        a, b = self._val(), o._val()
        if a is not None and b is not None:
            return self.P.const(a + b)
        if a == 0.0:
            return o
        if b == 0.0:
            return self
        return V(self.P, self.P._new("add", (self.n, o.n)))

    __radd__ = __add__

    def __sub__(self, o):
        o = self._lift(o)
        a, b = self._val(), o._val()
        if a is not None and b is not None:
            return self.P.const(a - b)
        if b == 0.0:
            return self
        if a == 0.0:
            return -o
        return V(self.P, self.P._new("sub", (self.n, o.n)))

    def __rsub__(self, o):
        return self._lift(o) - self

    def __mul__(self, o):
        o = self._lift(o)
        a, b = self._val(), o._val()
        if a is not None and b is not None:
            return self.P.const(a * b)
        if a == 0.0 or b == 0.0:
            return self.P.const(0.0)
        if a == 1.0:
            return o
        if b == 1.0:
            return self
        if a == -1.0:
            return -o
        if b == -1.0:
            return -self
        return V(self.P, self.P._new("mul", (self.n, o.n)))

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = self._lift(o)
        b = o._val()
        if b is not None:
            return self * (1.0 / b)
        return V(self.P, self.P._new("div", (self.n, o.n)))

    def __rtruediv__(self, o):
        return self._lift(o) / self

    def __neg__(self):
        a = self._val()
        if a is not None:
            return self.P.const(-a)
        return V(self.P, self.P._new("neg", (self.n,)))


def vsqrt(x):
    return V(x.P, x.P._new("sqrt", (x.n,)))


def vpow(x, c):
    return V(x.P, x.P._new("powc", (x.n,), float(c)))


def vmax(x, c):
    return V(x.P, x.P._new("maxc", (x.n,), float(c)))


def vsum(terms):
    acc = None
    for t in terms:
        acc = t if acc is None else acc + t
    return acc


# ----------------------------------------------------------------------------
# the pointwise BSSN algebra (kappa = 0, vacuum)
# ----------------------------------------------------------------------------

# Input layout of the pointwise function (also the layout of its adjoint):
#   0..20    state values in component order: gt(6) W At(6) K Gt(3) alpha beta(3)
#   21..38   d_k gt_s        at 21 + 6k + s
#   39..41   d_k W           42..44 d_k alpha     45..47 d_k K
#   48..56   d_j beta^i      at 48 + 3i + j
#   57..65   d_d Gt^i        at 57 + 3d + i
#   66..101  d_m d_n gt_s    at 66 + 6 pair(m,n) + s
#   102..107 d_m d_n W       108..113 d_m d_n alpha (pair slots)
#   114..131 d_m d_n beta^i  at 114 + 6i + pair(m,n)
NSTATE = 21
I_DG, I_DW, I_DAL, I_DK, I_DB, I_DGT = 21, 39, 42, 45, 48, 57
I_D2G, I_D2W, I_D2AL, I_D2B = 66, 102, 108, 114
NIN = 132
PARAMS = ("eta", "gdrv", "c_harm", "c_log", "shift_on")


def state_inputs(P):
    x = [P.input(f"x{i}") for i in range(NIN)]
    return x


def inverse(g):
    """Symmetric 3x3 inverse by cofactors (mathematically the reference's
    Cholesky inverse, tensor_algebra.py:20-71)."""
    c00 = g[3] * g[5] - g[4] * g[4]
    c01 = g[2] * g[4] - g[1] * g[5]
    c02 = g[1] * g[4] - g[2] * g[3]
    det = g[0] * c00 + g[1] * c01 + g[2] * c02
    r = 1.0 / det
    return [c00 * r, c01 * r, c02 * r, (g[0] * g[5] - g[2] * g[2]) * r, (g[1] * g[2] - g[0] * g[4]) * r,
            (g[0] * g[3] - g[1] * g[1]) * r]


def full(t6):
    return [[t6[SYM[i][j]] for j in range(3)] for i in range(3)]


def contract_sym(S, T):
    """sum_ij S_ij T_ij for symmetric 3x3 S and T (full nested lists)."""
    return (S[0][0] * T[0][0] + S[1][1] * T[1][1] + S[2][2] * T[2][2]
            + 2.0 * (S[0][1] * T[0][1] + S[0][2] * T[0][2] + S[1][2] * T[1][2]))


def rhs_algebra(x, prm):
    """F(x): the RHS without advection and dissipation, component order."""
    g = full(x[0:6])
    W = x[6]
    A = full(x[7:13])
    K = x[13]
    Gt = x[14:17]
    al = x[17]
    b = x[18:21]
    dg = [[[x[I_DG + 6 * k + SYM[i][j]] for j in range(3)] for i in range(3)] for k in range(3)]  # dg[k][i][j]
    dW = x[I_DW:I_DW + 3]
    dal = x[I_DAL:I_DAL + 3]
    dK = x[I_DK:I_DK + 3]
    db = [[x[I_DB + 3 * i + j] for j in range(3)] for i in range(3)]        # db[i][j] = d_j beta^i
    dGt = [[x[I_DGT + 3 * d + i] for i in range(3)] for d in range(3)]      # dGt[d][i] = d_d Gt^i
    d2g = [[full(x[I_D2G + 6 * SYM[m][n]:I_D2G + 6 * SYM[m][n] + 6]) for n in range(3)] for m in range(3)]
    d2W = full(x[I_D2W:I_D2W + 6])
    d2al = full(x[I_D2AL:I_D2AL + 6])
    d2b = [full(x[I_D2B + 6 * i:I_D2B + 6 * i + 6]) for i in range(3)]     # d2b[i][m][n] = d_m d_n beta^i
    eta, gdrv, c_harm, c_log, shift_on = prm
    R3 = range(3)

    gi = full(inverse(x[0:6]))
    # Christoffel symbols: chr1[i][j][k] = Gamma_ijk, chr2[i][j][k] = Gamma^i_jk (symmetric in j, k)
    chr1 = [[[0.5 * (dg[k][i][j] + dg[j][i][k] - dg[i][j][k]) for k in R3] for j in R3] for i in R3]
    chr2 = [[[vsum(gi[i][m] * chr1[m][j][k] for m in R3) for k in R3] for j in R3] for i in R3]
    divb = db[0][0] + db[1][1] + db[2][2]
    # U[k][i][n] = gt^nm Gamma^k_mi, shared by Ricci terms 4 and 5
    U = [[[vsum(gi[n][m] * chr2[k][m][i] for m in R3) for n in R3] for i in R3] for k in R3]
    # C = gt^-1 At (C[k][j] = gt^kl At_lj), Au = gt^-1 At gt^-1 (At with both indices raised)
    C = [[vsum(gi[k][l] * A[l][j] for l in R3) for j in R3] for k in R3]
    Au = [[vsum(gi[i][k] * C[j][k] for k in R3) for j in R3] for i in R3]

    out = [None] * 21
    # d_t gt_ij (spatial_metric.py:17-64)
    for s, (i, j) in enumerate(PAIRS):
        lie = vsum(g[m][i] * db[m][j] + g[m][j] * db[m][i] for m in R3)
        out[s] = lie + (-2.0 / 3.0) * g[i][j] * divb + (-2.0) * al * A[i][j]
    # d_t W (spatial_metric.py:67-106)
    out[6] = (1.0 / 3.0) * al * W * K - (1.0 / 3.0) * W * divb
    # W^2 D_i D_j alpha (geometry.py:122-186)
    giW = [vsum(gi[m][n] * dW[m] for m in R3) for n in R3]     # gt^mn d_m W
    gdWda = vsum(giW[n] * dal[n] for n in R3)
    DDa = [[None] * 3 for _ in R3]
    W2 = W * W
    for i, j in PAIRS:
        conf = d2al[i][j] - vsum(chr2[k][i][j] * dal[k] for k in R3)
        grad = dW[i] * dal[j] + dW[j] * dal[i] - g[i][j] * gdWda
        DDa[i][j] = DDa[j][i] = W2 * conf + W * grad
    # W^2 R_ij (geometry.py:21-119)
    DDW = [[None] * 3 for _ in R3]
    for i, j in PAIRS:
        DDW[i][j] = DDW[j][i] = d2W[i][j] - vsum(chr2[k][i][j] * dW[k] for k in R3)
    lapW = contract_sym(gi, DDW)
    grad2 = vsum(giW[n] * dW[n] for n in R3)
    W2R = [[None] * 3 for _ in R3]
    for i, j in PAIRS:
        t1 = -0.5 * vsum(gi[m][n] * d2g[m][n][i][j] for m in R3 for n in R3)
        t2 = 0.5 * vsum(g[m][i] * dGt[j][m] + g[m][j] * dGt[i][m] for m in R3)
        t3 = 0.5 * vsum(Gt[m] * (chr1[i][j][m] + chr1[j][i][m]) for m in R3)
        t4 = vsum(U[k][i][n] * chr1[j][k][n] + U[k][j][n] * chr1[i][k][n] for k in R3 for n in R3)
        t5 = vsum(U[k][i][n] * chr1[k][j][n] for k in R3 for n in R3)
        ricci = t1 + t2 + t3 + t4 + t5
        W2R[i][j] = W2R[j][i] = W2 * ricci + (W * (DDW[i][j] + g[i][j] * lapW) - 2.0 * g[i][j] * grad2)
    # d_t K (extrinsic_curvature.py:31-92)
    AA = contract_sym(A, Au)
    out[13] = -contract_sym(gi, DDa) + al * AA + al * K * K / 3.0
    # d_t At_ij (extrinsic_curvature.py:119-224)
    src = [[al * W2R[i][j] - DDa[i][j] for j in R3] for i in R3]
    trs = contract_sym(gi, src)
    for s, (i, j) in enumerate(PAIRS):
        first = al * K * A[i][j]
        second = -2.0 * al * vsum(A[i][k] * C[k][j] for k in R3)
        third = src[i][j] - (1.0 / 3.0) * g[i][j] * trs
        fifth = vsum(A[m][i] * db[m][j] + A[m][j] * db[m][i] for m in R3)
        sixth = (-2.0 / 3.0) * A[i][j] * divb
        out[7 + s] = first + second + third + fifth + sixth
    # d_t Gt^i (conformal_connection.py:19-162)
    Wf = vmax(W, 1.0e-12)
    grad_div = [vsum(d2b[n][m][n] for n in R3) for m in R3]
    for i in R3:
        first = (-4.0 / 3.0) * al * vsum(gi[i][j] * dK[j] for j in R3)
        second = 2.0 * al * contract_sym(chr2[i], Au)
        third = -6.0 * al / Wf * vsum(Au[i][j] * dW[j] for j in R3)
        fourth = -2.0 * vsum(Au[i][j] * dal[j] for j in R3)
        sixth = (2.0 / 3.0) * Gt[i] * divb
        seventh = -vsum(Gt[m] * db[i][m] for m in R3)
        eighth = contract_sym(gi, d2b[i])
        ninth = (1.0 / 3.0) * vsum(gi[i][m] * grad_div[m] for m in R3)
        out[14 + i] = first + second + third + fourth + sixth + seventh + eighth + ninth
    # d_t alpha, d_t beta^i (shift_and_lapse.py:65-132)
    out[17] = -(c_harm * al * al + 2.0 * c_log * al) * K
    for i in R3:
        out[18 + i] = shift_on * (gdrv * Gt[i] - eta * b[i])
    return out


def projection_algebra(x):
    """(gt, At) -> (gt det^-1/3, At - gt' tr(gt'^-1 At)/3) (time_evolve.py:94-141)."""
    g = x[0:6]
    A = x[6:12]
    det = (g[0] * g[3] * g[5] + g[1] * g[4] * g[2] + g[2] * g[1] * g[4]
           - g[2] * g[3] * g[2] - g[0] * g[4] * g[4] - g[1] * g[1] * g[5])
    s = vpow(det, -1.0 / 3.0)
    gp = [gc * s for gc in g]
    gi = full(inverse(gp))
    Af = full(A)
    tr = vsum(gi[i][j] * Af[i][j] for i in range(3) for j in range(3))
    Ap = [A[c] - (1.0 / 3.0) * gp[c] * tr for c in range(6)]
    return gp + Ap


# ----------------------------------------------------------------------------
# evaluation on NumPy arrays (CPU checks)
# ----------------------------------------------------------------------------

def evaluate(P, outs, inputs, params=None, kbar=None):
    """Values of the outputs (and, with kbar, the input adjoints) on arrays."""
    import numpy as np
    params = params or {}
    val = [None] * len(P.nodes)
    for n, (op, args, payload) in enumerate(P.nodes):
        if op == "in":
            val[n] = inputs[payload]
        elif op == "param":
            val[n] = params[payload]
        elif op == "const":
            val[n] = payload
        elif op == "add":
            val[n] = val[args[0]] + val[args[1]]
        elif op == "sub":
            val[n] = val[args[0]] - val[args[1]]
        elif op == "mul":
            val[n] = val[args[0]] * val[args[1]]
        elif op == "div":
            val[n] = val[args[0]] / val[args[1]]
        elif op == "neg":
            val[n] = -val[args[0]]
        elif op == "sqrt":
            val[n] = np.sqrt(val[args[0]])
        elif op == "powc":
            val[n] = np.power(val[args[0]], payload)
        elif op == "maxc":
            val[n] = np.maximum(val[args[0]], payload)
    result = [val[o.n] for o in outs]
    if kbar is None:
        return result
    adj = [0.0] * len(P.nodes)
    for o, kb in zip(outs, kbar):
        adj[o.n] = adj[o.n] + kb
    for n in range(len(P.nodes) - 1, -1, -1):
        op, args, payload = P.nodes[n]
        a = adj[n]
        if op in ("in", "param", "const") or (isinstance(a, float) and a == 0.0):
            continue
        if op == "add":
            adj[args[0]] = adj[args[0]] + a
            adj[args[1]] = adj[args[1]] + a
        elif op == "sub":
            adj[args[0]] = adj[args[0]] + a
            adj[args[1]] = adj[args[1]] - a
        elif op == "mul":
            adj[args[0]] = adj[args[0]] + a * val[args[1]]
            adj[args[1]] = adj[args[1]] + a * val[args[0]]
        elif op == "div":
            adj[args[0]] = adj[args[0]] + a / val[args[1]]
            adj[args[1]] = adj[args[1]] - a * val[n] / val[args[1]]
        elif op == "neg":
            adj[args[0]] = adj[args[0]] - a
        elif op == "sqrt":
            adj[args[0]] = adj[args[0]] + a * 0.5 / val[n]
        elif op == "powc":
            adj[args[0]] = adj[args[0]] + a * payload * val[n] / val[args[0]]
        elif op == "maxc":
            adj[args[0]] = adj[args[0]] + np.where(val[args[0]] > payload, a, 0.0)
    return result, {name: adj[n] for name, n in P.inputs}


def build_rhs():
    P = Program()
    x = state_inputs(P)
    prm = [P.param(p) for p in PARAMS]
    return P, rhs_algebra(x, prm)


def build_projection():
    P = Program()
    x = [P.input(f"x{i}") for i in range(12)]
    return P, projection_algebra(x)


# ----------------------------------------------------------------------------
# CUDA emission
# ----------------------------------------------------------------------------

def _lit(c):
    if c == int(c) and abs(c) < 1e15:
        return f"{int(c)}.0"
    return repr(c)


def _live(P, outs):
    """Nodes the outputs depend on."""
    need = [False] * len(P.nodes)
    stack = [o.n for o in outs]
    while stack:
        n = stack.pop()
        if need[n]:
            continue
        need[n] = True
        stack.extend(P.nodes[n][1])
    return need


def _expr(P, n, name):
    op, args, payload = P.nodes[n]
    a = [name(k) for k in args]
    if op == "add":
        return f"{a[0]} + {a[1]}"
    if op == "sub":
        return f"{a[0]} - {a[1]}"
    if op == "mul":
        return f"{a[0]} * {a[1]}"
    if op == "div":
        return f"{a[0]} / {a[1]}"
    if op == "neg":
        return f"-{a[0]}"
    if op == "sqrt":
        return f"sqrt({a[0]})"
    if op == "powc":
        if payload == -1.0 / 3.0:
            return f"rcbrt({a[0]})"
        return f"pow({a[0]}, {_lit(payload)})"
    if op == "maxc":
        return f"fmax({a[0]}, {_lit(payload)})"
    raise ValueError(op)


def emit_function(P, outs, fname, nin, nout, vjp, param_names=()):
    """C++ for the forward (vjp=False) or the reverse sweep (vjp=True)."""
    need = _live(P, outs)
    in_index = {n: int(name[1:]) for name, n in P.inputs}
    par_index = {n: name for name, n in P.params}

    def name(n):
        op, _, payload = P.nodes[n]
        if op == "in":
            return f"x[{in_index[n]}]"
        if op == "param":
            return f"pp.{payload}"
        if op == "const":
            return _lit(payload)
        return f"t{n}"

    lines = []
    if vjp:
        sig = (f"__device__ __forceinline__ void {fname}(const double (&x)[{nin}], const double (&kbar)[{nout}]"
               + (", const PointParams& pp" if param_names else "") + f", double (&xbar)[{nin}])")
    else:
        sig = (f"__device__ __forceinline__ void {fname}(const double (&x)[{nin}]"
               + (", const PointParams& pp" if param_names else "") + f", double (&y)[{nout}])")
    lines.append(sig + " {")
    if not vjp:
        for n, (op, args, payload) in enumerate(P.nodes):
            if need[n] and op not in ("in", "param", "const"):
                lines.append(f"    const double t{n} = {_expr(P, n, name)};")
        for k, o in enumerate(outs):
            lines.append(f"    y[{k}] = {name(o.n)};")
        lines.append("}")
        return "\n".join(lines)
    forward_at = len(lines)
    # reverse sweep: node adjoints as sums of their contributions, each
    # emitted once all users of the node (which come later) are processed;
    # input adjoints accumulate into xbar.
    contrib = {}

    def add(n, expr):
        if P.nodes[n][0] in ("const", "param"):
            return
        contrib.setdefault(n, []).append(expr)

    for k, o in enumerate(outs):
        add(o.n, f"kbar[{k}]")
    for n in range(len(P.nodes) - 1, -1, -1):
        op, args, payload = P.nodes[n]
        if not need[n] or op in ("in", "param", "const") or n not in contrib:
            continue
        terms = contrib.pop(n)
        if all(P.nodes[k][0] in ("const", "param") for k in args):
            continue   # nothing upstream takes an adjoint
        lines.append(f"    const double a{n} = {' + '.join(terms)};")
        a = f"a{n}"
        if op == "add":
            add(args[0], a)
            add(args[1], a)
        elif op == "sub":
            add(args[0], a)
            add(args[1], f"-{a}")
        elif op == "mul":
            add(args[0], f"{a} * {name(args[1])}")
            add(args[1], f"{a} * {name(args[0])}")
        elif op == "div":
            add(args[0], f"{a} / {name(args[1])}")
            add(args[1], f"-{a} * t{n} / {name(args[1])}")
        elif op == "neg":
            add(args[0], f"-{a}")
        elif op == "sqrt":
            add(args[0], f"{a} * 0.5 / t{n}")
        elif op == "powc":
            add(args[0], f"{a} * {_lit(payload)} * t{n} / {name(args[0])}")
        elif op == "maxc":
            add(args[0], f"({name(args[0])} > {_lit(payload)} ? {a} : 0.0)")
    for name_, n in P.inputs:
        terms = contrib.pop(n, [])
        k = int(name_[1:])
        lines.append(f"    xbar[{k}] = {' + '.join(terms) if terms else '0.0'};")
    lines.append("}")
    # forward values the reverse sweep reads, and what they depend on
    import re
    used = {int(m) for line in lines[forward_at:] for m in re.findall(r"\bt(\d+)\b", line)}
    keep = set()
    stack = list(used)
    while stack:
        n = stack.pop()
        if n in keep or P.nodes[n][0] in ("in", "param", "const"):
            continue
        keep.add(n)
        stack.extend(P.nodes[n][1])
    forward = [f"    const double t{n} = {_expr(P, n, name)};" for n in range(len(P.nodes)) if n in keep]
    lines[forward_at:forward_at] = forward
    return "\n".join(lines)


HEADER = '''// Generated by gen_adjoint.py -- do not edit by hand.
//
// Pointwise BSSN algebra (kappa = 0, vacuum) and its reverse sweep.  Input
// layout x[132]: state values (21, component order), d_k gt (18), d_k W (3),
// d_k alpha (3), d_k K (3), d_j beta^i (9), d_d Gt^i (9), d_m d_n gt (36),
// d_m d_n W (6), d_m d_n alpha (6), d_m d_n beta^i (18); see gen_adjoint.py.
#pragma once

namespace bssn {
namespace adjoint {

constexpr int kPointInputs = 132;

// Runtime scalars of the pointwise algebra: eta, the Gamma-driver factor g,
// the slicing selectors (harmonic: c_harm = 1; 1+log: c_log = 1) and
// shift_on = 1 - zero_shift.
struct PointParams {
    double eta, gdrv, c_harm, c_log, shift_on;
};

'''


def generate() -> str:
    P, outs = build_rhs()
    parts = [HEADER]
    parts.append(emit_function(P, outs, "rhs_point_forward", NIN, 21, False, PARAMS))
    parts.append("")
    parts.append(emit_function(P, outs, "rhs_point_vjp", NIN, 21, True, PARAMS))
    parts.append("")
    Q, qouts = build_projection()
    parts.append(emit_function(Q, qouts, "project_point_forward", 12, 12, False))
    parts.append("")
    parts.append(emit_function(Q, qouts, "project_point_vjp", 12, 12, True))
    parts.append("")
    parts.append("}  // namespace adjoint\n}  // namespace bssn\n")
    return "\n".join(parts)


if __name__ == "__main__":
    text = generate()
    TARGET.write_text(text)
    print(f"wrote {TARGET} ({text.count(chr(10))} lines)")
