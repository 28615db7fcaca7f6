"""The adjoint generator's pointwise algebra, checked on the CPU.

gen_adjoint.py restates the BSSN right-hand side as a function of the state
values and their finite-difference derivatives and emits its reverse sweep.
Here its NumPy evaluation is checked against the oracle's RHS (minus the
advection and dissipation stencils, which the adjoint kernels transpose
directly), the reverse sweep against central differences of the forward, and
the committed CUDA header against a fresh generation.
"""

import importlib.util
from pathlib import Path

import numpy as np
import pytest

from oracle import bssn as ob
from oracle.state import BSSNParameters as OP, BSSNVariables as OV
from oracle.stencils import D1, D2, kreiss_oliger

ROOT = Path(__file__).resolve().parents[1]
_spec = importlib.util.spec_from_file_location("gen_adjoint", ROOT / "jax_bssn_gb300" / "csrc" / "gen_adjoint.py")
gen = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(gen)

PAIRS = gen.PAIRS


def _state_and_params(seed, **kw):
    from jax_bssn_gb300.initial_data import random_smooth_state
    state = random_smooth_state((10, 9, 11), seed=seed)
    base = dict(eta=1.5, kappa=0.0, nu=0.07, g=0.75, dx=0.09, dt=0.01, gauge=1, zero_shift=0)
    base.update(kw)
    return OV(*(np.asarray(f) for f in state)), OP(**base)


def _components(v):
    g, W, A, K, G, al, b = (np.asarray(f) for f in v)
    return ([g[i, j] for i, j in PAIRS] + [W] + [A[i, j] for i, j in PAIRS] + [K] + [G[i] for i in range(3)]
            + [al] + [b[i] for i in range(3)])


def _pointwise_inputs(v, p):
    """The generator's 132 inputs from the oracle's own stencils."""
    u = _components(v)
    g = np.asarray(v.conformal_metric)
    x = list(u)
    x += [D1(g[i, j], k, p) for k in range(3) for i, j in PAIRS]
    x += [D1(v.conformal_factor, k, p) for k in range(3)]
    x += [D1(v.lapse, k, p) for k in range(3)]
    x += [D1(v.trace_K, k, p) for k in range(3)]
    x += [D1(v.shift[i], j, p) for i in range(3) for j in range(3)]
    x += [D1(v.conformal_connection[i], d, p) for d in range(3) for i in range(3)]

    def second(f, m, n):
        return D2(f, m, p) if m == n else D1(D1(f, m, p), n, p)
    x += [second(g[i, j], m, n) for m, n in PAIRS for i, j in PAIRS]
    x += [second(v.conformal_factor, m, n) for m, n in PAIRS]
    x += [second(v.lapse, m, n) for m, n in PAIRS]
    x += [second(v.shift[i], m, n) for i in range(3) for m, n in PAIRS]
    assert len(x) == gen.NIN
    return {f"x{i}": np.asarray(a, dtype=np.float64) for i, a in enumerate(x)}


def _params(p):
    return {"eta": p.eta, "gdrv": p.g, "c_harm": float(p.gauge == 0), "c_log": float(p.gauge == 1),
            "shift_on": float(p.zero_shift == 0)}


@pytest.mark.parametrize("kw", [dict(), dict(gauge=0, zero_shift=1, eta=0.0), dict(mad_q=1.0 / 16.0)])
def test_pointwise_algebra_matches_oracle_rhs(kw):
    v, p = _state_and_params(4, **kw)
    P, outs = gen.build_rhs()
    F = gen.evaluate(P, outs, _pointwise_inputs(v, p), _params(p))
    full = _components(ob.compute_rhs(v, p))
    geo = ob.Geometry(v, p)
    u = _components(v)
    for c in range(21):
        linear = 0.0 if (c >= 18 and p.zero_shift) else geo.advect(u[c]) + kreiss_oliger(u[c], p)
        expect = full[c] - linear
        scale = max(np.max(np.abs(full[c])), 1e-300)
        err = np.max(np.abs(F[c] - expect)) / scale
        assert err < 1e-12, (c, err)


def test_reverse_sweep_matches_central_differences():
    v, p = _state_and_params(7, gauge=1, eta=0.8)
    P, outs = gen.build_rhs()
    x = _pointwise_inputs(v, p)
    prm = _params(p)
    rng = np.random.default_rng(0)
    shape = x["x0"].shape
    kbar = [rng.standard_normal(shape) for _ in range(21)]
    _, xbar = gen.evaluate(P, outs, x, prm, kbar)
    for trial in range(3):
        dirs = {k: rng.standard_normal(shape) * max(np.max(np.abs(a)), 1e-3) for k, a in x.items()}
        h = 1e-6
        plus = gen.evaluate(P, outs, {k: x[k] + h * dirs[k] for k in x}, prm)
        minus = gen.evaluate(P, outs, {k: x[k] - h * dirs[k] for k in x}, prm)
        fd = sum(kb * (a - b) for kb, a, b in zip(kbar, plus, minus)) / (2 * h)
        ad = sum(xbar[k] * dirs[k] for k in x)
        err = np.max(np.abs(ad - fd)) / np.max(np.abs(fd))
        assert err < 1e-7, (trial, err)


def test_projection_matches_oracle_and_its_reverse_sweep():
    v, _ = _state_and_params(9)
    g = np.asarray(v.conformal_metric)
    A = np.asarray(v.traceless_K)
    Q, qouts = gen.build_projection()
    x = {f"x{c}": g[i, j] for c, (i, j) in enumerate(PAIRS)}
    x.update({f"x{6 + c}": A[i, j] for c, (i, j) in enumerate(PAIRS)})
    y = gen.evaluate(Q, qouts, x)
    ref = ob.project(v)
    for c, (i, j) in enumerate(PAIRS):
        assert np.max(np.abs(y[c] - ref.conformal_metric[i, j])) < 1e-14
        assert np.max(np.abs(y[6 + c] - ref.traceless_K[i, j])) < 1e-14
    rng = np.random.default_rng(1)
    kbar = [rng.standard_normal(g.shape[2:]) for _ in range(12)]
    _, xbar = gen.evaluate(Q, qouts, x, None, kbar)
    dirs = {k: rng.standard_normal(g.shape[2:]) for k in x}
    h = 1e-6
    plus = gen.evaluate(Q, qouts, {k: x[k] + h * dirs[k] for k in x})
    minus = gen.evaluate(Q, qouts, {k: x[k] - h * dirs[k] for k in x})
    fd = sum(kb * (a - b) for kb, a, b in zip(kbar, plus, minus)) / (2 * h)
    ad = sum(xbar[k] * dirs[k] for k in x)
    assert np.max(np.abs(ad - fd)) / np.max(np.abs(fd)) < 1e-8


def test_committed_cuda_header_is_current():
    assert gen.TARGET.read_text() == gen.generate(), "run jax_bssn_gb300/csrc/gen_adjoint.py"
