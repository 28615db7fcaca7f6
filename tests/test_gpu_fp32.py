"""The FP32-arithmetic forms (float RHS arithmetic, float64 state and RK4;
"fp32_paired" also holds the second-derivative fields as float pairs)
against the float64 reference goldens.

Error metric: per leaf, max|fp32-form - ref| divided by the leaf's deviation
from its flat background, max|ref - background| (background 1 on the
conformal-metric diagonal, W and alpha, 0 elsewhere).  That is the relative
error of the physics the state carries: for a 1e-5 wave on a unit metric a
plain max|ref| normalisation would hide five digits.  Tolerances, stated per
test, follow float's 6e-8 unit roundoff amplified by the stencils (up to
about 64/12 / (dx^2 k^2) for the second derivatives) and stay far below the
discretisation error of these grids.
"""

import json

import numpy as np
import pytest

from oracle.state import BSSNVariables as OracleVars

from .helpers import LEAVES, RHS_CASES, golden_params, golden_state, load_golden

pytestmark = pytest.mark.gpu

BACKGROUND = {"conformal_metric": np.eye(3)[:, :, None, None, None], "conformal_factor": 1.0,
              "traceless_K": 0.0, "trace_K": 0.0, "conformal_connection": 0.0, "lapse": 1.0, "shift": 0.0}


def _np(x):
    return x.detach().cpu().numpy() if hasattr(x, "detach") else np.asarray(x)


def deviation_errors(got, ref, background=True):
    """max|got - ref| / max(|ref - bg|) per leaf (bg = flat background or 0)."""
    out = {}
    for leaf, x, y in zip(LEAVES, got, ref):
        x, y = _np(x), _np(y)
        bg = BACKGROUND[leaf] if background else 0.0
        scale = float(np.max(np.abs(y - bg)))
        out[leaf] = float(np.max(np.abs(x - y))) / scale if scale > 0 else float(np.max(np.abs(x - y)))
    return out


@pytest.fixture(scope="module")
def gb(cuda, native):
    import jax_bssn_gb300 as pkg
    from jax_bssn_gb300.evolution import time_evolve
    return pkg, time_evolve


FORMS = ["fp32", "fp32_paired"]


def _inputs(data, pkg):
    return golden_state(data, "input", pkg.BSSNVariables), golden_params(data, pkg.BSSNParameters)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("name", RHS_CASES)
def test_fp32_rhs_against_reference(gb, name, form):
    """RHS of the FP32 form, error relative to the reference RHS's own scale."""
    pkg, te = gb
    data = load_golden(f"rhs_{name}")
    state, params = _inputs(data, pkg)
    with pkg.arithmetic(form):
        rhs = te.compute_bssn_rhs(state, params)
    err = deviation_errors(rhs, golden_state(data, "rhs", OracleVars), background=False)
    print(name, "fp32 rhs", {k: f"{v:.1e}" for k, v in err.items()})
    assert max(err.values()) < 2e-4


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("name", RHS_CASES)
def test_fp32_rk4_step_against_reference(gb, name, form):
    pkg, te = gb
    data = load_golden(f"rhs_{name}")
    state, params = _inputs(data, pkg)
    with pkg.arithmetic(form):
        one = te.rk4_step(state, params)
    err = deviation_errors(one, golden_state(data, "rk4_1", OracleVars))
    print(name, "fp32 rk4 1", {k: f"{v:.1e}" for k, v in err.items()})
    assert max(err.values()) < 1e-5


def test_fp32_gauge_wave_hundred_steps(gb):
    """32^3 gauge wave (A = 0.1): after 100 steps the FP32 form stays within
    1e-5 of the float64 reference relative to the wave's amplitude."""
    pkg, te = gb
    data = load_golden("run_gauge_wave32")
    state, params = _inputs(data, pkg)
    with pkg.arithmetic("fp32"):
        hundred = te.rk4_steps(state, params, 100)
    err = deviation_errors(hundred, golden_state(data, "rk4_100", OracleVars))
    print("fp32 gauge wave 100", {k: f"{v:.1e}" for k, v in err.items()})
    assert max(err.values()) < 1e-5


@pytest.mark.parametrize("form", FORMS)
def test_fp32_teukolsky_ten_steps_and_constraint_norms(gb, form):
    """Teukolsky 24^3 (amplitude 1e-5, Sommerfeld faces): ten steps, then the
    Hamiltonian and momentum constraint L2 norms within 1% of the float64 run's."""
    pkg, te = gb
    from jax_bssn_gb300.bssn.constraints import compute_all_constraints, compute_constraint_norms
    data = load_golden("run_teukolsky24")
    state, params = _inputs(data, pkg)
    with pkg.arithmetic(form):
        ten = te.rk4_steps(state, params, 10)
    ref = golden_state(data, "rk4_10", OracleVars)
    err = deviation_errors(ten, ref)
    print("fp32 teukolsky 10", {k: f"{v:.1e}" for k, v in err.items()})
    assert max(err.values()) < 1e-4
    n32 = compute_constraint_norms(compute_all_constraints(ten, params))
    n64 = compute_constraint_norms(compute_all_constraints(pkg.BSSNVariables(*ref), params))
    for key in ("hamiltonian_l2", "momentum_l2"):
        print(key, n32[key], n64[key])
        assert n32[key] == pytest.approx(n64[key], rel=1e-2), key


@pytest.mark.parametrize("form", FORMS)
def test_fp32_resident_patch_matches_drop_in(gb, form):
    pkg, te = gb
    from jax_bssn_gb300.evolution import PatchEvolution
    data = load_golden("run_teukolsky24")
    state, params = _inputs(data, pkg)
    evo = PatchEvolution(state, params, precision=form)
    evo.step(3)
    with pkg.arithmetic(form):
        want = te.rk4_steps(state, params, 3)
    for a, b in zip(evo.state(), want):
        np.testing.assert_array_equal(_np(a), _np(b))


@pytest.mark.parametrize("form", FORMS)
def test_fp32_fmr_against_reference(gb, form):
    """Nested FMR (three levels, MAD): two stage-synchronous RK4 steps."""
    pkg, _ = gb
    from jax_bssn_gb300.fmr import FMRHierarchySpec, FMRPatchSpec, TileLayout, fmr_rk4_step, prepare_fmr_states
    from .fmr_helpers import G, load_case, owned_of, owned_states
    data, hierarchy, oparams, shapes, _ = load_case("three_level_mad")
    h = FMRHierarchySpec(tuple(FMRPatchSpec(s.coarse_lo, s.coarse_hi, parent=s.parent) for s in hierarchy.patches),
                         use_mad=hierarchy.use_mad)
    params = tuple(pkg.BSSNParameters(**p._asdict()) for p in oparams)
    layouts = tuple(TileLayout(n) for n in shapes)
    raw = []
    for s, n in zip(owned_states(data, "initial", len(shapes)), shapes):
        leaves = []
        for leaf in s:
            full = np.zeros(leaf.shape[:-3] + tuple(m + 2 * G for m in n))
            full[(Ellipsis,) + tuple(slice(G, G + m) for m in n)] = leaf
            leaves.append(full.reshape(leaf.shape[:-3] + (1, 1, 1) + full.shape[-3:]))
        raw.append(pkg.BSSNVariables(*leaves))
    initial = prepare_fmr_states(tuple(raw), params, h, layouts=layouts, project=False)
    with pkg.arithmetic(form):
        two = fmr_rk4_step(fmr_rk4_step(initial, params, h, layouts=layouts), params, h, layouts=layouts)
    expect = owned_states(data, "rk4_2", len(shapes))
    for p, n in enumerate(shapes):
        got = OracleVars(*(_np(leaf).reshape(_np(leaf).shape[:-6] + _np(leaf).shape[-3:]) for leaf in two[p]))
        err = deviation_errors(owned_of(got, n), expect[p])
        print("fp32 fmr patch", p, {k: f"{v:.1e}" for k, v in err.items()})
        assert max(err.values()) < 1e-5, (p, err)


@pytest.mark.parametrize("form", FORMS)
def test_fp32_cartoon_against_reference(gb, form):
    pkg, _ = gb
    from jax_bssn_gb300.cartoon.axisymmetry import axisymmetric_rk4_step, compute_axisymmetric_rhs
    from jax_bssn_gb300.cartoon.spherical_symmetry import cartoon_rk4_step
    data = load_golden("cartoon_axisymmetric")
    state, params = _inputs(data, pkg)
    with pkg.arithmetic(form):
        rhs = compute_axisymmetric_rhs(state, params)
        two = axisymmetric_rk4_step(axisymmetric_rk4_step(state, params), params)
    e_rhs = deviation_errors(rhs, golden_state(data, "rhs", OracleVars), background=False)
    e_two = deviation_errors(two, golden_state(data, "rk4_2", OracleVars))
    print("fp32 axisymmetric rhs", f"{max(e_rhs.values()):.1e}", "rk4 2", f"{max(e_two.values()):.1e}")
    assert max(e_rhs.values()) < 2e-4
    assert max(e_two.values()) < 1e-5
    data = load_golden("cartoon_spherical")
    state, params = _inputs(data, pkg)
    with pkg.arithmetic(form):
        two = cartoon_rk4_step(cartoon_rk4_step(state, params), params)
    e_two = deviation_errors(two, golden_state(data, "rk4_2", OracleVars))
    print("fp32 spherical rk4 2", {k: f"{v:.1e}" for k, v in e_two.items()})
    assert max(e_two.values()) < 1e-5


def test_paired_form_removes_the_second_derivative_rounding(gb):
    """A 1e-8 plus-polarised wave at spacing 1/24 (the finest level of the
    benchmarked FMR hierarchy), periodic.  Float rounding of the metric's
    samples, amplified by 1/dx^2 in the Ricci tensor, dominates the plain
    FP32 RHS of At (about eps * 5 / (k dx)^2 of the signal); at this spacing
    even the FP64 form's unit-background numerators round at ~1e-5 of the
    signal.  Against the oracle evaluated in long double on the same input
    bits, the paired form must be at least five times more accurate than the
    plain FP32 form and within twice the FP64 form's error."""
    pkg, te = gb
    from oracle import bssn as ob
    from oracle.state import BSSNParameters as OracleParams
    from jax_bssn_gb300.initial_data import linear_wave_state
    n, dx = 96, 1.0 / 24.0
    x = -2.0 + dx * np.arange(n)
    X, Y, Z = np.meshgrid(x, x[:8], x[:8], indexing="ij")
    host = linear_wave_state(X, Y, Z, 1.0e-8, 4.0)
    state = pkg.BSSNVariables(*host)
    kw = dict(dx=dx, dt=0.25 * dx, eta=0.0, kappa=0.0, nu=0.0, g=0.0, zero_shift=1, gauge=0)
    params = pkg.BSSNParameters(**kw)
    wide = ob.compute_rhs(OracleVars(*(np.asarray(f, dtype=np.longdouble) for f in host)), OracleParams(**kw))
    ref = np.asarray(wide.traceless_K, dtype=np.float64)
    err = {}
    for form in ["fp64"] + FORMS:
        with pkg.arithmetic(form):
            got = _np(te.compute_bssn_rhs(state, params).traceless_K)
        err[form] = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
    print("At rhs error against the long-double oracle", {k: f"{v:.1e}" for k, v in err.items()})
    assert err["fp32_paired"] < 0.2 * err["fp32"], err
    assert err["fp32_paired"] < 2.0 * err["fp64"], err


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("faces,shape", [("periodic", (24, 20, 24)), ("sommerfeld", (24, 20, 24)),
                                         ("sommerfeld", (23, 22, 20)), ("sommerfeld", (26, 21, 28)),
                                         ("sommerfeld", (18, 25, 24)), ("sommerfeld_x_z", (21, 23, 24))])
def test_tma_kernels_match_the_generic_kernels(gb, form, faces, shape):
    """The FP32 forms' TMA-staged kernels (the gauge RHS, the first
    derivatives, dt At and dt K with dt Gt; z pitch a multiple of four) against
    the generic kernels on the same state: every RHS leaf equal to float
    rounding (1e-6 of its scale), with no tile wait given up.  With Sommerfeld
    faces the box kernels also take the rows next to the faces (their
    one-sided stencils, and at the upper faces lowered box origins), and the
    first derivatives the face planes too: the shapes put those rows at
    several positions within a tile along x and y."""
    pkg, te = gb
    from jax_bssn_gb300 import _native
    from jax_bssn_gb300.initial_data import random_smooth_state
    state = random_smooth_state(shape, seed=8)
    kw = dict(eta=1.5, kappa=0.0, nu=0.05, g=0.75, dx=0.08, dt=0.02, gauge=1)
    if faces == "sommerfeld":
        kw.update(xl_bc=1, xr_bc=1, yl_bc=1, yr_bc=1, zl_bc=1, zr_bc=1, x_min=-1.0, y_min=-0.8, z_min=-0.9)
    elif faces == "sommerfeld_x_z":   # y periodic: the boxes wrap through its filled ghosts
        kw.update(xl_bc=1, xr_bc=1, zl_bc=1, zr_bc=1, x_min=-1.0, y_min=0.0, z_min=-0.9)
    params = pkg.BSSNParameters(**kw)
    _, before = _native.tma_status()
    with pkg.arithmetic(form):
        try:
            _native.set_tma(_native.TMA_ALL)
            tiled = te.compute_bssn_rhs(state, params)
            _, after = _native.tma_status()
            _native.set_tma(False)
            generic = te.compute_bssn_rhs(state, params)
        finally:
            _native.set_tma(True)   # the library's default
    timeouts, last = _native.tma_status()
    assert after == before + 4 and last == after, (before, after, last)   # the four kernels tiled, then none
    assert timeouts == 0
    for leaf in ("conformal_metric", "conformal_factor", "traceless_K", "trace_K", "conformal_connection", "lapse",
                 "shift"):
        a, b = _np(getattr(tiled, leaf)), _np(getattr(generic, leaf))
        scale = float(np.max(np.abs(b)))
        err = float(np.max(np.abs(a - b))) / scale
        print(form, faces, shape, leaf, f"{err:.1e}")
        assert err < 1e-6, (leaf, err)


@pytest.mark.parametrize("form", FORMS)
def test_tma_kernels_match_the_generic_kernels_on_the_benchmarked_grid(gb, form):
    """The same comparison on the benchmarked Teukolsky 128^3 grid, Sommerfeld
    on every face, where the box kernels take the whole box minus the face
    planes, closure rows included.  The wave is first evolved 8 FP64 steps, so
    that At, K and the shift (zero in the initial data) carry signal too."""
    pkg, te = gb
    from jax_bssn_gb300 import _native
    from jax_bssn_gb300.evolution import PatchEvolution
    from jax_bssn_gb300.initial_data import teukolsky_config
    state0, params = teukolsky_config(n=128)
    evo = PatchEvolution(state0, params, precision="fp64")
    evo.step(8)
    state = evo.state()
    del evo
    _, before = _native.tma_status()
    with pkg.arithmetic(form):
        try:
            _native.set_tma(_native.TMA_ALL)
            tiled = te.compute_bssn_rhs(state, params)
            _, after = _native.tma_status()
            _native.set_tma(False)
            generic = te.compute_bssn_rhs(state, params)
        finally:
            _native.set_tma(True)
    timeouts, last = _native.tma_status()
    assert after == before + 4 and last == after, (before, after, last)
    assert timeouts == 0
    for leaf in ("conformal_metric", "conformal_factor", "traceless_K", "trace_K", "conformal_connection", "lapse",
                 "shift"):
        a, b = _np(getattr(tiled, leaf)), _np(getattr(generic, leaf))
        scale = float(np.max(np.abs(b)))
        err = float(np.max(np.abs(a - b))) / scale if scale > 0 else float(np.max(np.abs(a)))
        print(form, "teukolsky 128^3", leaf, f"{err:.1e}")
        assert err < 1e-6, (leaf, err)


def test_precision_argument_is_validated(gb):
    pkg, _ = gb
    with pytest.raises(ValueError):
        with pkg.arithmetic("fp16"):
            pass
