"""FMR on the GPU (through the C ABI) against the reference's tiled FMR goldens.

The initial tiled states are rebuilt from the stored owned samples exactly as
the reference's initialize_tiled_fmr does (refresh + prolongation); the
oracle reproduces the reference bit for bit, so halo/prolongation results are
expected to agree exactly and the evolved states to the parity tolerances.
"""

import json

import numpy as np
import pytest

from oracle import fmr as ofmr
from oracle.state import BSSNVariables as OracleVars

from .fmr_helpers import G, load_case, owned_of, owned_states
from .helpers import assert_norms_match, LEAVES, field_errors, worst

pytestmark = pytest.mark.gpu

CASES = ("three_level_mad", "sommerfeld_kappa", "siblings_no_mad")
RHS_TOL = 1e-11
STEP_TOL = 1e-12


def _tiled(state):
    """Patch arrays (..., P, P, P) -> the reference's tiled layout (..., 1, 1, 1, P, P, P)."""
    out = []
    for leaf in state:
        a = np.asarray(leaf)
        out.append(a.reshape(a.shape[:-3] + (1, 1, 1) + a.shape[-3:]))
    return tuple(out)


def _untile(state):
    out = []
    for leaf in state:
        a = leaf.detach().cpu().numpy() if hasattr(leaf, "detach") else np.asarray(leaf)
        out.append(a.reshape(a.shape[:-6] + a.shape[-3:]))
    return OracleVars(*out)


@pytest.fixture(scope="module", params=CASES)
def gpu_case(request, cuda, native):
    from jax_bssn_gb300 import BSSNParameters, BSSNVariables
    from jax_bssn_gb300.fmr import FMRHierarchySpec, FMRPatchSpec, TileLayout
    name = request.param
    data, hierarchy, oparams, shapes, oracle_initial = load_case(name)
    h = FMRHierarchySpec(tuple(FMRPatchSpec(s.coarse_lo, s.coarse_hi, parent=s.parent) for s in hierarchy.patches),
                         use_mad=hierarchy.use_mad)
    params = tuple(BSSNParameters(**p._asdict()) for p in oparams)
    layouts = tuple(TileLayout(n) for n in shapes)
    raw = []
    for s, n in zip(owned_states(data, "initial", len(shapes)), shapes):
        leaves = []
        for leaf in s:
            full = np.zeros(leaf.shape[:-3] + tuple(m + 2 * G for m in n))
            full[(Ellipsis,) + tuple(slice(G, G + m) for m in n)] = leaf
            leaves.append(full.reshape(leaf.shape[:-3] + (1, 1, 1) + full.shape[-3:]))
        raw.append(BSSNVariables(*leaves))
    return name, data, h, params, layouts, shapes, tuple(raw), oracle_initial, hierarchy, oparams


def test_initialisation_refresh_and_prolongation_bitwise(gpu_case):
    from jax_bssn_gb300.fmr import prepare_fmr_states
    name, data, h, params, layouts, shapes, raw, oracle_initial, _, _ = gpu_case
    got = prepare_fmr_states(raw, params, h, layouts=layouts, project=False)
    for p in range(len(shapes)):
        assert worst(field_errors(_untile(got[p]), oracle_initial[p])) == 0.0, (name, p)


def test_stage_matches_reference(gpu_case):
    from jax_bssn_gb300.fmr import fmr_stage, prepare_fmr_states
    name, data, h, params, layouts, shapes, raw, _, _, _ = gpu_case
    initial = prepare_fmr_states(raw, params, h, layouts=layouts, project=False)
    prepared, rhs = fmr_stage(initial, params, h, layouts=layouts)
    expect = owned_states(data, "stage1_rhs", len(shapes))
    for p, n in enumerate(shapes):
        err = field_errors(owned_of(_untile(rhs[p]), n), expect[p])
        print(name, "stage rhs", p, f"{worst(err):.2e}")
        assert worst(err) < RHS_TOL, (name, p, err)
    last = len(shapes) - 1
    shell = OracleVars(*(data[f"stage1_prepared.{last}.{leaf}"] for leaf in LEAVES))
    assert worst(field_errors(_untile(prepared[last]), shell)) == 0.0


def test_rk4_steps_and_norms_match_reference(gpu_case):
    from jax_bssn_gb300.fmr import fmr_constraint_norms, fmr_rk4_step, prepare_fmr_states
    name, data, h, params, layouts, shapes, raw, _, _, _ = gpu_case
    initial = prepare_fmr_states(raw, params, h, layouts=layouts, project=False)
    one = fmr_rk4_step(initial, params, h, layouts=layouts)
    expect = owned_states(data, "rk4_1", len(shapes))
    for p, n in enumerate(shapes):
        err = field_errors(owned_of(_untile(one[p]), n), expect[p])
        print(name, "rk4 1", p, f"{worst(err):.2e}")
        assert worst(err) < STEP_TOL, (name, p, err)
    last = len(shapes) - 1
    padded = OracleVars(*(data[f"rk4_1_padded.{last}.{leaf}"] for leaf in LEAVES))
    assert worst(field_errors(_untile(one[last]), padded)) < STEP_TOL
    two = fmr_rk4_step(one, params, h, layouts=layouts)
    expect = owned_states(data, "rk4_2", len(shapes))
    for p, n in enumerate(shapes):
        assert worst(field_errors(owned_of(_untile(two[p]), n), expect[p])) < 2 * STEP_TOL, (name, p)
    norms = fmr_constraint_norms(two, params, h, layouts=layouts)
    ref = json.loads(str(data["norms"]))
    assert_norms_match(norms, ref)


def test_resident_evolution_matches_drop_in(gpu_case):
    from jax_bssn_gb300.fmr import FMREvolution, fmr_rk4_steps, prepare_fmr_states
    name, data, h, params, layouts, shapes, raw, _, _, _ = gpu_case
    initial = prepare_fmr_states(raw, params, h, layouts=layouts, project=False)
    ref = fmr_rk4_steps(initial, params, h, 2, layouts=layouts)
    evo = FMREvolution(initial, params, h, layouts)
    evo.step(2)
    for got, want in zip(evo.states(), ref):
        assert worst(field_errors(_untile(got), _untile(want))) == 0.0


def test_transfers_match_oracle(gpu_case):
    from jax_bssn_gb300.fmr import fill_tiled_fine_ghosts, restrict_tiled_to_coarse
    name, data, h, params, layouts, shapes, raw, oracle_initial, ohier, _ = gpu_case
    from oracle.fmr import parents_of
    parents = parents_of(ohier)
    child = len(shapes) - 1
    parent = parents[child]
    spec = h.patches[child - 1]
    tiled = [_tiled(s) for s in oracle_initial]
    from jax_bssn_gb300 import BSSNVariables
    got = fill_tiled_fine_ghosts(BSSNVariables(*tiled[parent]), BSSNVariables(*tiled[child]), spec,
                                 parent_layout=layouts[parent], child_layout=layouts[child])
    expect = ofmr.prolong(oracle_initial[parent], oracle_initial[child], ohier.patches[child - 1], shapes[child])
    assert worst(field_errors(_untile(got), expect)) == 0.0
    got = restrict_tiled_to_coarse(BSSNVariables(*tiled[parent]), BSSNVariables(*tiled[child]), spec,
                                   parent_layout=layouts[parent], child_layout=layouts[child])
    expect = ofmr.inject(oracle_initial[parent], oracle_initial[child], ohier.patches[child - 1], shapes[child])
    assert worst(field_errors(_untile(got), expect)) == 0.0


def test_child_crossing_a_physical_root_face_is_rejected(cuda, native):
    from jax_bssn_gb300 import BSSNParameters
    from jax_bssn_gb300.fmr import FMRHierarchySpec, FMRPatchSpec, initialize_tiled_fmr
    params = BSSNParameters(dx=0.1, dt=0.01, xl_bc=1, xr_bc=1, x_min=-0.5, y_min=-0.5, z_min=-0.5)
    with pytest.raises(ValueError):
        initialize_tiled_fmr(None, params, (10, 10, 10), FMRHierarchySpec((FMRPatchSpec((2,) * 3, (5,) * 3),)))
