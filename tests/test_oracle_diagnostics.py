"""Oracle wave diagnostics against goldens from the reference
(diagnostics/waves.py) and the reference suite's known answers."""

import numpy as np

from oracle import diagnostics as od
from oracle.fmr import FMRHierarchySpec, FMRPatchSpec
from oracle.state import BSSNParameters, BSSNVariables

from .helpers import golden_params, golden_state, load_golden
from .wave_cases import assert_close, branching_tree, golden_tree, padded, vertex_count_tree


def test_h_plus_and_fields_match_reference():
    data = load_golden("waves")
    state = golden_state(data, "input", BSSNVariables)
    params = golden_params(data, BSSNParameters)
    assert np.array_equal(od.h_plus(state), data["h_plus"])
    fields = od.diagnostic_fields(state, params)
    assert np.array_equal(fields["hamiltonian_constraint"], data["hamiltonian"])
    assert np.array_equal(np.stack(fields["momentum_constraint"]), data["momentum"])


def test_composite_norms_match_reference():
    hierarchy, levels, coords, scalars, expect = golden_tree(FMRPatchSpec, FMRHierarchySpec)
    got = od.composite_wave_diagnostics(tuple(levels), tuple(coords), hierarchy, *scalars, active_fields=True)
    assert_close(got, expect["active"], 1e-13)
    plev, px = padded(hierarchy, levels, coords)
    got = od.composite_wave_diagnostics(tuple(plev), tuple(px), hierarchy, *scalars)
    assert_close(got, expect["guarded"], 1e-13)


def test_composite_known_answers():
    for case in (vertex_count_tree, branching_tree):
        hierarchy, fields, coords, answer = case(FMRPatchSpec, FMRHierarchySpec)
        got = od.composite_wave_diagnostics(fields, coords, hierarchy, 0.0, 1.0, 1.0, active_fields=True)
        assert_close(got, answer, 1e-14)
