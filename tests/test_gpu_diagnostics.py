"""CUDA wave diagnostics against goldens from the reference
(diagnostics/waves.py:11-91) and the reference suite's known answers."""

import numpy as np
import pytest

from .helpers import golden_params, golden_state, load_golden
from .wave_cases import assert_close, branching_tree, golden_tree, padded, vertex_count_tree

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def waves(cuda, native):
    import jax_bssn_gb300 as pkg
    from jax_bssn_gb300.diagnostics import waves
    from jax_bssn_gb300.fmr import FMRHierarchySpec, FMRPatchSpec
    return pkg, waves, FMRPatchSpec, FMRHierarchySpec


def test_h_plus_bitwise(waves):
    pkg, w, _, _ = waves
    data = load_golden("waves")
    state = golden_state(data, "input", pkg.BSSNVariables)
    got = np.asarray(w.h_plus(state))
    assert np.array_equal(got.view(np.int64), data["h_plus"].view(np.int64))


def test_diagnostic_fields_constraints(waves):
    pkg, w, _, _ = waves
    data = load_golden("waves")
    state = golden_state(data, "input", pkg.BSSNVariables)
    fields = w.diagnostic_fields(state, golden_params(data, pkg.BSSNParameters))
    for got, ref in ((fields["hamiltonian_constraint"], data["hamiltonian"]),
                     (np.stack(fields["momentum_constraint"]), data["momentum"])):
        err = np.max(np.abs(np.asarray(got) - ref)) / np.max(np.abs(ref))
        assert err < 1e-11, err
    assert np.array_equal(np.asarray(fields["W"]), data["input.conformal_factor"])


def test_composite_norms(waves):
    _, w, spec, hier = waves
    hierarchy, levels, coords, scalars, expect = golden_tree(spec, hier)
    got = w.composite_wave_diagnostics(tuple(levels), tuple(coords), hierarchy, *scalars, active_fields=True)
    assert_close(got, expect["active"], 1e-12)
    plev, px = padded(hierarchy, levels, coords)
    got = w.composite_wave_diagnostics(tuple(plev), tuple(px), hierarchy, *scalars)
    assert_close(got, expect["guarded"], 1e-12)


def test_composite_known_answers(waves):
    _, w, spec, hier = waves
    for case in (vertex_count_tree, branching_tree):
        hierarchy, fields, coords, answer = case(spec, hier)
        got = w.composite_wave_diagnostics(fields, coords, hierarchy, 0.0, 1.0, 1.0, active_fields=True)
        assert_close(got, answer, 1e-14)
