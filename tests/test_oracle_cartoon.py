"""The Cartoon oracle against the reference (goldens from the reference run)."""

import json

import numpy as np
import pytest

from oracle import cartoon as oc
from oracle.state import BSSNParameters, BSSNVariables

from .helpers import field_errors, golden_params, golden_state, load_golden, worst


@pytest.fixture(scope="module")
def axi():
    data = load_golden("cartoon_axisymmetric")
    return data, golden_state(data, "input", BSSNVariables), golden_params(data, BSSNParameters)


@pytest.fixture(scope="module")
def sph():
    data = load_golden("cartoon_spherical")
    return data, golden_state(data, "input", BSSNVariables), golden_params(data, BSSNParameters)


def test_axisymmetric_support_rhs_and_steps(axi):
    data, state, params = axi
    assert worst(field_errors(oc.axi_reconstruct(state, params), golden_state(data, "support", BSSNVariables))) == 0.0
    assert worst(field_errors(oc.axi_rhs(state, params), golden_state(data, "rhs", BSSNVariables))) == 0.0
    one = oc.axi_rk4_step(state, params)
    assert worst(field_errors(one, golden_state(data, "rk4_1", BSSNVariables))) == 0.0
    two = oc.axi_rk4_step(one, params)
    assert worst(field_errors(two, golden_state(data, "rk4_2", BSSNVariables))) == 0.0


def test_axisymmetric_constraints_and_norms(axi):
    data, state, params = axi
    one = oc.axi_rk4_step(state, params)
    ours = oc.axi_constraints(one, params)
    for value, field in zip(ours, ("hamiltonian", "momentum", "det_gamma", "trace_A", "gamma_condition")):
        np.testing.assert_array_equal(value, data[f"constraints.{field}"])
    norms = oc.axi_constraint_norms(ours, p=params)
    ref = json.loads(str(data["norms"]))
    for key, value in ref.items():
        # the constraint fields are bit-exact; the norms differ only by summation order
        assert norms[key] == pytest.approx(value, rel=1e-14, abs=1e-300), key


def test_spherical_support_rhs_and_steps(sph):
    data, state, params = sph
    assert worst(field_errors(oc.sph_reconstruct(state, params), golden_state(data, "support", BSSNVariables))) == 0.0
    assert worst(field_errors(oc.sph_rhs(state, params), golden_state(data, "rhs", BSSNVariables))) == 0.0
    one = oc.sph_rk4_step(state, params)
    assert worst(field_errors(one, golden_state(data, "rk4_1", BSSNVariables))) == 0.0
    two = oc.sph_rk4_step(one, params)
    assert worst(field_errors(two, golden_state(data, "rk4_2", BSSNVariables))) == 0.0


def test_spherical_constraints_norms_and_symmetry_norms(sph):
    data, state, params = sph
    if "constraints.hamiltonian" not in data:
        pytest.skip("fixture predates the spherical constraint vectors")
    one = oc.sph_rk4_step(state, params)
    ours = oc.sph_constraints(one, params)
    for value, field in zip(ours, ("hamiltonian", "momentum", "det_gamma", "trace_A", "gamma_condition")):
        np.testing.assert_array_equal(value, data[f"constraints.{field}"])
    norms = oc.sph_constraint_norms(ours)
    ref = json.loads(str(data["norms"]))
    for key, value in ref.items():
        assert norms[key] == pytest.approx(value, rel=1e-14, abs=1e-300), key
    sym = oc.sph_symmetry_norms(oc.sph_rhs(state, params))
    ref = json.loads(str(data["symmetry_norms"]))
    for key, value in ref.items():
        assert sym[key] == pytest.approx(value, rel=1e-14, abs=1e-300), key
