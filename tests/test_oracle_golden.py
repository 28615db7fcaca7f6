"""The oracle against golden vectors produced by the reference itself.

The goldens come from running the unmodified reference source under a NumPy
jax stand-in (tests/golden/make_golden.py), which evaluates pow(det, -1/3)
correctly rounded.  The oracle restates the same arithmetic and agrees with
the goldens bit for bit.
"""

import numpy as np
import pytest

from oracle import bssn as ob
from oracle import stencils as st
from oracle.state import BSSNParameters, BSSNVariables

from .helpers import RHS_CASES, field_errors, golden_params, golden_state, load_golden, worst


@pytest.fixture(scope="module")
def stencil_data():
    return load_golden("stencils")


@pytest.mark.parametrize("case,lbc,rbc", [("periodic", 0, 0), ("sommerfeld", 1, 1), ("left", 1, 0), ("right", 0, 1)])
@pytest.mark.parametrize("q", [1.0, 1.0 / 16.0])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_stencils_bitwise(stencil_data, case, lbc, rbc, q, axis):
    f, c, dx = stencil_data["field"], stencil_data["coefficient"], float(stencil_data["dx"])
    key = f"{case}.q{q:g}.axis{axis}"
    np.testing.assert_array_equal(st.d1(f, axis, dx, lbc, rbc, q), stencil_data[f"d1.{key}"])
    np.testing.assert_array_equal(st.d2(f, axis, dx, lbc, rbc, q), stencil_data[f"d2.{key}"])
    np.testing.assert_array_equal(st.d1_upwind(f, c, axis, dx, lbc, rbc, q), stencil_data[f"up.{key}"])
    if q == 1.0:
        np.testing.assert_array_equal(st.d6(f, axis, dx, lbc, rbc), stencil_data[f"d6.{key}"])


@pytest.mark.parametrize("name", RHS_CASES)
def test_rhs_matches_reference(name):
    data = load_golden(f"rhs_{name}")
    state = golden_state(data, "input", BSSNVariables)
    params = golden_params(data, BSSNParameters)
    rhs = ob.compute_rhs(state, params)
    assert worst(field_errors(rhs, golden_state(data, "rhs", BSSNVariables))) == 0.0


@pytest.mark.parametrize("name", RHS_CASES)
def test_projection_and_rk4_match_reference(name):
    data = load_golden(f"rhs_{name}")
    state = golden_state(data, "input", BSSNVariables)
    params = golden_params(data, BSSNParameters)
    assert worst(field_errors(ob.project(state), golden_state(data, "project", BSSNVariables))) == 0.0
    one = ob.rk4_step(state, params)
    assert worst(field_errors(one, golden_state(data, "rk4_1", BSSNVariables))) == 0.0
    two = ob.rk4_step(one, params)
    assert worst(field_errors(two, golden_state(data, "rk4_2", BSSNVariables))) == 0.0


@pytest.mark.parametrize("name", RHS_CASES)
def test_constraints_match_reference(name):
    data = load_golden(f"rhs_{name}")
    state = golden_state(data, "input", BSSNVariables)
    params = golden_params(data, BSSNParameters)
    ours = ob.constraints(state, params)
    for value, field in zip(ours, ("hamiltonian", "momentum", "det_gamma", "trace_A", "gamma_condition")):
        ref = data[f"constraints.{field}"]
        scale = max(np.max(np.abs(ref)), 1e-300)
        assert np.max(np.abs(value - ref)) / scale < 1e-13, field


def near_one_lattice():
    """Determinants as the projection meets them: 1 + k ulp (both sides of one),
    plus a scatter of small perturbations and a wide range."""
    ks = np.arange(-400, 401)
    rng = np.random.default_rng(11)
    return np.concatenate([1 + ks * 2.0 ** -52, 1 + ks * 2.0 ** -53, 1 + 1e-9 * rng.normal(size=300),
                           1 + 2.0 ** -28 * (1 + rng.random(100)), 1 - 2.0 ** -28 * (1 + rng.random(100)),
                           1 + 1e-7 * rng.normal(size=300), 1 + 5e-7 * rng.normal(size=300),
                           1 + 1e-3 * rng.normal(size=300), np.exp(rng.normal(size=300))])


def exact_pow_minus_third(x):
    import decimal
    decimal.getcontext().prec = 90
    exponent = decimal.Decimal(-1.0 / 3.0)
    return np.array([float(decimal.Decimal(float(v)) ** exponent) for v in x])


def test_inv_cbrt_is_correctly_rounded():
    x = near_one_lattice()
    np.testing.assert_array_equal(ob.inv_cbrt(x), exact_pow_minus_third(x))


@pytest.mark.parametrize("name", ["run_gauge_wave32", "run_teukolsky24"])
def test_long_run_first_step_matches_reference(name):
    """The oracle's RK4 step reproduces the first step of the reference's long
    runs (gauge wave 32^3, Teukolsky 24^3 with Sommerfeld faces) bit for bit;
    the later steps of those runs are the GPU's long-horizon targets."""
    data = load_golden(name)
    state = golden_state(data, "input", BSSNVariables)
    params = golden_params(data, BSSNParameters)
    one = ob.rk4_step(state, params)
    assert worst(field_errors(one, golden_state(data, "rk4_1", BSSNVariables))) == 0.0


MATTER_CASES = ("generic_kappa", "sommerfeld", "mad_mixed")


def matter_of(data):
    return (data["matter.energy_density"], data["matter.momentum_density"], data["matter.spatial_stress"])


@pytest.mark.parametrize("name", MATTER_CASES)
def test_rhs_with_matter_matches_reference(name):
    """compute_bssn_rhs_with_matter (time_evolve.py:60-91): kappa damping with the
    matter momentum, Sommerfeld faces after the sources, MAD weights."""
    data = load_golden(f"matter_{name}")
    state = golden_state(data, "input", BSSNVariables)
    params = golden_params(data, BSSNParameters)
    rhs = ob.compute_rhs(state, params, matter_of(data))
    assert worst(field_errors(rhs, golden_state(data, "rhs", BSSNVariables))) == 0.0
