"""Matter-coupled RHS on the GPU (compute_bssn_rhs_with_matter,
JAX_BSSN/evolution/time_evolve.py:60-91) against the reference's goldens."""

import numpy as np
import pytest

from oracle.state import BSSNVariables as OracleVars

from .helpers import field_errors, golden_params, golden_state, load_golden, worst

pytestmark = pytest.mark.gpu

CASES = ("generic_kappa", "sommerfeld", "mad_mixed")
RHS_TOL = 1e-11


@pytest.fixture(scope="module")
def te(cuda, native):
    import jax_bssn_gb300 as pkg
    from jax_bssn_gb300.evolution import time_evolve
    return pkg, time_evolve


def _inputs(data, pkg):
    sources = (data["matter.energy_density"], data["matter.momentum_density"], data["matter.spatial_stress"])
    return golden_state(data, "input", pkg.BSSNVariables), golden_params(data, pkg.BSSNParameters), sources


@pytest.mark.parametrize("name", CASES)
def test_rhs_with_matter_matches_reference(te, name):
    pkg, t = te
    data = load_golden(f"matter_{name}")
    state, params, sources = _inputs(data, pkg)
    rhs = t.compute_bssn_rhs_with_matter(state, params, *sources)
    err = field_errors(rhs, golden_state(data, "rhs", OracleVars))
    print(name, "matter rhs", {k: f"{v:.1e}" for k, v in err.items()})
    assert worst(err) < RHS_TOL
    # the sources change the K, At and Gt equations (and nothing else)
    vacuum = t.compute_bssn_rhs(state, params)
    for leaf, a, b in zip(OracleVars._fields, rhs, vacuum):
        changed = not np.array_equal(np.asarray(a), np.asarray(b))
        assert changed == (leaf in ("traceless_K", "trace_K", "conformal_connection")), leaf


@pytest.mark.parametrize("name", CASES)
def test_rhs_with_matter_fp32_form(te, name):
    pkg, t = te
    data = load_golden(f"matter_{name}")
    state, params, sources = _inputs(data, pkg)
    with pkg.arithmetic("fp32"):
        rhs = t.compute_bssn_rhs_with_matter(state, params, *sources)
    ref = golden_state(data, "rhs", OracleVars)
    for leaf, a, b in zip(OracleVars._fields, rhs, ref):
        scale = max(float(np.max(np.abs(b))), 1e-300)
        err = float(np.max(np.abs(np.asarray(a) - b))) / scale
        assert err < 2e-4, (name, leaf, err)


def test_rhs_with_matter_needs_every_source(te):
    pkg, t = te
    data = load_golden("matter_generic_kappa")
    state, params, sources = _inputs(data, pkg)
    with pytest.raises(ValueError):
        t.compute_bssn_rhs_with_matter(state, params, sources[0], None, sources[2])
    with pytest.raises(ValueError):
        t.compute_bssn_rhs_with_matter(state, params, sources[0], sources[1], sources[2][0])
