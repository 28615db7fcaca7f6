"""The reference's lower triangles of At and gt through the reference-layout RK4.

The reference evolves all nine entries of both tensors, and its two orderings
of the mixed derivatives round differently on the rows next to a Sommerfeld
face, so its lower triangles drift from its upper ones by roundoff there
(JAX_BSSN/bssn/geometry.py:47-56, 131-135).  bssn_rk4_step carries those
differences to first order.  Here a 32^3 Teukolsky wave with Sommerfeld faces
runs three steps through rk4_steps (JAX_BSSN/evolution/time_evolve.py:144-217)
against the oracle's full-tensor RK4: each triangle of each tensor must agree
within 1e-13 of the leaf's largest value, while the lower triangle the oracle
evolves differs from its own upper one by far more than that.
"""

import numpy as np
import pytest

from oracle import bssn as ob
from oracle.state import BSSNParameters as OracleParams
from oracle.state import BSSNVariables as OracleVars

pytestmark = pytest.mark.gpu

PAIRS = ((0, 1), (0, 2), (1, 2))
TOL = 1e-13


def _host(a):
    return a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)


def test_lower_triangles_follow_the_reference(cuda, native):
    from jax_bssn_gb300.evolution import time_evolve as te
    from jax_bssn_gb300.initial_data import teukolsky_config
    state, params = teukolsky_config(n=32)
    oparams = OracleParams(**{k: getattr(params, k) for k in OracleParams._fields if hasattr(params, k)})
    ref = OracleVars(*(np.asarray(f) for f in state))
    steps = 3
    for _ in range(steps):
        ref = ob.rk4_step(ref, oparams)
    got = te.rk4_steps(state, params, steps)
    for leaf in ("traceless_K", "conformal_metric"):
        a = _host(getattr(got, leaf))
        r = np.asarray(getattr(ref, leaf))
        scale = float(np.max(np.abs(r)))
        upper = max(float(np.max(np.abs(a[i, j] - r[i, j]))) for i in range(3) for j in range(i, 3)) / scale
        lower = max(float(np.max(np.abs(a[j, i] - r[j, i]))) for i, j in PAIRS) / scale
        spread = max(float(np.max(np.abs(r[j, i] - r[i, j]))) for i, j in PAIRS) / scale
        print(leaf, f"upper {upper:.1e} lower {lower:.1e} (reference lower - upper {spread:.1e})")
        assert upper < TOL and lower < TOL, (leaf, upper, lower)
    At = np.asarray(ref.traceless_K)
    spread = max(float(np.max(np.abs(At[j, i] - At[i, j]))) for i, j in PAIRS) / float(np.max(np.abs(At)))
    assert spread > 5 * TOL, spread       # the reference's triangles do differ


def test_lower_triangles_with_mixed_faces_shift_and_damping(cuda, native):
    """A generic smooth state with every term active (shift, kappa != 0),
    Sommerfeld faces on x and z and a periodic y axis (the carried differences'
    periodic ghosts): three steps against the oracle's full-tensor RK4, every
    leaf within 1e-12 of its largest value."""
    import jax_bssn_gb300 as pkg
    from jax_bssn_gb300.evolution import time_evolve as te
    from jax_bssn_gb300.initial_data import random_smooth_state
    from .helpers import field_errors, worst
    state = random_smooth_state((14, 12, 16), seed=21)
    params = pkg.BSSNParameters(eta=1.5, kappa=0.05, nu=0.03, g=0.75, dx=0.07, dt=0.01, gauge=1,
                                xl_bc=1, xr_bc=1, zl_bc=1, zr_bc=1, x_min=-0.4, y_min=0.0, z_min=-0.5)
    ref = OracleVars(*(np.asarray(f) for f in state))
    for _ in range(3):
        ref = ob.rk4_step(ref, OracleParams(**params._asdict()))
    got = te.rk4_steps(state, params, 3)
    err = field_errors(got, ref)
    At = np.asarray(ref.traceless_K)
    spread = max(float(np.max(np.abs(At[j, i] - At[i, j]))) for i, j in PAIRS) / float(np.max(np.abs(At)))
    print("generic, 3 steps", {k: f"{v:.1e}" for k, v in err.items()}, f"(reference At lower - upper {spread:.1e})")
    assert worst(err) < 1e-12, err
