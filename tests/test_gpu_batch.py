"""Instance batches: many independent states of one grid in the same launches.

A batch is the reference's rk4_step (JAX_BSSN/evolution/time_evolve.py:144-217)
applied to each instance; the batched launches must reproduce separate
single-instance runs bit for bit, in both arithmetic forms, on periodic and
Sommerfeld grids, directly and from a captured CUDA graph.
"""

import pytest

from .helpers import field_errors, worst

pytestmark = pytest.mark.gpu


def _cases():
    from jax_bssn_gb300 import BSSNParameters
    from jax_bssn_gb300.initial_data import gauge_wave_config, random_smooth_state, teukolsky_config
    periodic = BSSNParameters(eta=1.0, kappa=0.0, nu=0.05, g=0.75, dx=0.07, dt=0.012, gauge=1, mad_q=1.0 / 16.0)
    damped = periodic._replace(kappa=0.05, xl_bc=1, xr_bc=1, zl_bc=1, zr_bc=1, x_min=-0.5, z_min=-0.6, mad_q=1.0)
    teuk_state, teuk_params = teukolsky_config(n=20)
    gw_state, gw_params = gauge_wave_config(n=16)
    return [
        ("periodic_mad", [random_smooth_state((14, 12, 16), seed=s) for s in range(3)], periodic),
        ("sommerfeld_kappa", [random_smooth_state((12, 14, 12), seed=10 + s) for s in range(2)], damped),
        ("teukolsky20", [teuk_state, random_smooth_state((20, 20, 20), seed=5, amplitude=1e-3)], teuk_params),
        ("gauge_wave16", [gw_state] * 4, gw_params),
    ]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_equals_separate_runs_bitwise(cuda, native, precision):
    from jax_bssn_gb300.evolution import BatchEvolution, PatchEvolution
    for name, states, params in _cases():
        batch = BatchEvolution(states, params, precision=precision)
        batch.step(3)
        assert batch.nonfinite_count() == 0
        for i, state in enumerate(states):
            single = PatchEvolution(state, params, precision=precision)
            single.step(3)
            err = field_errors(batch.state(i), single.state())
            assert worst(err) == 0.0, (name, precision, i, err)


def test_batch_graph_replay_is_bitwise(cuda, native):
    from jax_bssn_gb300 import BSSNParameters
    from jax_bssn_gb300.evolution import BatchEvolution
    from jax_bssn_gb300.initial_data import random_smooth_state
    params = BSSNParameters(eta=2.0, nu=0.02, g=0.75, dx=0.08, dt=0.01, gauge=1, yl_bc=1, yr_bc=1, y_min=-0.5)
    states = [random_smooth_state((12, 12, 12), seed=40 + s) for s in range(5)]
    direct = BatchEvolution(states, params)
    direct.step(4)
    graphed = BatchEvolution(states, params)
    graphed.capture(2)
    graphed.step(4)
    for i in range(len(states)):
        assert worst(field_errors(graphed.state(i), direct.state(i))) == 0.0, i


def test_batch_rejects_mismatched_instances(cuda, native):
    from jax_bssn_gb300 import BSSNParameters
    from jax_bssn_gb300.evolution import BatchEvolution
    from jax_bssn_gb300.initial_data import random_smooth_state
    with pytest.raises(ValueError, match="same grid shape"):
        BatchEvolution([random_smooth_state((10, 10, 10)), random_smooth_state((10, 10, 12))],
                       BSSNParameters(dx=0.1, dt=0.01))


def test_monitored_run_reports_non_finite_values(cuda, native):
    """Failure detection: a NaN planted in one instance's host-prepared input
    stops the monitored run before the first step with BSSN_ERR_NONFINITE; an
    overflow planted in K turns non-finite during the run and is caught at the
    next check; a finite batch runs through and equals the unmonitored run."""
    import numpy as np
    from jax_bssn_gb300.evolution import BatchEvolution, NonFiniteStateError
    from jax_bssn_gb300.initial_data import gauge_wave_config
    state, params = gauge_wave_config(n=12)
    clean = BatchEvolution([state, state], params)
    assert clean.step_monitored(6, check_every=2) == 6
    plain = BatchEvolution([state, state], params)
    plain.step(6)
    for i in range(2):
        assert worst(field_errors(clean.state(i), plain.state(i))) == 0.0
    bad = state._replace(lapse=np.array(state.lapse, copy=True))
    bad.lapse[3, 4, 5] = np.nan
    evo = BatchEvolution([state, bad], params)
    with pytest.raises(NonFiniteStateError, match="before step 1") as info:
        evo.step_monitored(4, check_every=1)
    assert info.value.steps_done == 0
    hot = state._replace(trace_K=np.array(state.trace_K, copy=True))
    hot.trace_K[6, 6, 6] = 1.0e200          # finite, but K^2 overflows in the first RHS
    evo = BatchEvolution([hot, state], params)
    with pytest.raises(NonFiniteStateError, match="after step") as info:
        evo.step_monitored(6, check_every=2)
    assert info.value.steps_done == 2


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_autotuned_launch_shapes_leave_results_unchanged(cuda, native, precision):
    """bssn_tune_patch times each RHS launch slot with 32, 64 and 128 threads
    per block and keeps the fastest (margin 10: whatever the heuristic's time,
    so the tuned table is exercised); later launches (direct and captured) use
    it.  Every thread still computes the same point, so the evolution is
    bit-identical to the heuristic launch shapes, for single patches, batches
    and FMR patches."""
    from jax_bssn_gb300.evolution import BatchEvolution, PatchEvolution
    from jax_bssn_gb300.fmr import FMREvolution, initialize_tiled_fmr
    from jax_bssn_gb300.initial_data import (fmr_linear_wave_hierarchy, fmr_linear_wave_root, linear_wave_callback,
                                             teukolsky_config)
    state, params = teukolsky_config(n=22)
    before = PatchEvolution(state, params, precision=precision)
    before.step(2)
    batch_before = BatchEvolution([state, state], params, precision=precision)
    batch_before.step(2)
    hierarchy = fmr_linear_wave_hierarchy(24)
    states, parameters, layouts = initialize_tiled_fmr(linear_wave_callback(), fmr_linear_wave_root(24), (24,) * 3,
                                                       hierarchy)
    fmr_before = FMREvolution(states, parameters, hierarchy, layouts, precision=precision)
    fmr_before.step(2)

    tuned = PatchEvolution(state, params, precision=precision)
    assert "threads" in tuned.tune(margin=10.0)
    tuned.step(2)
    assert worst(field_errors(tuned.state(), before.state())) == 0.0
    batch = BatchEvolution([state, state], params, precision=precision)
    batch.tune(margin=10.0)
    batch.capture(1)
    batch.step(2)
    for i in range(2):
        assert worst(field_errors(batch.state(i), batch_before.state(i))) == 0.0
    fmr = FMREvolution(states, parameters, hierarchy, layouts, precision=precision)
    fmr.tune(margin=10.0)
    fmr.step(2)
    for a, b in zip(fmr.states(), fmr_before.states()):
        assert worst(field_errors(a, b)) == 0.0
