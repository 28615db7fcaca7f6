"""CUDA-graph replay of resident RK4 steps equals direct steps bit for bit.

``capture(n)`` records n steps without running them; replays run exactly the
captured kernels on the object's own buffers, so a replayed run and a direct
run of the same steps must agree in every bit, for both arithmetic forms.
"""

import math

import pytest
import torch

pytestmark = pytest.mark.gpu


def _bitwise_equal(a, b):
    for x, y in zip(a, b):
        assert torch.equal(x.view(torch.int64), y.view(torch.int64))


def _check(make, snapshot, steps=4, chunk=2):
    direct, graphed = make(), make()
    direct.step(steps)
    graphed.capture(chunk)
    assert graphed.captured and graphed.graph_launches > 0
    graphed.step(steps)
    torch.cuda.synchronize()
    _bitwise_equal(snapshot(direct), snapshot(graphed))
    # a step count the capture does not divide runs directly
    direct.step(1)
    graphed.step(1)
    torch.cuda.synchronize()
    _bitwise_equal(snapshot(direct), snapshot(graphed))
    graphed.release_graph()
    assert not graphed.captured


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_patch_evolution_graph(cuda, native, precision):
    from jax_bssn_gb300.evolution import PatchEvolution
    from jax_bssn_gb300.initial_data import teukolsky_config
    state, params = teukolsky_config(n=20)

    def snapshot(evo):
        return [evo.components().flatten()]
    _check(lambda: PatchEvolution(state, params, precision=precision), snapshot)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fmr_evolution_graph(cuda, native, precision):
    from jax_bssn_gb300.fmr import FMREvolution, initialize_tiled_fmr
    from jax_bssn_gb300.initial_data import fmr_linear_wave_hierarchy, fmr_linear_wave_root, linear_wave_callback
    hierarchy = fmr_linear_wave_hierarchy(32)
    root = fmr_linear_wave_root(32)
    states, parameters, layouts = initialize_tiled_fmr(linear_wave_callback(), root, (32,) * 3, hierarchy)
    assert sum(math.prod(l.active_shape) for l in layouts) > 0

    def snapshot(evo):
        return [leaf.flatten() for s in evo.states() for leaf in s]
    _check(lambda: FMREvolution(states, parameters, hierarchy, layouts, precision=precision), snapshot)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_axisymmetric_evolution_graph(cuda, native, precision):
    from jax_bssn_gb300.cartoon.axisymmetry import AxisymmetricEvolution
    from jax_bssn_gb300.initial_data import brill_lindquist_config
    state, params = brill_lindquist_config(num_radial_points=32, r_max=1.0)

    def snapshot(evo):
        return [evo.components().flatten()]
    _check(lambda: AxisymmetricEvolution(state, params, precision=precision), snapshot)


def _serial(lib, fn):
    """Run fn with per-kernel profiling on: every launch then goes to the
    caller's stream in order, with no auxiliary-stream branches."""
    lib.bssn_profile_reset()
    lib.bssn_profile_enable(1)
    try:
        return fn()
    finally:
        torch.cuda.synchronize()
        lib.bssn_profile_enable(0)
        lib.bssn_profile_reset()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_stream_branches_equal_serial_launches(cuda, native, precision):
    """The RHS kernels' auxiliary-stream branches and the FMR children's
    streams give the same bits as one in-order stream."""
    from jax_bssn_gb300.cartoon.axisymmetry import AxisymmetricEvolution
    from jax_bssn_gb300.evolution import PatchEvolution
    from jax_bssn_gb300.fmr import FMREvolution, initialize_tiled_fmr
    from jax_bssn_gb300.initial_data import (brill_lindquist_config, fmr_linear_wave_hierarchy,
                                             fmr_linear_wave_root, linear_wave_callback, teukolsky_config)
    state, params = teukolsky_config(n=20)
    hierarchy = fmr_linear_wave_hierarchy(32)
    states, parameters, layouts = initialize_tiled_fmr(linear_wave_callback(), fmr_linear_wave_root(32), (32,) * 3,
                                                       hierarchy)
    bl_state, bl_params = brill_lindquist_config(num_radial_points=32, r_max=1.0)
    cases = [
        (lambda: PatchEvolution(state, params, precision=precision), lambda e: [e.components().flatten()]),
        (lambda: FMREvolution(states, parameters, hierarchy, layouts, precision=precision),
         lambda e: [leaf.flatten() for s in e.states() for leaf in s]),
        (lambda: AxisymmetricEvolution(bl_state, bl_params, precision=precision), lambda e: [e.components().flatten()]),
    ]
    for make, snapshot in cases:
        branched, serial = make(), make()
        branched.step(3)
        _serial(native, lambda: serial.step(3))
        torch.cuda.synchronize()
        _bitwise_equal(snapshot(branched), snapshot(serial))
