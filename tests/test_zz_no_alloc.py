"""bssn_rhs_noalloc: the RHS entry point for callers that cannot allocate.

Some callers cannot call cudaMalloc (a host framework that owns all device
memory, a solver whose memory budget is fixed at start-up).  For them the
library offers bssn_rhs_noalloc, which works in an array built into the
library instead of a caller-provided workspace.  These tests call it through
the C ABI twice in a row -- on different states, with and without the
constraint-damping branch that uses the larger part of the array -- and check
each result against the ordinary bssn_rhs entry point.  This file is named so
that pytest collects it last.
"""

import ctypes

import numpy as np
import pytest
import torch

from .helpers import field_errors, worst

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-11  # the RHS tolerance of the other parity tests


def _call_noalloc(native, state, params):
    from jax_bssn_gb300 import _device
    dev_state, _ = _device.device_state(state)
    shape = _device.spatial_shape(dev_state)
    out = _device.empty_state(shape, dev_state.lapse.device)
    status = native.bssn_rhs_noalloc(ctypes.byref(_device.fields_struct(dev_state)),
                                     ctypes.byref(_device.fields_struct(out)), _device.shape3(shape),
                                     ctypes.byref(_device.to_params(params)), _device.stream_handle())
    torch.cuda.synchronize()
    return status, out


def test_noalloc_matches_workspace_entry_point_on_two_calls(cuda, native):
    from jax_bssn_gb300 import BSSNParameters
    from jax_bssn_gb300.evolution.time_evolve import compute_bssn_rhs
    from jax_bssn_gb300.initial_data import random_smooth_state

    cases = [
        (random_smooth_state((16, 14, 18), seed=31),
         BSSNParameters(eta=1.5, kappa=0.2, nu=0.03, g=0.75, dx=0.07, dt=0.01, gauge=1,
                        xl_bc=1, xr_bc=1, x_min=-0.5, y_min=0.1, z_min=-0.6)),
        (random_smooth_state((20, 20, 20), seed=32),
         BSSNParameters(eta=2.0, kappa=0.0, nu=0.05, g=0.75, dx=0.05, dt=0.01, gauge=0, mad_q=1.0 / 16.0)),
        # the largest array served, with the damping branch: all 153 blocks
        (random_smooth_state((20, 20, 20), seed=33),
         BSSNParameters(eta=1.0, kappa=0.1, nu=0.04, g=0.75, dx=0.06, dt=0.01, gauge=1,
                        zl_bc=1, zr_bc=1, x_min=-0.6, y_min=-0.6, z_min=-0.6)),
    ]
    for state, params in cases:
        status, got = _call_noalloc(native, state, params)
        assert status == 0, native.bssn_last_error()
        expect = compute_bssn_rhs(state, params)
        err = field_errors(got, expect)
        assert worst(err) < RHS_TOL, err


def test_noalloc_rejects_arrays_beyond_its_limit(cuda, native):
    from jax_bssn_gb300 import BSSNParameters
    from jax_bssn_gb300.initial_data import random_smooth_state
    state = random_smooth_state((21, 20, 20), seed=1)
    status, _ = _call_noalloc(native, state, BSSNParameters(dx=0.05))
    assert status == 1
    assert b"too large" in native.bssn_last_error()
