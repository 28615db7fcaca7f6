"""Drop-in replacements for JAX_BSSN.evolution.time_evolve on GB300.

Same names, arguments and field order as the reference
(JAX_BSSN/evolution/time_evolve.py:41-217); the work runs in
``libbssn_gb300.so`` through its C ABI.  Invalid arguments raise ValueError
before any launch, as the reference's host-side validators do.
"""

from __future__ import annotations

import torch

from .. import _device, _native
from ..bssn.variables import BSSNParameters, BSSNVariables


def _finish(result, host):
    return _device.to_host(result) if host else result


def compute_bssn_rhs(vars: BSSNVariables, params: BSSNParameters) -> BSSNVariables:
    """Bulk BSSN RHS with active Sommerfeld faces (time_evolve.py:41-57)."""
    lib = _native.load()
    state, host = _device.device_state(vars)
    shape = _device.spatial_shape(state)
    p = _device.to_params(params)
    out = _device.empty_state(shape, state.lapse.device)
    nbytes = lib.bssn_workspace_bytes(_native.OP_RHS, _device.shape3(shape), p)
    ws = _device.workspace(nbytes, state.lapse.device)
    fin, fout = _device.fields_struct(state), _device.fields_struct(out)
    _native.check(lib.bssn_rhs(fin, fout, _device.shape3(shape), p, None, ws.data_ptr(), ws.numel(),
                               _device.stream_handle()), "compute_bssn_rhs")
    return _finish(out, host)


def compute_bssn_rhs_with_matter(vars, params, energy_density, momentum_density, spatial_stress):
    """Matter-coupled RHS (time_evolve.py:60-91): not provided by this build."""
    raise NotImplementedError("matter-coupled BSSN RHS is not provided by the GB300 kernels yet")


def enforce_algebraic_constraints(vars: BSSNVariables) -> BSSNVariables:
    """det(gamma_tilde) = 1 and trace-free A_tilde (time_evolve.py:134-141)."""
    lib = _native.load()
    state, host = _device.device_state(vars)
    out = BSSNVariables(*(leaf.clone() for leaf in state))
    shape = _device.spatial_shape(out)
    _native.check(lib.bssn_project(_device.fields_struct(out), _device.shape3(shape),
                                   _device.stream_handle()), "enforce_algebraic_constraints")
    return _finish(out, host)


def rk4_step(vars: BSSNVariables, params: BSSNParameters) -> BSSNVariables:
    """One classical RK4 step with projection at every stage (time_evolve.py:144-217)."""
    return rk4_steps(vars, params, 1)


def rk4_steps(vars: BSSNVariables, params: BSSNParameters, steps: int) -> BSSNVariables:
    """``steps`` consecutive rk4_step calls fused into one device-side loop."""
    lib = _native.load()
    state, host = _device.device_state(vars)
    out = BSSNVariables(*(leaf.clone() for leaf in state))
    shape = _device.spatial_shape(out)
    p = _device.to_params(params)
    nbytes = lib.bssn_workspace_bytes(_native.OP_RK4, _device.shape3(shape), p)
    ws = _device.workspace(nbytes, out.lapse.device)
    _native.check(lib.bssn_rk4_step(_device.fields_struct(out), _device.shape3(shape), p, int(steps),
                                    ws.data_ptr(), ws.numel(), _device.stream_handle()), "rk4_step")
    return _finish(out, host)


__all__ = ["compute_bssn_rhs", "compute_bssn_rhs_with_matter", "enforce_algebraic_constraints",
           "rk4_step", "rk4_steps"]
