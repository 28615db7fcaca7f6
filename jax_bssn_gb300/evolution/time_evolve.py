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


def _rhs(vars, params, sources, what):
    lib = _native.load()
    state, host = _device.device_state(vars)
    shape = _device.spatial_shape(state)
    device = state.lapse.device
    p = _device.to_params(params)
    out = _device.empty_state(shape, device)
    matter = None
    op = _native.OP_RHS
    if sources is not None:
        leads = ((), (3,), (3, 3))
        names = ("energy_density", "momentum_density", "spatial_stress")
        tensors = []
        for value, lead, name in zip(sources, leads, names):
            if value is None:
                raise ValueError(f"{name} is required for the matter-coupled RHS")
            tensors.append(_device.as_device(value, lead + shape, device, name))
        matter = _native.BssnMatter(*(t.data_ptr() for t in tensors))
        op = _native.OP_RHS_MATTER
    nbytes = lib.bssn_workspace_bytes(op, _device.shape3(shape), p)
    ws = _device.workspace(nbytes, device)
    fin, fout = _device.fields_struct(state), _device.fields_struct(out)
    _native.check(lib.bssn_rhs(fin, fout, _device.shape3(shape), p, matter, ws.data_ptr(), ws.numel(),
                               _device.stream_handle()), what)
    return _finish(out, host)


def compute_bssn_rhs(vars: BSSNVariables, params: BSSNParameters) -> BSSNVariables:
    """Bulk BSSN RHS with active Sommerfeld faces (time_evolve.py:41-57)."""
    return _rhs(vars, params, None, "compute_bssn_rhs")


def compute_bssn_rhs_with_matter(vars: BSSNVariables, params: BSSNParameters, energy_density, momentum_density,
                                 spatial_stress) -> BSSNVariables:
    """BSSN RHS with Eulerian matter sources (time_evolve.py:60-91).

    Layouts ``rho[nx, ny, nz]``, ``S_i[3, nx, ny, nz]``, ``S_ij[3, 3, nx, ny, nz]``
    (read from its upper triangle: a symmetric stress).  Sources enter the
    bulk equations -- +4 pi alpha (rho + S) in dt K, -8 pi alpha W^2 S_ij inside
    the trace-free part of dt At, -16 pi alpha gt^ij S_j in dt Gt^i and, with
    kappa != 0, the matter momentum in the damping term -- before the active
    Sommerfeld faces are imposed."""
    return _rhs(vars, params, (energy_density, momentum_density, spatial_stress), "compute_bssn_rhs_with_matter")


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
