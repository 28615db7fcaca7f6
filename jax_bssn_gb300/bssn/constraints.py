"""Constraint fields on GB300 (mirrors JAX_BSSN/bssn/constraints.py:262-412).

``compute_all_constraints`` returns the reference's ``ConstraintViolations``
tuple: Hamiltonian H, momentum M_i, det(gamma_tilde) - 1, trace of A_tilde and
the conformal-connection constraint, evaluated by one kernel pass.
"""

from __future__ import annotations

from typing import NamedTuple

import torch

from .. import _device, _native
from .variables import BSSNParameters, BSSNVariables


class ConstraintViolations(NamedTuple):
    hamiltonian: object
    momentum: object
    det_gamma: object
    trace_A: object
    gamma_condition: object


def compute_all_constraints(vars: BSSNVariables, params: BSSNParameters) -> ConstraintViolations:
    lib = _native.load()
    state, host = _device.device_state(vars)
    shape = _device.spatial_shape(state)
    dev = state.lapse.device
    p = _device.to_params(params)
    H = torch.empty(shape, dtype=torch.float64, device=dev)
    M = torch.empty((3,) + shape, dtype=torch.float64, device=dev)
    det = torch.empty(shape, dtype=torch.float64, device=dev)
    trA = torch.empty(shape, dtype=torch.float64, device=dev)
    gam = torch.empty((3,) + shape, dtype=torch.float64, device=dev)
    nbytes = lib.bssn_workspace_bytes(_native.OP_CONSTRAINTS, _device.shape3(shape), p)
    ws = _device.workspace(nbytes, dev)
    _native.check(lib.bssn_constraints(_device.fields_struct(state), _device.shape3(shape), p,
                                       H.data_ptr(), M.data_ptr(), det.data_ptr(), trA.data_ptr(),
                                       gam.data_ptr(), ws.data_ptr(), ws.numel(), _device.stream_handle()),
                  "compute_all_constraints")
    out = ConstraintViolations(H, M, det, trA, gam)
    if host:
        out = ConstraintViolations(*(t.cpu().numpy() for t in out))
    return out


def compute_hamiltonian_constraint(vars, params):
    return compute_all_constraints(vars, params).hamiltonian


def compute_momentum_constraint(vars, params):
    return compute_all_constraints(vars, params).momentum


def compute_constraint_norms(violations: ConstraintViolations) -> dict:
    """RMS and max-abs per constraint (JAX_BSSN/diagnostics/constraints.py:9-36)."""
    names = ("hamiltonian", "momentum", "det_gamma", "trace_A", "gamma")
    norms = {}
    for name, field in zip(names, violations):
        t = field if isinstance(field, torch.Tensor) else torch.as_tensor(field)
        norms[name + "_l2"] = float(torch.sqrt(torch.mean(t * t)))
        norms[name + "_linf"] = float(torch.max(torch.abs(t)))
    return norms
