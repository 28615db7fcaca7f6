"""Constraints and output mappings of compact axisymmetric Cartoon states
(mirrors JAX_BSSN/cartoon/axisymmetry/diagnostics.py)."""

from __future__ import annotations

import torch

from ...bssn.constraints import ConstraintViolations
from ...bssn.variables import BSSNParameters, BSSNVariables
from .. import _calls
from ..symmetry import _dev
from .reconstruction import (AXISYMMETRIC_GHOST_CELLS, expand_axisymmetric_plane, expand_axisymmetric_scalar,
                             expand_axisymmetric_vector)


def compute_axisymmetric_constraints(vars: BSSNVariables, params: BSSNParameters) -> ConstraintViolations:
    """H, M_i, det-1, tr A and the connection constraint on the centre plane of
    the reconstructed support, compacted with parity ghosts (diagnostics.py:22-37)."""
    return _calls.constraints(vars, params, axi=True)


def compute_axisymmetric_constraint_norms(violations: ConstraintViolations, exclude_outer_rho: int = 4,
                                          exclude_z: int = 4, params: BSSNParameters | None = None) -> dict:
    """|rho|-weighted L2 (normalised by the weight sum and component count) and
    max-abs norms over the positive radii, dropping ``exclude_outer_rho`` outer
    radii and ``exclude_z`` samples at each z end (diagnostics.py:40-78)."""

    def physical(f):
        f = f[..., AXISYMMETRIC_GHOST_CELLS:, 0, :]
        if exclude_outer_rho:
            f = f[..., :-exclude_outer_rho, :]
        if exclude_z:
            f = f[..., exclude_z:-exclude_z]
        return f

    fields = [_dev(f)[0] for f in violations]
    H = fields[0]
    if params is not None:
        nx, nz = H.shape[0], H.shape[-1]
        rho = float(params.x_min) + float(params.dx) * torch.arange(nx, dtype=torch.float64, device=H.device)
        full = torch.abs(rho)[:, None].expand(nx, nz)
        coordinate_weight = physical(full[:, None, :])
    names = ("hamiltonian", "momentum", "det_gamma", "trace_A", "gamma")
    norms = {}
    for name, f in zip(names, fields):
        f = physical(f)
        nrho, nz = f.shape[-2:]
        if params is None:
            w = (torch.arange(nrho, dtype=torch.float64, device=f.device) + 0.5)[:, None].expand(nrho, nz)
        else:
            w = coordinate_weight
        comps = 1
        for size in f.shape[:-2]:
            comps *= size
        norms[name + "_l2"] = float(torch.sqrt(torch.sum(w * f * f) / (torch.sum(w) * comps)))
        norms[name + "_linf"] = float(torch.max(torch.abs(f)))
    return norms


def axisymmetric_plane_output_fields(vars: BSSNVariables, hamiltonian, momentum, det_gamma=None, trace_A=None,
                                     gamma_condition=None) -> dict:
    """The complete state and constraints on the signed x-z plane (diagnostics.py:81-124)."""
    full = expand_axisymmetric_plane(vars)
    full_m = expand_axisymmetric_vector(momentum)
    fields = {
        "W": full.conformal_factor,
        "K": full.trace_K,
        "lapse": full.lapse,
        "shift": tuple(full.shift[i] for i in range(3)),
        "conformal_connection": tuple(full.conformal_connection[i] for i in range(3)),
        "hamiltonian_constraint": expand_axisymmetric_scalar(hamiltonian),
        "momentum_constraint": tuple(full_m[i] for i in range(3)),
    }
    if det_gamma is not None:
        fields["det_gamma_constraint"] = expand_axisymmetric_scalar(det_gamma)
    if trace_A is not None:
        fields["trace_A_constraint"] = expand_axisymmetric_scalar(trace_A)
    if gamma_condition is not None:
        g = expand_axisymmetric_vector(gamma_condition)
        fields["gamma_constraint"] = tuple(g[i] for i in range(3))
    for name, tensor in (("conformal_metric", full.conformal_metric), ("traceless_K", full.traceless_K)):
        for suffix, (i, j) in (("xx", (0, 0)), ("xy", (0, 1)), ("xz", (0, 2)), ("yy", (1, 1)), ("yz", (1, 2)),
                               ("zz", (2, 2))):
            fields[f"{name}_{suffix}"] = tensor[i, j]
    return fields


__all__ = ["axisymmetric_plane_output_fields", "compute_axisymmetric_constraint_norms",
           "compute_axisymmetric_constraints"]
