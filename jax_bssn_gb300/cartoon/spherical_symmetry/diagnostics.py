"""Constraints and output mappings of compact spherical Cartoon states
(mirrors JAX_BSSN/cartoon/spherical_symmetry/diagnostics.py)."""

from __future__ import annotations

import torch

from ...bssn.constraints import ConstraintViolations
from ...bssn.variables import BSSNParameters, BSSNVariables
from .. import _calls
from ..symmetry import _dev
from .reconstruction import cartoon_positive_radius, expand_cartoon_axis, expand_cartoon_scalar, expand_cartoon_vector


def compute_cartoon_constraints(vars: BSSNVariables, params: BSSNParameters) -> ConstraintViolations:
    """Constraints on the centre line of the support, compacted with parity
    ghosts (diagnostics.py:21-37)."""
    return _calls.constraints(vars, params, axi=False)


def _radius_norms(fields: dict, exclude_outer: int) -> dict:
    norms = {}
    for name, f in fields.items():
        f = cartoon_positive_radius(_dev(f)[0])
        if exclude_outer:
            f = f[..., :-exclude_outer]
        norms[f"{name}_l2"] = float(torch.sqrt(torch.mean(f * f)))
        norms[f"{name}_linf"] = float(torch.max(torch.abs(f)))
    return norms


def compute_cartoon_constraint_norms(violations: ConstraintViolations, exclude_outer: int = 4) -> dict:
    """RMS and max-abs over the positive radii away from the outer edge (diagnostics.py:40-65)."""
    names = ("hamiltonian", "momentum", "det_gamma", "trace_A", "gamma")
    return _radius_norms(dict(zip(names, violations)), exclude_outer)


def compute_spherical_symmetry_norms(vars: BSSNVariables, exclude_outer: int = 0) -> dict:
    """Norms of the reference-axis components spherical symmetry forbids (diagnostics.py:68-111)."""
    g = _dev(vars.conformal_metric)[0]
    A = _dev(vars.traceless_K)[0]
    beta = _dev(vars.shift)[0]
    gam = _dev(vars.conformal_connection)[0]
    errors = {
        "metric_tangential": g[1, 1] - g[2, 2],
        "A_tangential": A[1, 1] - A[2, 2],
        "metric_xy": g[0, 1], "metric_xz": g[0, 2], "metric_yz": g[1, 2],
        "A_xy": A[0, 1], "A_xz": A[0, 2], "A_yz": A[1, 2],
        "shift_y": beta[1], "shift_z": beta[2],
        "connection_y": gam[1], "connection_z": gam[2],
    }
    return _radius_norms(errors, exclude_outer)


def cartoon_axis_output_fields(vars: BSSNVariables, hamiltonian, momentum, det_gamma=None, trace_A=None,
                               gamma_condition=None) -> dict:
    """The complete state and constraints on the signed x axis (diagnostics.py:114-165)."""
    full = expand_cartoon_axis(vars)
    full_m = expand_cartoon_vector(momentum)
    fields = {
        "W": full.conformal_factor,
        "K": full.trace_K,
        "lapse": full.lapse,
        "shift": tuple(full.shift[i] for i in range(3)),
        "conformal_connection": tuple(full.conformal_connection[i] for i in range(3)),
        "hamiltonian_constraint": expand_cartoon_scalar(hamiltonian),
        "momentum_constraint": tuple(full_m[i] for i in range(3)),
    }
    if det_gamma is not None:
        fields["det_gamma_constraint"] = expand_cartoon_scalar(det_gamma)
    if trace_A is not None:
        fields["trace_A_constraint"] = expand_cartoon_scalar(trace_A)
    if gamma_condition is not None:
        g = expand_cartoon_vector(gamma_condition)
        fields["gamma_constraint"] = tuple(g[i] for i in range(3))
    for name, tensor in (("conformal_metric", full.conformal_metric), ("traceless_K", full.traceless_K)):
        for suffix, (i, j) in (("xx", (0, 0)), ("xy", (0, 1)), ("xz", (0, 2)), ("yy", (1, 1)), ("yz", (1, 2)),
                               ("zz", (2, 2))):
            fields[f"{name}_{suffix}"] = tensor[i, j]
    return fields


__all__ = ["cartoon_axis_output_fields", "compute_cartoon_constraint_norms", "compute_cartoon_constraints",
           "compute_spherical_symmetry_norms"]
