"""Compact z-axis axisymmetric Cartoon storage and support reconstruction
(mirrors JAX_BSSN/cartoon/axisymmetry/reconstruction.py).

The evolved state lives on the y = 0 half-plane, shape (Nrho+4, 1, Nz): four
negative-x parity ghosts, then positive half-cell radii.  Reconstruction onto
the nine Cartesian y planes and the ghost fill run in ``libbssn_gb300.so``
(``bssn_cartoon_reconstruct``, ``bssn_cartoon_fill_ghosts``); the projection and
expansion helpers here are layout moves on device tensors.
"""

from __future__ import annotations

import math

import torch

from ...bssn.variables import BSSNParameters, BSSNVariables
from .. import _calls
from ..interpolation import lagrange6_nonperiodic
from ..symmetry import SCALAR_PARITY, _back, _dev, field_parity, reflect_tensor

AXISYMMETRIC_GHOST_CELLS = 4
AXISYMMETRIC_SUPPORT_SIZE = 9
AXISYMMETRIC_CENTER = 4
AXISYMMETRIC_OUTER_BUFFER_CELLS = 3

VECTOR_RADIAL_REFLECTION_PARITY = (-1.0, -1.0, 1.0)

PERIODIC_BC = 0
SOMMERFELD_BC = 1


def _map(vars: BSSNVariables, transform) -> BSSNVariables:
    out, host = [], False
    for f in vars:
        t, h = _dev(f)
        host = host or h
        out.append(transform(t, field_parity(t, VECTOR_RADIAL_REFLECTION_PARITY)))
    return BSSNVariables(*(_back(t, host) for t in out))


def _compact_field(positive_plane, parity):
    return reflect_tensor(positive_plane, parity, axis=-2, count=AXISYMMETRIC_GHOST_CELLS).unsqueeze(-2)


def _expanded_field(positive_plane, parity):
    return reflect_tensor(positive_plane, parity, axis=-2).unsqueeze(-2)


def _reference_plane(field):
    return field[..., :, 0, :]


def _positive_plane(field):
    return _reference_plane(field)[..., AXISYMMETRIC_GHOST_CELLS:, :]


def validate_axisymmetric_grid(vars: BSSNVariables, params: BSSNParameters) -> None:
    """Compact storage, support geometry and face checks (reconstruction.py:65-112)."""
    nx, ny, nz = tuple(vars.conformal_factor.shape)
    spatial = (nx, ny, nz)
    if ny != 1:
        raise ValueError("axisymmetric Cartoon state requires a singleton y plane")
    if nx - AXISYMMETRIC_GHOST_CELLS < 6:
        raise ValueError("axisymmetric Cartoon mode requires at least six radial points")
    if nz < 9:
        raise ValueError("axisymmetric Cartoon mode requires at least nine z points")
    names = ("conformal_metric", "conformal_factor", "traceless_K", "trace_K", "conformal_connection", "lapse",
             "shift")
    leads = ((3, 3), (), (3, 3), (), (3,), (), (3,))
    for field, lead, name in zip(vars, leads, names):
        if tuple(field.shape) != lead + spatial:
            raise ValueError(f"{name} has shape {tuple(field.shape)}; expected {lead + spatial}")
    if params.xl_bc != PERIODIC_BC:
        raise ValueError("axisymmetric x-left is a parity ghost region")
    if params.xr_bc != SOMMERFELD_BC:
        raise ValueError("axisymmetric x-right must use the Sommerfeld boundary")
    if params.yl_bc != PERIODIC_BC or params.yr_bc != PERIODIC_BC:
        raise ValueError("axisymmetric reconstructed y faces must be periodic")
    if params.zl_bc not in (PERIODIC_BC, SOMMERFELD_BC) or params.zr_bc not in (PERIODIC_BC, SOMMERFELD_BC):
        raise ValueError("axisymmetric z faces must be periodic or Sommerfeld")
    if params.mad_q != 1:
        raise ValueError("axisymmetric Cartoon requires mad_q=1")
    dx = float(params.dx)
    if not math.isfinite(dx) or dx <= 0.0:
        raise ValueError("axisymmetric Cartoon requires finite dx > 0")
    # jnp.isclose defaults: |a - b| <= 1e-8 + 1e-5 |b|
    if not abs(float(params.x_min) + 3.5 * dx) <= 1e-8 + 1e-5 * abs(3.5 * dx):
        raise ValueError("axisymmetric Cartoon requires x_min=-3.5*dx")
    if not abs(float(params.y_min) + 4.0 * dx) <= 1e-8 + 1e-5 * abs(4.0 * dx):
        raise ValueError("axisymmetric Cartoon requires y_min=-4*dx")


def compact_axisymmetric_state(vars: BSSNVariables) -> BSSNVariables:
    """Compact a complete signed x-z plane into positive-rho storage (reconstruction.py:115-128)."""
    nx, ny, _ = tuple(vars.conformal_factor.shape)
    if ny != 1 or nx % 2:
        raise ValueError("input must be an even-length signed x plane with y=1")
    return _map(vars, lambda f, p: _compact_field(_reference_plane(f)[..., nx // 2:, :], p))


def fill_axisymmetric_ghosts(vars: BSSNVariables) -> BSSNVariables:
    """Rebuild the four negative-rho samples by rotation-by-pi parity (reconstruction.py:131-143)."""
    return _calls.fill_ghosts(vars, axi=True)


def _outer_buffer(reference: torch.Tensor, asymptotic, params) -> torch.Tensor:
    nx, nz = reference.shape[-2:]
    dx = torch.tensor(float(params.dx), dtype=torch.float64, device=reference.device)
    rho_edge = (nx - AXISYMMETRIC_GHOST_CELLS - 0.5) * dx
    z = float(params.z_min) + dx * torch.arange(nz, dtype=torch.float64, device=reference.device)
    rho_b = rho_edge + dx * torch.arange(1, AXISYMMETRIC_OUTER_BUFFER_CELLS + 1, dtype=torch.float64,
                                         device=reference.device)
    r_edge = torch.sqrt(rho_edge * rho_edge + z * z)
    r_b = torch.sqrt(rho_b[:, None] * rho_b[:, None] + z[None, :] * z[None, :])
    ratio = r_edge[None, :] / r_b
    a = torch.as_tensor(asymptotic, dtype=torch.float64, device=reference.device)
    a = a.reshape(tuple(a.shape) + (1, 1))
    lead = reference.ndim - 2
    buffer = a + (reference[..., -1:, :] - a) * ratio.reshape((1,) * lead + tuple(ratio.shape))
    return torch.cat((reference, buffer), dim=-2)


def radial_interpolate(positive_plane, rho, params: BSSNParameters, parity=SCALAR_PARITY, asymptotic_value=0.0):
    """Interpolate a positive-rho plane profile at arbitrary radii: parity
    reflection through the axis, 1/r continuation past the outer face
    (reconstruction.py:181-203)."""
    plane, host = _dev(positive_plane)
    r, _ = _dev(rho)
    plane = reflect_tensor(plane, parity, axis=-2, count=AXISYMMETRIC_GHOST_CELLS)
    source = _outer_buffer(plane, asymptotic_value, params)
    q = r / float(params.dx) + AXISYMMETRIC_GHOST_CELLS - 0.5
    return _back(lagrange6_nonperiodic(source, q, axis=-2), host)


def transformation_matrix(x, y):
    """Lambda^i_jbar: rotation by phi about z, identity on the axis (reconstruction.py:206-238)."""
    xt, host = _dev(x)
    yt, _ = _dev(y)
    xt, yt = torch.broadcast_tensors(xt, yt)
    rho = torch.sqrt(xt * xt + yt * yt)
    on_axis = rho <= 0.0
    safe = torch.where(on_axis, torch.ones_like(rho), rho)
    c = torch.where(on_axis, torch.ones_like(xt), xt / safe)
    s = torch.where(on_axis, torch.zeros_like(xt), yt / safe)
    zero, one = torch.zeros_like(xt), torch.ones_like(xt)
    m = torch.stack((torch.stack((c, s, zero)), torch.stack((-s, c, zero)), torch.stack((zero, zero, one))), dim=1)
    return _back(m, host)


def reconstruct_axisymmetric_support(vars: BSSNVariables, params: BSSNParameters) -> BSSNVariables:
    """The nine Cartesian y planes of the compact state, shape (Nrho+4, 9, Nz)
    (reconstruction.py:251-289), computed by ``bssn_cartoon_reconstruct``."""
    return _calls.reconstruct(vars, params, axi=True)


def _project_support_field(field, parity):
    return _compact_field(field[..., AXISYMMETRIC_GHOST_CELLS:, AXISYMMETRIC_CENTER, :], parity)


def project_axisymmetric_rhs(rhs: BSSNVariables) -> BSSNVariables:
    """Keep the positive-rho centre-plane values and rebuild ghosts (reconstruction.py:292-300)."""
    return _map(rhs, _project_support_field)


def project_axisymmetric_scalar(field):
    t, host = _dev(field)
    return _back(_project_support_field(t, SCALAR_PARITY), host)


def project_axisymmetric_vector(field):
    t, host = _dev(field)
    return _back(_project_support_field(t, torch.tensor(VECTOR_RADIAL_REFLECTION_PARITY, device=t.device)), host)


def expand_axisymmetric_plane(vars: BSSNVariables) -> BSSNVariables:
    """Mirror the positive radius onto the complete signed x-z plane (reconstruction.py:317-323)."""
    return _map(vars, lambda f, p: _expanded_field(_positive_plane(f), p))


def expand_axisymmetric_scalar(field):
    t, host = _dev(field)
    return _back(_expanded_field(_positive_plane(t), SCALAR_PARITY), host)


def expand_axisymmetric_vector(field):
    t, host = _dev(field)
    return _back(_expanded_field(_positive_plane(t), torch.tensor(VECTOR_RADIAL_REFLECTION_PARITY,
                                                                   device=t.device)), host)


__all__ = [
    "AXISYMMETRIC_CENTER", "AXISYMMETRIC_GHOST_CELLS", "AXISYMMETRIC_OUTER_BUFFER_CELLS",
    "AXISYMMETRIC_SUPPORT_SIZE", "VECTOR_RADIAL_REFLECTION_PARITY", "compact_axisymmetric_state",
    "expand_axisymmetric_plane", "expand_axisymmetric_scalar", "expand_axisymmetric_vector",
    "fill_axisymmetric_ghosts", "project_axisymmetric_rhs", "project_axisymmetric_scalar",
    "project_axisymmetric_vector", "radial_interpolate", "reconstruct_axisymmetric_support",
    "transformation_matrix", "validate_axisymmetric_grid",
]
