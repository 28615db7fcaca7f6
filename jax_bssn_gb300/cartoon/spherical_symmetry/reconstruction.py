"""Compact spherical Cartoon storage and support reconstruction
(mirrors JAX_BSSN/cartoon/spherical_symmetry/reconstruction.py).

The evolved state is the x axis, shape (Nr+4, 1, 1): four parity ghosts, then
positive half-cell radii.  The symmetric-subspace projection and the 9 x 9
support reconstruction run in ``libbssn_gb300.so`` (``bssn_cartoon_fill_ghosts``
and ``bssn_cartoon_reconstruct`` with axisymmetric = 0); the projection and
expansion helpers here are layout moves on device tensors.
"""

from __future__ import annotations

import math

import torch

from ...bssn.variables import BSSNParameters, BSSNVariables
from .. import _calls
from ..interpolation import lagrange6_nonperiodic
from ..symmetry import SCALAR_PARITY, _back, _dev, field_parity, reflect_tensor

CARTOON_GHOST_CELLS = 4
CARTOON_SUPPORT_SIZE = 2 * CARTOON_GHOST_CELLS + 1
CARTOON_CENTER = CARTOON_GHOST_CELLS
CARTOON_OUTER_BUFFER_CELLS = 3

VECTOR_X_REFLECTION_PARITY = (-1.0, 1.0, 1.0)
RADIAL_VECTOR_PARITY = VECTOR_X_REFLECTION_PARITY[0]

PERIODIC_BC = 0
SOMMERFELD_BC = 1


def _map(vars: BSSNVariables, transform) -> BSSNVariables:
    out, host = [], False
    for f in vars:
        t, h = _dev(f)
        host = host or h
        out.append(transform(t, field_parity(t, VECTOR_X_REFLECTION_PARITY)))
    return BSSNVariables(*(_back(t, host) for t in out))


def _compact(positive_axis, parity):
    return reflect_tensor(positive_axis, parity, axis=-1, count=CARTOON_GHOST_CELLS)[..., :, None, None]


def _expanded(positive_axis, parity):
    return reflect_tensor(positive_axis, parity, axis=-1)[..., :, None, None]


def validate_cartoon_grid(vars: BSSNVariables, params: BSSNParameters) -> None:
    """Compact radial state and support geometry checks (reconstruction.py:61-111)."""
    nx, ny, nz = tuple(vars.conformal_factor.shape)
    if ny != 1 or nz != 1:
        raise ValueError("spherical Cartoon state requires an (Nr + 4) x 1 x 1 grid")
    if nx - CARTOON_GHOST_CELLS < 6:
        raise ValueError("spherical Cartoon mode requires at least six radial points")
    if params.xl_bc != PERIODIC_BC:
        raise ValueError("Cartoon x-left is a parity ghost region, not a physical boundary")
    if params.xr_bc != SOMMERFELD_BC:
        raise ValueError("Cartoon x-right must use the Sommerfeld boundary")
    if any(c != PERIODIC_BC for c in (params.yl_bc, params.yr_bc, params.zl_bc, params.zr_bc)):
        raise ValueError("Cartoon y/z support faces must be periodic")
    if float(params.mad_q) != 1.0:
        raise ValueError("Cartoon reconstruction requires mad_q=1 for its 9 x 9 support")
    dx = float(params.dx)
    if not math.isfinite(dx) or dx <= 0.0:
        raise ValueError("spherical Cartoon requires finite dx > 0")
    expected = (-(CARTOON_GHOST_CELLS - 0.5) * dx, -CARTOON_GHOST_CELLS * dx, -CARTOON_GHOST_CELLS * dx)
    actual = (params.x_min, params.y_min, params.z_min)
    if any(abs(float(a) - e) > 1.0e-12 * max(1.0, abs(e)) for a, e in zip(actual, expected)):
        raise ValueError("Cartoon coordinate minima must be (-3.5dx, -4dx, -4dx)")


def cartoon_centerline(field):
    """The x axis of compact storage or of a reconstructed support (reconstruction.py:114-119)."""
    if tuple(field.shape[-2:]) == (1, 1):
        return field[..., :, 0, 0]
    return field[..., :, CARTOON_CENTER, CARTOON_CENTER]


def cartoon_positive_radius(field):
    """The authoritative positive half-axis (reconstruction.py:122-125)."""
    return cartoon_centerline(field)[..., CARTOON_GHOST_CELLS:]


def compact_cartoon_state(vars: BSSNVariables) -> BSSNVariables:
    """Even full signed x axis -> compact storage (reconstruction.py:128-144)."""
    nx, ny, nz = tuple(vars.conformal_factor.shape)
    if ny != 1 or nz != 1 or nx % 2:
        raise ValueError("Cartoon initialization requires an even Nx x 1 x 1 signed axis")
    return _map(vars, lambda f, p: _compact(f[..., nx // 2:, 0, 0], p))


def enforce_spherical_symmetry(vars: BSSNVariables) -> BSSNVariables:
    """Discard the components spherical symmetry forbids on the positive radius
    (tensor off-diagonals, zz := yy, transverse vector components), then
    rebuild the parity ghosts (reconstruction.py:147-189)."""
    return _calls.fill_ghosts(vars, axi=False)


def _outer_buffer(axis: torch.Tensor, asymptotic, dx: float) -> torch.Tensor:
    spacing = torch.tensor(float(dx), dtype=torch.float64, device=axis.device)
    a = torch.as_tensor(asymptotic, dtype=torch.float64, device=axis.device).expand(axis.shape[:-1])[..., None]
    outer = (axis.shape[-1] - CARTOON_GHOST_CELLS - 0.5) * spacing
    radius = outer + spacing * torch.arange(1, CARTOON_OUTER_BUFFER_CELLS + 1, dtype=torch.float64,
                                            device=axis.device)
    buffer = a + (axis[..., -1:] - a) * (outer / radius)
    return torch.cat((axis, buffer), dim=-1)


def radial_interpolate(positive_axis, radius, dx: float, parity=SCALAR_PARITY, asymptotic_value=0.0):
    """Interpolate a positive-axis profile at arbitrary radii: parity through the
    origin, Sommerfeld 1/r continuation past the outer face (reconstruction.py:235-262)."""
    axis, host = _dev(positive_axis)
    r, _ = _dev(radius)
    axis = reflect_tensor(axis, parity, axis=-1, count=CARTOON_GHOST_CELLS)
    axis = _outer_buffer(axis, asymptotic_value, dx)
    q = r / float(dx) + CARTOON_GHOST_CELLS - 0.5
    return _back(lagrange6_nonperiodic(axis, q, axis=-1), host)


def transformation_matrix(x, y, z):
    """Lambda^i_jbar with radial, azimuthal and polar unit columns (reconstruction.py:265-309)."""
    xt, host = _dev(x)
    yt, _ = _dev(y)
    zt, _ = _dev(z)
    xt, yt, zt = torch.broadcast_tensors(xt, yt, zt)
    r = torch.sqrt(xt * xt + yt * yt + zt * zt)
    rho = torch.sqrt(xt * xt + yt * yt)
    safe = torch.where(rho > 0.0, rho, torch.ones_like(rho))
    zero, one = torch.zeros_like(xt), torch.ones_like(xt)
    off = (rho > 0.0)[None]
    radial = torch.stack((xt / r, yt / r, zt / r))
    azimuthal = torch.where(off, torch.stack((-yt / safe, xt / safe, zero)), torch.stack((zero, one, zero)))
    polar = torch.where(off, torch.stack((-xt * zt / (r * safe), -yt * zt / (r * safe), rho / r)),
                        torch.stack((-zt / r, zero, zero)))
    return _back(torch.stack((radial, azimuthal, polar), dim=1), host)


def reconstruct_cartoon_support(vars: BSSNVariables, params: BSSNParameters) -> BSSNVariables:
    """The (Nr+4) x 9 x 9 Cartesian support from the four independent radial
    profiles (reconstruction.py:336-385), computed by ``bssn_cartoon_reconstruct``."""
    return _calls.reconstruct(vars, params, axi=False)


def _project_support_field(field, parity):
    return _compact(field[..., CARTOON_GHOST_CELLS:, CARTOON_CENTER, CARTOON_CENTER], parity)


def project_cartoon_rhs(rhs: BSSNVariables) -> BSSNVariables:
    """Keep the centre-line positive radii and rebuild ghosts (reconstruction.py:388-398)."""
    return _map(rhs, _project_support_field)


def project_cartoon_scalar(field):
    t, host = _dev(field)
    return _back(_project_support_field(t, SCALAR_PARITY), host)


def project_cartoon_vector(field):
    t, host = _dev(field)
    return _back(_project_support_field(t, torch.tensor(VECTOR_X_REFLECTION_PARITY, device=t.device)), host)


def expand_cartoon_axis(vars: BSSNVariables) -> BSSNVariables:
    """Mirror the positive radius onto the complete signed x axis (reconstruction.py:415-423)."""
    return _map(vars, lambda f, p: _expanded(cartoon_positive_radius(f), p))


def expand_cartoon_scalar(field):
    t, host = _dev(field)
    return _back(_expanded(cartoon_positive_radius(t), SCALAR_PARITY), host)


def expand_cartoon_vector(field):
    t, host = _dev(field)
    return _back(_expanded(cartoon_positive_radius(t), torch.tensor(VECTOR_X_REFLECTION_PARITY, device=t.device)),
                 host)


__all__ = [
    "CARTOON_CENTER", "CARTOON_GHOST_CELLS", "CARTOON_OUTER_BUFFER_CELLS", "CARTOON_SUPPORT_SIZE",
    "RADIAL_VECTOR_PARITY", "cartoon_centerline", "cartoon_positive_radius", "compact_cartoon_state",
    "enforce_spherical_symmetry", "expand_cartoon_axis", "expand_cartoon_scalar", "expand_cartoon_vector",
    "project_cartoon_rhs", "project_cartoon_scalar", "project_cartoon_vector", "radial_interpolate",
    "reconstruct_cartoon_support", "transformation_matrix", "validate_cartoon_grid",
]
