"""Apparent-horizon finder on the GPU (mirrors JAX_BSSN/utilities/apparent_horizon.py).

Same names, arguments, defaults and error messages as the reference: one
dense-Newton finder for star-shaped marginally outer trapped surfaces about a
fixed centre, on geometry stored as a radial line (r,), a signed x-z plane
(x, z) or a Cartesian volume (x, y, z).  The arithmetic runs in
``libbssn_gb300.so``:

- ``bssn_horizon_surface``: the expansion and area density at every node
  (C1 Hermite geometry, fourth-order angular differences), with the residual
  norm's ingredients and the area summed on the device;
- ``bssn_horizon_newton_direction``: the Newton Jacobian assembled row by row
  in band storage from each node's pointwise partials, and the band LU solve;
- ``bssn_horizon_regrid``: the angular audit and refinement interpolation.

The host keeps the reference's control flow (line search, audit, refinement)
and reads four numbers per surface evaluation.  The reference differentiates
its residual with JAX; here each node's partials come from central
differences of relative step ``FD_STEP``, so the Newton iterates differ from
the reference's at that level while the converged surface does not.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _device, _native

FD_STEP = 1.0e-6


def _host_f64(a) -> np.ndarray:
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    return np.asarray(a, dtype=np.float64)


def _dev(a, device) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        return a.detach().to(device=device, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(np.asarray(a, dtype=np.float64)), device=device)


def _check(status: int) -> None:
    if status != _native.BSSN_OK:
        message = _native.last_error()
        if status in (_native.BSSN_ERR_INVALID, _native.BSSN_ERR_WORKSPACE):
            raise ValueError(message)
        raise RuntimeError(message)


class HorizonGeometry:
    """The device geometry ``build_geometry`` returns as its table."""

    def __init__(self, axes, gamma: torch.Tensor, kij: torch.Tensor, margin: int):
        self.axes = axes
        self.gamma = gamma
        self.kij = kij
        self.margin = int(margin)
        self.device = gamma.device
        s = _native.BssnHorizonGeometry()
        s.gamma = gamma.data_ptr()
        s.curvature = kij.data_ptr()
        s.dims = len(axes)
        for a, axis in enumerate(axes):
            s.size[a] = len(axis)
            s.origin[a] = float(axis[0])
            s.spacing[a] = float(axis[1] - axis[0])
        s.margin = self.margin
        self.struct = s


def sample(table: HorizonGeometry, points):
    """gamma[n,i,j], d_gamma[n,k,i,j], Kij[n,i,j], valid[n] at Cartesian points (:91-98)."""
    pts = _dev(points, table.device).reshape(-1, 3).contiguous()
    n = pts.shape[0]
    gamma = torch.empty((n, 3, 3), dtype=torch.float64, device=table.device)
    d_gamma = torch.empty((n, 3, 3, 3), dtype=torch.float64, device=table.device)
    kij = torch.empty((n, 3, 3), dtype=torch.float64, device=table.device)
    valid = torch.empty(n, dtype=torch.int32, device=table.device)
    _check(_native.load().bssn_horizon_sample(ctypes.byref(table.struct), pts.data_ptr(), n, gamma.data_ptr(),
                                              d_gamma.data_ptr(), kij.data_ptr(), valid.data_ptr(),
                                              _device.stream_handle()))
    return gamma, d_gamma, kij, valid.bool()


def build_geometry(coordinates, gamma, Kij, margin=4):
    """Return (table, sample), where sample(table, points) evaluates the geometry (:22-98).

    Coordinates are (r,), (x,z), or (x,y,z); tensors have shape (3,3,*grid).
    """
    if isinstance(coordinates, np.ndarray) and coordinates.ndim == 1:
        coordinates = (coordinates,)
    axes = tuple(np.asarray(_host_f64(axis), dtype=float) for axis in coordinates)
    if len(axes) not in (1, 2, 3):
        raise ValueError('Pass (r,), (x,z), or (x,y,z) coordinates')
    if margin < 2:
        raise ValueError('Hermite interpolation needs at least two margin cells')
    for axis in axes:
        if (axis.ndim != 1 or len(axis) < max(6, 2 * margin + 2) or axis[1] <= axis[0]
                or not np.allclose(np.diff(axis), axis[1] - axis[0], rtol=1.e-10, atol=1.e-14)):
            raise ValueError('Coordinates must be increasing uniform axes with a resolved interior')
    device = _device.require_cuda()
    shape = (3, 3) + tuple(len(axis) for axis in axes)
    g, k = _dev(gamma, device), _dev(Kij, device)
    if tuple(g.shape) != shape or tuple(k.shape) != shape:
        raise ValueError(f'Physical gamma and Kij must have shape {shape}')
    for tensor in (g, k):
        if not torch.allclose(tensor, tensor.transpose(0, 1), rtol=1.e-12, atol=1.e-14):
            raise ValueError('Physical gamma and Kij must be symmetric')
    if len(axes) == 1:
        if axes[0][0] <= 0:
            raise ValueError('The radial line must contain positive radii')
        for tensor in (g, k):
            scale = tensor.abs().amax(dim=(0, 1))
            error = torch.stack([(tensor[1, 1] - tensor[2, 2]).abs(), tensor[0, 1].abs(), tensor[0, 2].abs(),
                                 tensor[1, 2].abs()]).amax(dim=0)
            # Evolved Cartoon data can carry roundoff in nominally zero terms.
            if bool(torch.any(error > 1.e-10 * scale + 1.e-14)):
                raise ValueError('Radial tensors must be diagonal with equal transverse components')
    elif len(axes) == 2 and not axes[0][margin] < 0 < axes[0][-margin - 1]:
        raise ValueError('Axisymmetric input needs a signed x-z plane')
    return HorizonGeometry(axes, g, k, margin), sample


def angular_grid(n_theta, n_phi):
    """Cell-centered polar nodes, periodic azimuthal nodes, and polar area weights (:101-117)."""
    if n_theta < 6 or n_phi < 6 or n_phi % 2:
        raise ValueError('Use at least six nodes per angle and an even n_phi')
    theta = (np.arange(n_theta) + 0.5) * np.pi / n_theta
    phi = np.arange(n_phi) * 2 * np.pi / n_phi
    # The regular area factor against sin(theta), exact for the resolved cosine modes.
    modes = np.arange(n_theta)
    integrals = np.zeros(n_theta)
    even = modes[modes % 2 == 0]
    integrals[even] = 2 / (1 - even ** 2)
    integrals[1:] *= 2
    weights = integrals @ np.cos(np.outer(modes, theta)) / n_theta
    return theta, phi, weights


def theta_ghosts(field, width):
    """A scalar crossing a pole reappears half a turn around the azimuth (:120-125)."""
    f = field if isinstance(field, torch.Tensor) else _dev(field, _device.require_cuda())
    shift = f.shape[1] // 2
    low = torch.flip(torch.roll(f[:width], shift, dims=1), dims=(0,))
    high = torch.flip(torch.roll(f[-width:], shift, dims=1), dims=(0,))
    return torch.cat((low, f, high), dim=0)


def angular_derivatives(field):
    """h_theta, h_thetatheta, h_phi, h_phiphi, h_thetaphi on the full sphere (:125-144)."""
    device = _device.require_cuda()
    f = _dev(field, device)
    n_theta, n_phi = f.shape
    out = torch.empty((5, n_theta, n_phi), dtype=torch.float64, device=device)
    _check(_native.load().bssn_horizon_angular_derivatives(f.data_ptr(), n_theta, n_phi, out.data_ptr(),
                                                           _device.stream_handle()))
    return tuple(out[m] for m in range(5))


def interpolate_angular(radius, theta, phi):
    """Interpolate a surface onto new angular nodes with the same pole extension (:147-157)."""
    device = _device.require_cuda()
    h = _dev(radius, device)
    t = _dev(theta, device).reshape(-1)
    p = _dev(phi, device).reshape(-1)
    out = torch.empty((t.numel(), p.numel()), dtype=torch.float64, device=device)
    _check(_native.load().bssn_horizon_regrid(h.data_ptr(), h.shape[0], h.shape[1], t.data_ptr(), t.numel(),
                                              p.data_ptr(), p.numel(), out.data_ptr(), _device.stream_handle()))
    return out


class _Surfaces:
    """Device buffers of one angular resolution."""

    def __init__(self, table: HorizonGeometry, center, n_theta: int, n_phi: int):
        self.lib = _native.load()
        self.table = table
        self.nt, self.np = int(n_theta), int(n_phi)
        self.n = self.nt * self.np
        _, _, weights = angular_grid(self.nt, self.np)
        dev = table.device
        self.weights = torch.as_tensor(weights, device=dev)
        self.center = (ctypes.c_double * 3)(*[float(c) for c in center])
        nbytes = self.lib.bssn_horizon_workspace_bytes(self.nt, self.np)
        if nbytes == 0:
            raise ValueError(_native.last_error() or 'invalid angular surface')
        self.ws = _device.workspace(nbytes, dev, tag="horizon")
        self.expansion = torch.empty((self.nt, self.np), dtype=torch.float64, device=dev)
        self.density = torch.empty_like(self.expansion)
        self.trial = torch.empty_like(self.expansion)
        self.trial_expansion = torch.empty_like(self.expansion)
        self.delta = torch.empty_like(self.expansion)
        self.summary = torch.empty(4, dtype=torch.float64, device=dev)
        self.dsummary = torch.empty(2, dtype=torch.float64, device=dev)

    def measure(self, radius, direction=None, step=0.0, expansion=None, density=True):
        """Evaluate a surface; returns (sum h, max |Theta|, unusable nodes, area)."""
        exp = self.expansion if expansion is None else expansion
        _check(self.lib.bssn_horizon_surface(
            ctypes.byref(self.table.struct), self.center, radius.data_ptr(),
            direction.data_ptr() if direction is not None else None, float(step), self.nt, self.np,
            self.weights.data_ptr(), self.trial.data_ptr() if direction is not None else None, exp.data_ptr(),
            self.density.data_ptr() if density else None, self.summary.data_ptr(), self.ws.data_ptr(),
            self.ws.numel(), _device.stream_handle()))
        s = self.summary.cpu().numpy()
        return float(s[0]), float(s[1]), int(s[2]), float(s[3])

    def direction(self, radius):
        """Newton direction -J^-1 Theta at radius (Theta from the last measure); (max |delta|, nonfinite)."""
        _check(self.lib.bssn_horizon_newton_direction(
            ctypes.byref(self.table.struct), self.center, radius.data_ptr(), self.expansion.data_ptr(), self.nt,
            self.np, FD_STEP, self.delta.data_ptr(), self.dsummary.data_ptr(), self.ws.data_ptr(), self.ws.numel(),
            _device.stream_handle()))
        s = self.dsummary.cpu().numpy()
        return float(s[0]), int(s[1])

    def jacobian(self, radius):
        dense = torch.empty((self.n, self.n), dtype=torch.float64, device=self.table.device)
        _check(self.lib.bssn_horizon_jacobian(
            ctypes.byref(self.table.struct), self.center, radius.data_ptr(), self.nt, self.np, FD_STEP,
            dense.data_ptr(), self.ws.data_ptr(), self.ws.numel(), _device.stream_handle()))
        return dense


def surface(radius, center, table, sample=sample):
    """Expansion, regular area density, and validity on a full angular grid (:160-236)."""
    h = _dev(radius, table.device)
    buffers = _Surfaces(table, _host_f64(center).reshape(3), *h.shape)
    _, _, bad, _ = buffers.measure(h)
    return buffers.expansion, buffers.density, bad == 0


class ExpansionResidual:
    """residual(h) = surface(h, center, table)[0].reshape(-1), differentiable by dense_jacobian."""

    def __init__(self, center, table: HorizonGeometry):
        self.center = _host_f64(center).reshape(3)
        self.table = table

    def __call__(self, radius):
        return surface(radius, self.center, self.table)[0].reshape(-1)


def dense_jacobian(residual, radius):
    """Differentiate all residuals with respect to all radii (:239-250).

    An ``ExpansionResidual`` is assembled by the band kernel; any other
    callable is differentiated column by column with central differences.
    """
    device = _device.require_cuda()
    h = _dev(radius, device)
    if isinstance(residual, ExpansionResidual):
        return _Surfaces(residual.table, residual.center, *h.shape).jacobian(h)
    columns = []
    flat = h.reshape(-1)
    for j in range(flat.numel()):
        e = torch.zeros_like(flat)
        step = FD_STEP * max(abs(float(flat[j])), 1.0)
        e[j] = step
        up = residual((flat + e).reshape(h.shape)).reshape(-1)
        dn = residual((flat - e).reshape(h.shape)).reshape(-1)
        columns.append((up - dn) / (2 * step))
    return torch.stack(columns, dim=1)


def find_apparent_horizon(coordinates, gamma, Kij, *, center, initial_radius, n_theta=12, n_phi=24, max_angular=48,
                          tolerance=1.e-8, audit_tolerance=1.e-4, mass_tolerance=1.e-3, max_iterations=50, margin=4):
    """Find the marginal surface reached from the supplied center and guess (:253-338).

    initial_radius is a scalar or a positive (n_theta,n_phi) array; an array
    defines the starting grid, overriding n_theta and n_phi.  The center stays
    fixed.  Every accepted result passes an angular audit and area-mass
    convergence between two resolutions; residuals are mean(h)*max(abs(Theta)).
    Returns a plain dictionary; raises RuntimeError on numerical failure.
    """
    table, _ = build_geometry(coordinates, gamma, Kij, margin=margin)
    center = np.asarray(_host_f64(center), dtype=float)
    if center.shape != (3,) or not np.all(np.isfinite(center)):
        raise ValueError('center must be a finite Cartesian triple')
    initial = np.asarray(_host_f64(initial_radius), dtype=float)
    if initial.ndim == 0:
        initial = np.full((n_theta, n_phi), initial)
    elif initial.ndim != 2:
        raise ValueError('initial_radius must be a scalar or a two-dimensional angular surface')
    angular_grid(*initial.shape)
    if not np.all(np.isfinite(initial)) or np.any(initial <= 0):
        raise ValueError('The initial surface must have finite positive radii')
    if max_angular < 2 * initial.shape[0]:
        raise ValueError('max_angular must allow at least one angular refinement')
    device = table.device
    radius = torch.as_tensor(np.ascontiguousarray(initial), device=device)
    history = []
    previous_mass = None
    while True:
        S = _Surfaces(table, center, *radius.shape)
        for iteration in range(max_iterations + 1):
            total, peak, bad, area = S.measure(radius)
            mean = total / S.n
            residual_norm = mean * peak
            if bad:
                raise RuntimeError('Surface leaves the resolved domain or has nonphysical geometry')
            if residual_norm < tolerance:
                break
            if iteration == max_iterations:
                raise RuntimeError(f'Newton did not converge after {max_iterations} iterations: {residual_norm:.3e}')
            largest, nonfinite = S.direction(radius)
            if nonfinite:
                raise RuntimeError('Newton Jacobian solve is singular or nonfinite')
            step = min(1., 0.1 * mean / largest)
            # The physical domain and positive-definite metric are checked on
            # every trial, including those rejected by the line search.
            for _ in range(20):
                t_total, t_peak, t_bad, _ = S.measure(radius, S.delta, step, expansion=S.trial_expansion,
                                                      density=False)
                trial_norm = (t_total / S.n) * t_peak
                if not t_bad and trial_norm < residual_norm * (1 - 1.e-4 * step):
                    radius = S.trial.clone()
                    break
                step *= 0.5
            else:
                raise RuntimeError(f'Newton line search stalled at residual {residual_norm:.3e}')

        nt, nphi = radius.shape
        theta, phi, weights = angular_grid(nt, nphi)
        mass = np.sqrt(area / (16 * np.pi))
        audit_theta, audit_phi, _ = angular_grid(2 * nt + 2, 2 * nphi + 2)
        audit_radius = interpolate_angular(radius, audit_theta, audit_phi)
        A = _Surfaces(table, center, *audit_radius.shape)
        a_total, a_peak, a_bad, _ = A.measure(audit_radius, density=False)
        if a_bad:
            raise RuntimeError('Angular audit leaves the resolved domain or has nonphysical geometry')
        audit = (a_total / A.n) * a_peak
        mass_change = np.inf if previous_mass is None else abs(mass / previous_mass - 1)
        history.append((nt, nphi, mass, residual_norm, audit, iteration))
        if previous_mass is not None and audit < audit_tolerance and mass_change < mass_tolerance:
            return dict(theta=theta, phi=phi, radius=radius.cpu().numpy(), center=center,
                        expansion=S.expansion.cpu().numpy(), area=area, mass=float(mass),
                        residual=residual_norm, audit_residual=audit, mass_relative_change=mass_change,
                        convergence=np.asarray(history), iterations=sum(int(row[5]) for row in history))
        if 2 * nt > max_angular:
            raise RuntimeError(f'Angular convergence failed: audit={audit:.3e}, mass change={mass_change:.3e}')
        theta, phi, _ = angular_grid(2 * nt, 2 * nphi)
        radius = interpolate_angular(radius, theta, phi)
        previous_mass = mass
