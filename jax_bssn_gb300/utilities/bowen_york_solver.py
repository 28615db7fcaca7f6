"""Bowen-York puncture initial data (mirrors JAX_BSSN/utilities/bowen_york_solver.py).

Same names, arguments, defaults and error messages as the reference.  The
grids are float64 CUDA tensors; every other function accepts device tensors or
host arrays and returns device tensors for device inputs, NumPy arrays for
host inputs.  All arithmetic runs in ``libbssn_gb300.so``:

- ``bssn_puncture_fields``: Brill-Lindquist psi, the Bowen-York curvature and
  its contraction, one kernel over the grid;
- ``bssn_puncture_operator``: the Laplacians, sources, linearised operators and
  residuals, in the reference's operation order;
- ``bssn_puncture_solve``: the whole Newton iteration with its Krylov solves
  (conjugate gradients on Cartesian grids, BiCGSTAB on meridional grids), each
  Krylov iteration a few kernels with on-device dot products; the host reads
  the residual once per Newton step.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np
import torch

from .. import _device, _native

_CONTRACT, _SOURCE, _LIN_SOURCE, _LAPLACIAN, _LIN_OPERATOR, _RESIDUAL = range(6)


def _is_host(*arrays) -> bool:
    return not any(isinstance(a, torch.Tensor) and a.is_cuda for a in arrays)


def _dev(a, device) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.asarray(a, dtype=np.float64), device=device).contiguous()


def _out(t: torch.Tensor, host: bool):
    return t.cpu().numpy() if host else t


def _host_f64(a) -> np.ndarray:
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def cell_centered_grid(num_points=48, half_width=12.0):
    """A cubic cell-centred grid and its spacing (:11-19)."""
    device = _device.require_cuda()
    dx = 2.0 * half_width / num_points
    axis = -half_width + (torch.arange(num_points, dtype=torch.float64, device=device) + 0.5) * dx
    X, Y, Z = torch.meshgrid(axis, axis, axis, indexing="ij")
    return torch.stack((X, Y, Z), dim=-1).contiguous(), dx


def axisymmetric_cell_centered_grid(num_radial_points=48, radial_extent=12.0):
    """The positive-rho meridional grid (Nrho, 1, 2 Nrho, 3) and its spacing (:22-49)."""
    if not isinstance(num_radial_points, int) or num_radial_points < 2:
        raise ValueError("num_radial_points must be an integer of at least two")
    if not math.isfinite(radial_extent) or radial_extent <= 0.0:
        raise ValueError("radial_extent must be finite and positive")
    device = _device.require_cuda()
    dx = radial_extent / num_radial_points
    rho = (torch.arange(num_radial_points, dtype=torch.float64, device=device) + 0.5) * dx
    y = torch.zeros(1, dtype=torch.float64, device=device)
    z = -radial_extent + (torch.arange(2 * num_radial_points, dtype=torch.float64, device=device) + 0.5) * dx
    R, Y, Z = torch.meshgrid(rho, y, z, indexing="ij")
    return torch.stack((R, Y, Z), dim=-1).contiguous(), dx


def _punctures(masses, positions, momenta):
    m = _host_f64(masses).reshape(-1)
    x = _host_f64(positions).reshape(-1, 3)
    p = _host_f64(momenta).reshape(-1, 3)
    if not (len(m) == len(x) == len(p)) or len(m) == 0:
        raise ValueError("masses, positions and momenta must describe the same nonempty set of punctures")
    return m, x, p


def _fields(masses, positions, momenta, grid, want_psi, want_curvature, want_a2):
    lib = _native.load()
    device = _device.require_cuda()
    host = _is_host(grid)
    g = _dev(grid, device)
    if g.shape[-1] != 3:
        raise ValueError("grid must end with an axis of three coordinates")
    m, x, p = _punctures(masses, positions, momenta)
    lead = tuple(g.shape[:-1])
    npts = _device.prod(lead)
    psi = torch.empty(lead, dtype=torch.float64, device=device) if want_psi else None
    K = torch.empty(lead + (3, 3), dtype=torch.float64, device=device) if want_curvature else None
    a2 = torch.empty(lead, dtype=torch.float64, device=device) if want_a2 else None
    ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    dp = ctypes.POINTER(ctypes.c_double)
    _native.check(lib.bssn_puncture_fields(g.data_ptr(), npts, m.ctypes.data_as(dp), x.ctypes.data_as(dp),
                                           p.ctypes.data_as(dp), len(m), ptr(psi), ptr(K), ptr(a2),
                                           _device.stream_handle()), "puncture fields")
    return host, psi, K, a2


def brill_lindquist_conformal_factor(masses, positions, grid):
    """psi_BL = 1 + sum_a m_a / (2 r_a) (:52-63)."""
    m = _host_f64(masses).reshape(-1)
    host, psi, _, _ = _fields(m, positions, np.zeros((len(m), 3)), grid, True, False, False)
    return _out(psi, host)


def bowen_york_extrinsic_curvature(momenta, positions, grid):
    """The conformal Bowen-York curvature of boosted punctures (:66-91)."""
    p = _host_f64(momenta).reshape(-1, 3)
    host, _, K, _ = _fields(np.ones(len(p)), positions, p, grid, False, True, False)
    return _out(K, host)


def _operator(op, a, b, c, shape, dx, axi, out_shape, workspace=False):
    lib = _native.load()
    device = _device.require_cuda()
    host = _is_host(a, b, c)
    ta = _dev(a, device)
    tb = _dev(b, device) if b is not None else None
    tc = _dev(c, device) if c is not None else None
    out = torch.empty(out_shape, dtype=torch.float64, device=device)
    ws = _device.workspace(_device.prod(shape) * 8, device, tag="puncture_op") if workspace else None
    ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    _native.check(lib.bssn_puncture_operator(op, ta.data_ptr(), ptr(tb), ptr(tc), _device.shape3(shape), float(dx),
                                             int(axi), out.data_ptr(), ptr(ws), 0 if ws is None else ws.numel(),
                                             _device.stream_handle()), "puncture operator")
    return _out(out, host)


def contract_conformal_curvature(conformal_curvature):
    """A_ij A^ij with the flat metric (:93-101)."""
    lead = tuple(conformal_curvature.shape[:-2])
    if tuple(conformal_curvature.shape[-2:]) != (3, 3):
        raise ValueError("conformal_curvature must end with a 3x3 tensor")
    return _operator(_CONTRACT, conformal_curvature, None, None, (_device.prod(lead), 1, 1), 1.0, 0, lead)


def _same_shape(*arrays):
    shape = tuple(arrays[0].shape)
    if any(tuple(a.shape) != shape for a in arrays[1:]):
        raise ValueError("pointwise operands must share one shape")
    return shape


def hamiltonian_source(psi, curvature_squared):
    """S(psi) = A^2 psi^-7 / 8 (:151-155)."""
    shape = _same_shape(psi, curvature_squared)
    return _operator(_SOURCE, psi, curvature_squared, None, (_device.prod(shape), 1, 1), 1.0, 0, shape)


def linearized_hamiltonian_source(delta_u, psi_background, curvature_squared):
    """dS = -7/8 A^2 psi^-8 delta_u (:158-162)."""
    shape = _same_shape(delta_u, psi_background, curvature_squared)
    return _operator(_LIN_SOURCE, delta_u, psi_background, curvature_squared, (_device.prod(shape), 1, 1), 1.0, 0,
                     shape)


def _full_cartesian(interior_shape):
    if len(interior_shape) != 3 or min(interior_shape) < 1:
        raise ValueError("interior_field must be a nonempty three-dimensional array")
    return tuple(n + 2 for n in interior_shape)


def _full_meridional(interior_shape):
    if len(interior_shape) != 2 or min(interior_shape) < 1:
        raise ValueError("interior_field must be a nonempty (rho, z) array")
    return (interior_shape[0] + 1, 1, interior_shape[1] + 2)


def laplacian(interior_field, dx):
    """Seven-point Laplacian with zero values outside the interior (:104-118)."""
    shape = tuple(interior_field.shape)
    return _operator(_LAPLACIAN, interior_field, None, None, _full_cartesian(shape), dx, 0, shape, workspace=True)


def axisymmetric_laplacian(interior_field, dx):
    """Centred axisymmetric Laplacian with zero outer values (:121-148)."""
    shape = tuple(interior_field.shape)
    return _operator(_LAPLACIAN, interior_field, None, None, _full_meridional(shape), dx, 1, shape, workspace=True)


def linearized_hamiltonian_operator(delta_u, psi_background, curvature_squared, dx):
    """Laplacian(delta_u) + dS (:165-180)."""
    shape = _same_shape(delta_u, psi_background, curvature_squared)
    return _operator(_LIN_OPERATOR, delta_u, psi_background, curvature_squared, _full_cartesian(shape), dx, 0, shape,
                     workspace=True)


def axisymmetric_linearized_hamiltonian_operator(delta_u, psi_background, curvature_squared, dx):
    """The Newton Jacobian on the active axisymmetric cells (:183-198)."""
    shape = _same_shape(delta_u, psi_background, curvature_squared)
    return _operator(_LIN_OPERATOR, delta_u, psi_background, curvature_squared, _full_meridional(shape), dx, 1,
                     shape, workspace=True)


def hamiltonian_residual(u, psi_bl, conformal_curvature, dx):
    """The nonlinear Hamiltonian residual at interior grid points (:201-212)."""
    shape = _same_shape(u, psi_bl)
    if len(shape) != 3 or min(shape) < 3:
        raise ValueError("u must be a three-dimensional grid with at least three cells per axis")
    a2 = contract_conformal_curvature(conformal_curvature)
    return _operator(_RESIDUAL, u, psi_bl, a2, shape, dx, 0, tuple(n - 2 for n in shape))


def axisymmetric_hamiltonian_residual(u, psi_bl, conformal_curvature, dx):
    """The Hamiltonian residual on active meridional-grid cells (:215-230)."""
    shape = _same_shape(u, psi_bl)
    if len(shape) != 3 or shape[1] != 1:
        raise ValueError("u must have shape (Nrho, 1, Nz)")
    a2 = contract_conformal_curvature(conformal_curvature)
    return _operator(_RESIDUAL, u, psi_bl, a2, shape, dx, 1, (shape[0] - 1, shape[2] - 2))


@dataclass
class PunctureSolve:
    """A finished Newton solve: psi, u, the residual history and the Krylov
    iterations each correction took."""
    psi: object
    u: object
    residual_history: list
    linear_iterations: list


def puncture_solve(masses, positions, momenta, grid, dx, *, axisymmetric, newton_tolerance, max_newton_iterations,
                   linear_tolerance, max_linear_iterations) -> PunctureSolve:
    """The Newton-Krylov solve shared by both solvers, with its iteration counts."""
    lib = _native.load()
    device = _device.require_cuda()
    host, psi_bl, _, a2 = _fields(masses, positions, momenta, grid, True, False, True)
    shape = tuple(psi_bl.shape)
    if len(shape) != 3:
        raise ValueError("grid must be a three-dimensional grid of coordinates")
    nbytes = lib.bssn_puncture_workspace_bytes(_device.shape3(shape), int(axisymmetric))
    if nbytes == 0:
        raise ValueError(f"puncture solve: {_native.last_error()}")
    ws = _device.workspace(nbytes, device, tag="puncture")
    u = torch.empty(shape, dtype=torch.float64, device=device)
    psi = torch.empty(shape, dtype=torch.float64, device=device)
    nmax = max(int(max_newton_iterations), 0)
    history = (ctypes.c_double * (nmax + 1))()
    counts = (ctypes.c_int32 * max(nmax, 1))()
    length = ctypes.c_int32(0)
    status = lib.bssn_puncture_solve(psi_bl.data_ptr(), a2.data_ptr(), _device.shape3(shape), float(dx),
                                     int(axisymmetric), float(newton_tolerance), int(max_newton_iterations),
                                     float(linear_tolerance), int(max_linear_iterations), u.data_ptr(),
                                     psi.data_ptr(), history, ctypes.byref(length), counts, ws.data_ptr(),
                                     ws.numel(), _device.stream_handle())
    if status != _native.BSSN_OK:
        message = _native.last_error()
        if status in (_native.BSSN_ERR_INVALID, _native.BSSN_ERR_WORKSPACE):
            raise ValueError(message)
        raise RuntimeError(message)
    n = length.value
    return PunctureSolve(_out(psi, host), _out(u, host), [float(history[i]) for i in range(n)],
                         [int(counts[i]) for i in range(max(n - 1, 0))])


def solve_conformal_factor(masses, positions, momenta, grid, dx, newton_tolerance=1.0e-10, max_newton_iterations=12,
                           cg_tolerance=1.0e-10, max_cg_iterations=1000, verbose=False):
    """Newton iterations for the regular correction u on a Cartesian grid, each
    correction from conjugate gradients on the negative linearised operator
    (:283-366).  Returns (psi, u, residual_history)."""
    r = puncture_solve(masses, positions, momenta, grid, dx, axisymmetric=False, newton_tolerance=newton_tolerance,
                       max_newton_iterations=max_newton_iterations, linear_tolerance=cg_tolerance,
                       max_linear_iterations=max_cg_iterations)
    if verbose:
        for i, rms in enumerate(r.residual_history):
            print(f"Newton iteration {i:2d}: RMS residual = {rms:.3e}")
    return r.psi, r.u, r.residual_history


def _validate_axisymmetric_solver_inputs(masses, positions, momenta, grid, dx):
    """The reference's geometry checks (:233-280)."""
    masses_np = _host_f64(masses)
    positions_np = _host_f64(positions)
    momenta_np = _host_f64(momenta)
    grid_np = _host_f64(grid)
    if masses_np.ndim != 1 or masses_np.size == 0:
        raise ValueError("masses must be a nonempty one-dimensional array")
    expected_shape = (masses_np.size, 3)
    if positions_np.shape != expected_shape:
        raise ValueError(f"positions must have shape {expected_shape}")
    if momenta_np.shape != expected_shape:
        raise ValueError(f"momenta must have shape {expected_shape}")
    if not np.all(np.isfinite(masses_np)) or np.any(masses_np <= 0.0):
        raise ValueError("masses must be finite and positive")
    if not np.all(np.isfinite(positions_np)):
        raise ValueError("positions must be finite")
    if not np.all(np.isfinite(momenta_np)):
        raise ValueError("momenta must be finite")
    if not np.allclose(positions_np[:, :2], 0.0, rtol=0.0, atol=1.0e-14):
        raise ValueError("axisymmetric punctures must lie on the z axis")
    if not np.allclose(momenta_np[:, :2], 0.0, rtol=0.0, atol=1.0e-14):
        raise ValueError("axisymmetric puncture momenta must be parallel to z")
    if grid_np.ndim != 4 or grid_np.shape[1] != 1 or grid_np.shape[-1] != 3:
        raise ValueError("grid must have shape (Nrho, 1, Nz, 3)")
    if grid_np.shape[0] < 2 or grid_np.shape[2] < 3:
        raise ValueError("grid requires at least two rho and three z cells")
    if not math.isfinite(float(dx)) or float(dx) <= 0.0:
        raise ValueError("dx must be finite and positive")
    if not np.all(np.isfinite(grid_np)):
        raise ValueError("grid coordinates must be finite")
    rho = grid_np[:, 0, 0, 0]
    z = grid_np[0, 0, :, 2]
    expected_rho = (np.arange(grid_np.shape[0]) + 0.5) * float(dx)
    if not np.allclose(rho, expected_rho):
        raise ValueError("grid rho coordinates must be positive half-cell centers")
    if not np.allclose(grid_np[..., 0], rho[:, None, None]):
        raise ValueError("grid rho coordinates must be constant along z")
    if not np.allclose(grid_np[..., 1], 0.0):
        raise ValueError("axisymmetric grid must lie on y=0")
    if not np.allclose(grid_np[..., 2], z[None, None, :]):
        raise ValueError("grid z coordinates must be constant along rho")
    if not np.allclose(np.diff(z), float(dx)):
        raise ValueError("grid z spacing must equal dx")


def solve_axisymmetric_conformal_factor(masses, positions, momenta, grid, dx, newton_tolerance=1.0e-10,
                                        max_newton_iterations=12, linear_tolerance=1.0e-10,
                                        max_linear_iterations=1000, verbose=False):
    """Bowen-York puncture data on a cell-centred meridional grid, Newton with
    BiCGSTAB corrections (:369-479).  Returns (psi, u, residual_history)."""
    _validate_axisymmetric_solver_inputs(masses, positions, momenta, grid, dx)
    for name, value in (("newton_tolerance", newton_tolerance), ("linear_tolerance", linear_tolerance)):
        if not math.isfinite(value) or value <= 0.0:
            raise ValueError(f"{name} must be finite and positive")
    if not isinstance(max_newton_iterations, int) or max_newton_iterations < 0:
        raise ValueError("max_newton_iterations must be a nonnegative integer")
    if not isinstance(max_linear_iterations, int) or max_linear_iterations < 1:
        raise ValueError("max_linear_iterations must be a positive integer")
    r = puncture_solve(masses, positions, momenta, grid, dx, axisymmetric=True, newton_tolerance=newton_tolerance,
                       max_newton_iterations=max_newton_iterations, linear_tolerance=linear_tolerance,
                       max_linear_iterations=max_linear_iterations)
    if verbose:
        for i, rms in enumerate(r.residual_history):
            print(f"Newton iteration {i:2d}: RMS residual = {rms:.3e}")
    return r.psi, r.u, r.residual_history
