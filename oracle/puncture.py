"""Bowen-York puncture initial data restated in NumPy (test infrastructure).

Follows uwplasma/JAX_BSSN/utilities/bowen_york_solver.py:
  cell_centered_grid                        :11-19
  axisymmetric_cell_centered_grid           :22-49
  brill_lindquist_conformal_factor          :52-63   1 + sum_a m_a / (2 r_a)
  bowen_york_extrinsic_curvature            :66-91   3/(2 r^2) (P n + n P - (I - n n) P.n)
  contract_conformal_curvature              :93-101
  laplacian, axisymmetric_laplacian         :104-148 zero outer values; even axis ghost
  hamiltonian_source / linearized source    :151-162
  linearized operators and residuals        :165-230
  solve_conformal_factor                    :283-366 Newton + CG
  solve_axisymmetric_conformal_factor       :369-479 Newton + BiCGSTAB

The reference's Krylov solvers are jax.scipy.sparse.linalg.cg / bicgstab (JAX,
absent here).  Both are the textbook methods started from zero with the
stopping bound r.r <= max(tol^2 b.b, atol^2); SciPy's cg / bicgstab (rtol =
tol) implement the same methods with the same bound and stand in for them
here, as they do under the NumPy jax stand-in that produced the goldens.
Integer powers psi^-7, psi^-8 go through the C library's pow, as under that
stand-in.  ``counts``, when given, collects the Krylov iterations of each
Newton correction.  Only the tests and the bench's CPU legs import this module.
"""

from __future__ import annotations

import math

import numpy as np


def _pow(x, y):
    x = np.asarray(x, dtype=np.float64)
    return np.frompyfunc(math.pow, 2, 1)(x, float(y)).astype(np.float64)


def cell_centered_grid(num_points=48, half_width=12.0):
    dx = 2.0 * half_width / num_points
    axis = -half_width + (np.arange(num_points, dtype=np.float64) + 0.5) * dx
    return np.stack(np.meshgrid(axis, axis, axis, indexing="ij"), axis=-1), dx


def axisymmetric_cell_centered_grid(num_radial_points=48, radial_extent=12.0):
    dx = radial_extent / num_radial_points
    rho = (np.arange(num_radial_points, dtype=np.float64) + 0.5) * dx
    z = -radial_extent + (np.arange(2 * num_radial_points, dtype=np.float64) + 0.5) * dx
    R, Y, Z = np.meshgrid(rho, np.zeros(1), z, indexing="ij")
    return np.stack((R, Y, Z), axis=-1), dx


def _offsets(positions, grid):
    """Per puncture: displacement (..., 3) and its length."""
    out = []
    for x in np.asarray(positions, dtype=np.float64):
        d = grid - x
        r = np.sqrt(d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2])
        out.append((d, r))
    return out


def brill_lindquist_conformal_factor(masses, positions, grid):
    grid = np.asarray(grid, dtype=np.float64)
    total = None
    for m, (_, r) in zip(np.asarray(masses, dtype=np.float64), _offsets(positions, grid)):
        term = m / (2.0 * r)
        total = term if total is None else total + term
    return 1.0 + total


def bowen_york_extrinsic_curvature(momenta, positions, grid):
    grid = np.asarray(grid, dtype=np.float64)
    total = None
    for P, (d, r) in zip(np.asarray(momenta, dtype=np.float64), _offsets(positions, grid)):
        n = d / r[..., None]
        pn = P[0] * n[..., 0] + P[1] * n[..., 1] + P[2] * n[..., 2]
        K = np.empty(grid.shape[:-1] + (3, 3))
        c = 3.0 / (2.0 * (r * r))
        for i in range(3):
            for j in range(3):
                transverse = (1.0 if i == j else 0.0) - n[..., i] * n[..., j]
                K[..., i, j] = c * ((P[i] * n[..., j] + n[..., i] * P[j]) - transverse * pn)
        total = K if total is None else total + K
    return total


def contract_conformal_curvature(K):
    K = np.asarray(K, dtype=np.float64)
    s = K[..., 0, 0] * K[..., 0, 0]
    for q in range(1, 9):
        i, j = divmod(q, 3)
        s = s + K[..., i, j] * K[..., i, j]
    return s


def laplacian(interior, dx):
    f = np.pad(np.asarray(interior, dtype=np.float64), 1)
    c = f[1:-1, 1:-1, 1:-1]
    s = f[2:, 1:-1, 1:-1] + f[:-2, 1:-1, 1:-1]
    s = s + f[1:-1, 2:, 1:-1]
    s = s + f[1:-1, :-2, 1:-1]
    s = s + f[1:-1, 1:-1, 2:]
    s = s + f[1:-1, 1:-1, :-2]
    return (s - 6.0 * c) / dx ** 2


def axisymmetric_laplacian(interior, dx):
    f = np.pad(np.asarray(interior, dtype=np.float64), ((0, 1), (1, 1)))
    c = f[:-1, 1:-1]
    rp = f[1:, 1:-1]
    rm = np.concatenate((f[:1, 1:-1], f[:-2, 1:-1]), axis=0)   # even ghost at the axis
    rho = (np.arange(c.shape[0], dtype=np.float64) + 0.5) * dx
    radial_second = (rp - 2.0 * c + rm) / dx ** 2
    radial_first = (rp - rm) / (2.0 * rho[:, None] * dx)
    axial_second = (f[:-1, 2:] + f[:-1, :-2] - 2.0 * c) / dx ** 2
    return radial_second + radial_first + axial_second


def hamiltonian_source(psi, a2):
    return 1.0 / 8.0 * np.asarray(a2) * _pow(psi, -7)


def linearized_hamiltonian_source(delta, psi, a2):
    return -7.0 / 8.0 * np.asarray(a2) * _pow(psi, -8) * np.asarray(delta)


def linearized_hamiltonian_operator(delta, psi, a2, dx):
    return laplacian(delta, dx) + linearized_hamiltonian_source(delta, psi, a2)


def axisymmetric_linearized_hamiltonian_operator(delta, psi, a2, dx):
    return axisymmetric_laplacian(delta, dx) + linearized_hamiltonian_source(delta, psi, a2)


def hamiltonian_residual(u, psi_bl, K, dx):
    ui = np.asarray(u)[1:-1, 1:-1, 1:-1]
    a2 = contract_conformal_curvature(K)[1:-1, 1:-1, 1:-1]
    return laplacian(ui, dx) + hamiltonian_source(np.asarray(psi_bl)[1:-1, 1:-1, 1:-1] + ui, a2)


def axisymmetric_hamiltonian_residual(u, psi_bl, K, dx):
    ui = np.asarray(u)[:-1, 0, 1:-1]
    a2 = contract_conformal_curvature(K)[:-1, 0, 1:-1]
    return axisymmetric_laplacian(ui, dx) + hamiltonian_source(np.asarray(psi_bl)[:-1, 0, 1:-1] + ui, a2)


def _krylov(method, apply, b, tol, maxiter, counts=None):
    import scipy.sparse.linalg as sla
    shape = b.shape
    op = sla.LinearOperator((b.size, b.size), matvec=lambda v: apply(v.reshape(shape)).ravel())
    n = [0]

    def tick(_):
        n[0] += 1
    x, _ = method(op, b.ravel(), rtol=tol, atol=0.0, maxiter=maxiter, callback=tick)
    if counts is not None:
        counts.append(n[0])
    return x.reshape(shape)


def _newton(psi_bl_i, a2_i, lap, tol, max_newton, lin_tol, max_lin, method, checks, counts=None):
    u = np.zeros_like(psi_bl_i)
    history = []
    for it in range(max_newton + 1):
        psi = psi_bl_i + u
        res = lap(u) + hamiltonian_source(psi, a2_i)
        rms = float(np.sqrt(np.mean(res ** 2)))
        history.append(rms)
        if checks and not math.isfinite(rms):
            raise RuntimeError("Newton-Raphson solve produced a nonfinite residual")
        if rms <= tol:
            break
        if it == max_newton:
            raise RuntimeError(f"Newton-Raphson solve did not converge: RMS residual {rms:.3e} exceeds {tol:.3e}.")
        coef = -7.0 / 8.0 * a2_i * _pow(psi, -8)
        u = u + _krylov(method, lambda d: -(lap(d) + coef * d), res, lin_tol, max_lin, counts)
        if checks:
            if not np.all(np.isfinite(u)):
                raise RuntimeError("Newton-Raphson correction is nonfinite")
            if not np.all(psi_bl_i + u > 0.0):
                raise RuntimeError("Newton-Raphson correction made psi nonpositive")
    return u, history


def solve_conformal_factor(masses, positions, momenta, grid, dx, newton_tolerance=1.0e-10,
                           max_newton_iterations=12, cg_tolerance=1.0e-10, max_cg_iterations=1000, counts=None):
    import scipy.sparse.linalg as sla
    psi_bl = brill_lindquist_conformal_factor(masses, positions, grid)
    a2 = contract_conformal_curvature(bowen_york_extrinsic_curvature(momenta, positions, grid))
    inner = (slice(1, -1),) * 3
    u_i, history = _newton(psi_bl[inner], a2[inner], lambda f: laplacian(f, dx), newton_tolerance,
                           max_newton_iterations, cg_tolerance, max_cg_iterations, sla.cg, False, counts)
    u = np.pad(u_i, 1)
    return psi_bl + u, u, history


def solve_axisymmetric_conformal_factor(masses, positions, momenta, grid, dx, newton_tolerance=1.0e-10,
                                        max_newton_iterations=12, linear_tolerance=1.0e-10,
                                        max_linear_iterations=1000, counts=None):
    import scipy.sparse.linalg as sla
    psi_bl = brill_lindquist_conformal_factor(masses, positions, grid)
    a2 = contract_conformal_curvature(bowen_york_extrinsic_curvature(momenta, positions, grid))
    u_i, history = _newton(psi_bl[:-1, 0, 1:-1], a2[:-1, 0, 1:-1], lambda f: axisymmetric_laplacian(f, dx),
                           newton_tolerance, max_newton_iterations, linear_tolerance, max_linear_iterations,
                           sla.bicgstab, True, counts)
    u = np.pad(u_i, ((0, 1), (1, 1)))[:, None, :]
    return psi_bl + u, u, history
