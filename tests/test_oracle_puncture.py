"""The NumPy restatement of the Bowen-York solver against goldens produced by
the reference's own utilities/bowen_york_solver.py, and the reference suite's
known answers (tests/test_bowen_york.py)."""

import json

import numpy as np
import pytest

from oracle import puncture as op

from .helpers import load_golden

CASES = ("cart_single", "cart_binary", "axi_single", "axi_binary", "axi_zero")


@pytest.fixture(scope="module")
def gold():
    return load_golden("puncture")


def _case(gold, name):
    return json.loads(str(gold[f"{name}.case"]))


@pytest.mark.parametrize("name", CASES)
def test_grids_and_puncture_fields(gold, name):
    case = _case(gold, name)
    n, extent = case["grid"]
    grid, dx = (op.axisymmetric_cell_centered_grid if case["axi"] else op.cell_centered_grid)(n, extent)
    np.testing.assert_array_equal(grid, gold[f"{name}.grid"])
    assert dx == float(gold[f"{name}.dx"])
    psi_bl = op.brill_lindquist_conformal_factor(case["masses"], case["positions"], grid)
    # the stand-in's einsum sums the three squares of |x - x_a|^2 in its own
    # order, so radii (and all that follows) agree to an ulp, not bitwise
    np.testing.assert_allclose(psi_bl, gold[f"{name}.psi_bl"], rtol=5e-16, atol=0)
    K = op.bowen_york_extrinsic_curvature(case["momenta"], case["positions"], grid)
    ref = gold[f"{name}.curvature"]
    np.testing.assert_allclose(K, ref, rtol=0, atol=1e-15 * max(np.abs(ref).max(), 1e-300))


@pytest.mark.parametrize("name", ["cart_binary", "axi_binary"])
def test_operators(gold, name):
    dx = float(gold[f"{name}.dx"])
    axi = name.startswith("axi")
    inner = (slice(None, -1), 0, slice(1, -1)) if axi else (slice(1, -1),) * 3
    a2 = op.contract_conformal_curvature(gold[f"{name}.curvature"])
    np.testing.assert_allclose(a2, gold[f"{name}.a2"], rtol=1e-15, atol=0)
    a2 = gold[f"{name}.a2"]
    delta, u = gold[f"{name}.delta"], gold[f"{name}.u_probe"]
    psi = gold[f"{name}.psi_bl"][inner] + u[inner]
    lap = op.axisymmetric_laplacian if axi else op.laplacian
    lin = op.axisymmetric_linearized_hamiltonian_operator if axi else op.linearized_hamiltonian_operator
    res = op.axisymmetric_hamiltonian_residual if axi else op.hamiltonian_residual
    np.testing.assert_array_equal(lap(delta, dx), gold[f"{name}.laplacian"])
    np.testing.assert_array_equal(lin(delta, psi, a2[inner], dx), gold[f"{name}.linearized"])
    scale = np.abs(gold[f"{name}.residual"]).max()
    np.testing.assert_allclose(res(u, gold[f"{name}.psi_bl"], gold[f"{name}.curvature"], dx),
                               gold[f"{name}.residual"], rtol=0, atol=1e-15 * scale)
    np.testing.assert_array_equal(op.hamiltonian_source(psi, a2[inner]), gold[f"{name}.source"])
    np.testing.assert_array_equal(op.linearized_hamiltonian_source(delta, psi, a2[inner]),
                                  gold[f"{name}.linearized_source"])


@pytest.mark.parametrize("name", CASES)
def test_newton_solve(gold, name):
    case = _case(gold, name)
    grid, dx = gold[f"{name}.grid"], float(gold[f"{name}.dx"])
    tol, max_newton, lin_tol, max_lin = case["tol"]
    solve = op.solve_axisymmetric_conformal_factor if case["axi"] else op.solve_conformal_factor
    psi, u, history = solve(case["masses"], case["positions"], case["momenta"], grid, dx, tol, max_newton,
                            lin_tol, max_lin)
    ref_u = gold[f"{name}.u"]
    scale = max(np.abs(ref_u).max(), 1e-300)
    np.testing.assert_allclose(u, ref_u, rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(psi, gold[f"{name}.psi"], rtol=1e-14, atol=0)
    ref_h = gold[f"{name}.history"]
    assert len(history) == len(ref_h)
    np.testing.assert_allclose(history[0], ref_h[0], rtol=1e-13)
    assert history[-1] <= tol


def test_reference_known_answers():
    """tests/test_bowen_york.py:18-134 restated on the oracle."""
    grid, dx = op.axisymmetric_cell_centered_grid(8, 4.0)
    assert grid.shape == (8, 1, 16, 3) and dx == 0.5
    np.testing.assert_allclose(grid[0, 0, :, 2], -grid[0, 0, ::-1, 2])
    # the axisymmetric Laplacian is exact for rho^2 + z^2 away from the outer cells
    dx = 0.2
    rho = (np.arange(9) + 0.5) * dx
    z = -2.0 + (np.arange(1, 19) + 0.5) * dx
    R, Z = np.meshgrid(rho, z, indexing="ij")
    np.testing.assert_allclose(op.axisymmetric_laplacian(R ** 2 + Z ** 2, dx)[:-1, 1:-1], 6.0, atol=2e-13)
    # the Bowen-York curvature is symmetric and traceless, zero at zero momentum
    grid, _ = op.cell_centered_grid(8, 4.0)
    K = op.bowen_york_extrinsic_curvature([[0.2, -0.1, 0.5]], np.zeros((1, 3)), grid)
    np.testing.assert_allclose(K, np.swapaxes(K, -1, -2))
    np.testing.assert_allclose(np.trace(K, axis1=-2, axis2=-1), 0.0, atol=2e-14)
    np.testing.assert_array_equal(op.bowen_york_extrinsic_curvature(np.zeros((1, 3)), np.zeros((1, 3)), grid), 0.0)
    # zero momentum: u = 0 and psi = Brill-Lindquist exactly
    grid, dx = op.axisymmetric_cell_centered_grid(8, 4.0)
    psi, u, history = op.solve_axisymmetric_conformal_factor([1.0], np.zeros((1, 3)), np.zeros((1, 3)), grid, dx)
    np.testing.assert_array_equal(u, 0.0)
    np.testing.assert_allclose(psi, 1.0 + 0.5 / np.sqrt(np.sum(grid ** 2, axis=-1)))
    assert history == [0.0]
