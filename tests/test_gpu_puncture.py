"""Bowen-York puncture data on the GPU against the reference's goldens, the
oracle and the reference suite's known answers (tests/test_bowen_york.py).

Setup fields and operators follow the reference's operation order: they agree
with the goldens to an ulp (the golden's radii come from an einsum whose
summation order differs; its integer powers from the C library's pow).  The
Newton-Krylov solves agree to the accuracy the tolerances ask for: the
Krylov iterates differ from SciPy's by rounding, so the corrections agree to
about the linear tolerance times the operator's condition, and the final
residual of each solve is checked on its own.
"""

import json

import numpy as np
import pytest
import torch

from oracle import puncture as op

from .helpers import load_golden

pytestmark = pytest.mark.gpu

CASES = ("cart_single", "cart_binary", "axi_single", "axi_binary", "axi_zero")


@pytest.fixture(scope="module")
def gold():
    return load_golden("puncture")


@pytest.fixture(scope="module")
def by(cuda, native):
    from jax_bssn_gb300.utilities import bowen_york_solver
    return bowen_york_solver


def _case(gold, name):
    return json.loads(str(gold[f"{name}.case"]))


def _np(x):
    return x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)


@pytest.mark.parametrize("name", CASES)
def test_grids_and_fields(by, gold, name):
    case = _case(gold, name)
    n, extent = case["grid"]
    grid, dx = (by.axisymmetric_cell_centered_grid if case["axi"] else by.cell_centered_grid)(n, extent)
    np.testing.assert_array_equal(_np(grid), gold[f"{name}.grid"])
    assert dx == float(gold[f"{name}.dx"])
    psi_bl = by.brill_lindquist_conformal_factor(case["masses"], case["positions"], grid)
    np.testing.assert_allclose(_np(psi_bl), gold[f"{name}.psi_bl"], rtol=5e-16, atol=0)
    # bit-identical to the oracle, whose radii sum the squares left to right
    np.testing.assert_array_equal(_np(psi_bl), op.brill_lindquist_conformal_factor(
        case["masses"], case["positions"], gold[f"{name}.grid"]))
    K = _np(by.bowen_york_extrinsic_curvature(case["momenta"], case["positions"], grid))
    ref = gold[f"{name}.curvature"]
    np.testing.assert_allclose(K, ref, rtol=0, atol=1e-15 * max(np.abs(ref).max(), 1e-300))
    np.testing.assert_array_equal(K, op.bowen_york_extrinsic_curvature(case["momenta"], case["positions"],
                                                                       gold[f"{name}.grid"]))


@pytest.mark.parametrize("name", ["cart_binary", "axi_binary"])
def test_operators(by, gold, name):
    dx = float(gold[f"{name}.dx"])
    axi = name.startswith("axi")
    inner = (slice(None, -1), 0, slice(1, -1)) if axi else (slice(1, -1),) * 3
    a2 = gold[f"{name}.a2"]
    np.testing.assert_array_equal(_np(by.contract_conformal_curvature(torch.as_tensor(
        gold[f"{name}.curvature"], device="cuda"))), op.contract_conformal_curvature(gold[f"{name}.curvature"]))
    delta, u = gold[f"{name}.delta"], gold[f"{name}.u_probe"]
    psi = gold[f"{name}.psi_bl"][inner] + u[inner]
    lap = by.axisymmetric_laplacian if axi else by.laplacian
    lin = by.axisymmetric_linearized_hamiltonian_operator if axi else by.linearized_hamiltonian_operator
    res = by.axisymmetric_hamiltonian_residual if axi else by.hamiltonian_residual
    # the Laplacians are bit-identical to the reference's
    np.testing.assert_array_equal(lap(delta, dx), gold[f"{name}.laplacian"])

    def close(got, want):
        scale = np.abs(want).max()
        np.testing.assert_allclose(got, want, rtol=0, atol=2e-15 * scale)
    close(lin(delta, psi, a2[inner], dx), gold[f"{name}.linearized"])
    close(res(u, gold[f"{name}.psi_bl"], gold[f"{name}.curvature"], dx), gold[f"{name}.residual"])
    close(by.hamiltonian_source(psi, a2[inner]), gold[f"{name}.source"])
    close(by.linearized_hamiltonian_source(delta, psi, a2[inner]), gold[f"{name}.linearized_source"])


def _solve(by, case, grid, dx):
    tol, max_newton, lin_tol, max_lin = case["tol"]
    return by.puncture_solve(case["masses"], case["positions"], case["momenta"], grid, dx, axisymmetric=case["axi"],
                             newton_tolerance=tol, max_newton_iterations=max_newton, linear_tolerance=lin_tol,
                             max_linear_iterations=max_lin)


@pytest.mark.parametrize("name", CASES)
def test_newton_solve_against_reference(by, gold, name):
    case = _case(gold, name)
    grid = torch.as_tensor(gold[f"{name}.grid"], device="cuda")
    dx = float(gold[f"{name}.dx"])
    r = _solve(by, case, grid, dx)
    u, psi = _np(r.u), _np(r.psi)
    ref_u, ref_h = gold[f"{name}.u"], gold[f"{name}.history"]
    scale = max(np.abs(ref_u).max(), 1e-300)
    err = np.abs(u - ref_u).max() / scale
    print(name, "u rel err", f"{err:.2e}", "history", r.residual_history, "krylov", r.linear_iterations)
    assert len(r.residual_history) == len(ref_h)
    np.testing.assert_allclose(r.residual_history[0], ref_h[0], rtol=1e-13)
    assert r.residual_history[-1] <= case["tol"][0]
    assert err < 1e-8
    np.testing.assert_allclose(psi, gold[f"{name}.psi"], rtol=1e-10, atol=0)
    # the outer cells carry no correction
    if case["axi"]:
        for face in (u[-1], u[:, :, 0], u[:, :, -1]):
            np.testing.assert_array_equal(face, 0.0)
    else:
        for face in (u[0], u[-1], u[:, 0], u[:, -1], u[:, :, 0], u[:, :, -1]):
            np.testing.assert_array_equal(face, 0.0)
    # the returned psi satisfies the discrete constraint on its own
    resid = (op.axisymmetric_hamiltonian_residual if case["axi"] else op.hamiltonian_residual)(
        u, gold[f"{name}.psi_bl"], gold[f"{name}.curvature"], dx)
    assert np.sqrt(np.mean(resid ** 2)) <= 10 * case["tol"][0]


def test_solve_is_deterministic(by, gold):
    case = _case(gold, "cart_binary")
    grid = torch.as_tensor(gold["cart_binary.grid"], device="cuda")
    a = _solve(by, case, grid, float(gold["cart_binary.dx"]))
    b = _solve(by, case, grid, float(gold["cart_binary.dx"]))
    assert torch.equal(a.u.view(torch.int64), b.u.view(torch.int64))
    assert a.residual_history == b.residual_history and a.linear_iterations == b.linear_iterations


@pytest.mark.parametrize("shape", [(12, 17, 23), (35, 9, 40)])
def test_non_cubic_grid_against_oracle(by, shape):
    """Tile edges of the conjugate-gradient operator on ragged extents."""
    dx = 0.4
    axes = [(np.arange(n) + 0.5) * dx - 0.5 * n * dx for n in shape]
    grid_np = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1)
    masses, positions, momenta = [0.6, 0.3], [[0.11, -0.07, -0.93], [-0.05, 0.09, 0.87]], [[0.05, 0.1, -0.2],
                                                                                         [0.0, -0.1, 0.1]]
    psi, u, hist = by.solve_conformal_factor(masses, positions, momenta, torch.as_tensor(grid_np, device="cuda"), dx)
    rpsi, ru, rhist = op.solve_conformal_factor(masses, positions, momenta, grid_np, dx)
    assert len(hist) == len(rhist) and hist[-1] <= 1e-10
    err = np.abs(_np(u) - ru).max() / np.abs(ru).max()
    print(shape, "u rel err", f"{err:.2e}", hist)
    assert err < 1e-8


def test_default_grid_binary_against_oracle(by):
    """The reference's default 48^3 cell-centred grid, a boosted binary."""
    grid, dx = by.cell_centered_grid()
    masses, positions, momenta = [0.5, 0.5], [[0.0, 0.0, -1.5], [0.0, 0.0, 1.5]], [[0.2, 0.0, 0.0], [-0.2, 0.0, 0.0]]
    r = by.puncture_solve(masses, positions, momenta, grid, dx, axisymmetric=False, newton_tolerance=1e-10,
                          max_newton_iterations=12, linear_tolerance=1e-10, max_linear_iterations=1000)
    rpsi, ru, rhist = op.solve_conformal_factor(masses, positions, momenta, _np(grid), dx)
    err = np.abs(_np(r.u) - ru).max() / np.abs(ru).max()
    print("48^3 u rel err", f"{err:.2e}", r.residual_history, r.linear_iterations)
    assert len(r.residual_history) == len(rhist) and r.residual_history[-1] <= 1e-10
    assert err < 1e-8


# --- the reference suite's known answers (tests/test_bowen_york.py) ---------

def test_axisymmetric_grid(by):
    grid, dx = by.axisymmetric_cell_centered_grid(num_radial_points=8, radial_extent=4.0)
    g = _np(grid)
    assert g.shape == (8, 1, 16, 3) and dx == 0.5
    np.testing.assert_allclose(g[:, 0, 0, 0], (np.arange(8) + 0.5) * dx)
    np.testing.assert_allclose(g[..., 1], 0.0)
    np.testing.assert_allclose(g[0, 0, :, 2], -g[0, 0, ::-1, 2])


def test_axisymmetric_laplacian_exact_for_quadratic(by):
    dx = 0.2
    rho = (np.arange(9) + 0.5) * dx
    z = -2.0 + (np.arange(1, 19) + 0.5) * dx
    R, Z = np.meshgrid(rho, z, indexing="ij")
    np.testing.assert_allclose(by.axisymmetric_laplacian(R ** 2 + Z ** 2, dx)[:-1, 1:-1], 6.0, atol=2.0e-13)


def test_curvature_symmetric_traceless_zero_at_zero_momentum(by):
    grid, _ = by.cell_centered_grid(num_points=8, half_width=4.0)
    K = _np(by.bowen_york_extrinsic_curvature([[0.2, -0.1, 0.5]], np.zeros((1, 3)), grid))
    np.testing.assert_allclose(K, np.swapaxes(K, -1, -2))
    np.testing.assert_allclose(np.trace(K, axis1=-2, axis2=-1), 0.0, atol=2.0e-14)
    np.testing.assert_array_equal(_np(by.bowen_york_extrinsic_curvature(np.zeros((1, 3)), np.zeros((1, 3)), grid)),
                                  0.0)


def test_axisymmetric_zero_momentum_is_brill_lindquist(by):
    grid, dx = by.axisymmetric_cell_centered_grid(8, 4.0)
    psi, u, history = by.solve_axisymmetric_conformal_factor([1.0], np.zeros((1, 3)), np.zeros((1, 3)), grid, dx)
    g = _np(grid)
    np.testing.assert_array_equal(_np(u), 0.0)
    np.testing.assert_allclose(_np(psi), 1.0 + 0.5 / np.sqrt(np.sum(g ** 2, axis=-1)))
    assert history == [0.0]


@pytest.mark.parametrize(("positions", "momenta", "message"), [
    ([[0.1, 0.0, 0.0]], [[0.0, 0.0, 0.2]], "z axis"),
    ([[0.0, 0.0, 0.0]], [[0.1, 0.0, 0.2]], "parallel to z"),
])
def test_axisymmetric_rejects_nonaxisymmetric_punctures(by, positions, momenta, message):
    grid, dx = by.axisymmetric_cell_centered_grid(8, 4.0)
    with pytest.raises(ValueError, match=message):
        by.solve_axisymmetric_conformal_factor(masses=[1.0], positions=positions, momenta=momenta, grid=grid, dx=dx)


def test_newton_not_converged_raises(by):
    grid, dx = by.cell_centered_grid(num_points=10, half_width=5.0)
    with pytest.raises(RuntimeError, match="did not converge"):
        by.solve_conformal_factor([1.0], np.zeros((1, 3)), [[0.0, 0.0, 0.2]], grid, dx, max_newton_iterations=0)
    with pytest.raises(RuntimeError, match="did not converge"):
        by.solve_axisymmetric_conformal_factor([1.0], np.zeros((1, 3)), [[0.0, 0.0, 0.2]],
                                               by.axisymmetric_cell_centered_grid(8, 4.0)[0], 0.5,
                                               max_newton_iterations=1, max_linear_iterations=1)


@pytest.mark.parametrize("name", ["cart_binary", "axi_binary"])
def test_graph_replay_equals_direct_launches(by, gold, native, name):
    """Krylov chunks replayed as a CUDA graph give the bits of direct launches
    (per-kernel profiling launches them directly)."""
    case = _case(gold, name)
    grid = torch.as_tensor(gold[f"{name}.grid"], device="cuda")
    dx = float(gold[f"{name}.dx"])
    graphed = _solve(by, case, grid, dx)
    native.bssn_profile_reset()
    native.bssn_profile_enable(1)
    try:
        direct = _solve(by, case, grid, dx)
    finally:
        torch.cuda.synchronize()
        native.bssn_profile_enable(0)
        native.bssn_profile_reset()
    assert torch.equal(graphed.u.view(torch.int64), direct.u.view(torch.int64))
    assert graphed.residual_history == direct.residual_history
    assert graphed.linear_iterations == direct.linear_iterations


def test_smallest_grids(by, gold):
    """One unknown on the Cartesian (3^3) and the meridional (2 x 1 x 3) grid:
    the operator kernels' tiles and the fixed cells around a single cell."""
    masses, positions, momenta = [0.4], [[0.05, -0.02, 0.11]], [[0.1, 0.0, 0.2]]
    axes = [(np.arange(3) + 0.5) * 0.7 - 1.05] * 3
    grid = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1)
    psi, u, hist = by.solve_conformal_factor(masses, positions, momenta, torch.as_tensor(grid, device="cuda"), 0.7)
    rpsi, ru, rhist = op.solve_conformal_factor(masses, positions, momenta, grid, 0.7)
    assert len(hist) == len(rhist)
    np.testing.assert_allclose(_np(u), ru, rtol=0, atol=1e-12 * max(np.abs(ru).max(), 1e-300))
    agrid, adx = by.axisymmetric_cell_centered_grid(2, 1.0)
    assert tuple(agrid.shape) == (2, 1, 4, 3)
    psi, u, hist = by.solve_axisymmetric_conformal_factor([0.5], [[0.0, 0.0, 0.1]], [[0.0, 0.0, 0.3]], agrid, adx)
    rpsi, ru, rhist = op.solve_axisymmetric_conformal_factor([0.5], [[0.0, 0.0, 0.1]], [[0.0, 0.0, 0.3]],
                                                             _np(agrid), adx)
    assert len(hist) == len(rhist)
    np.testing.assert_allclose(_np(u), ru, rtol=0, atol=1e-12 * max(np.abs(ru).max(), 1e-300))


def test_cartesian_zero_momentum_is_brill_lindquist(by):
    grid, dx = by.cell_centered_grid(num_points=8, half_width=4.0)
    psi, u, history = by.solve_conformal_factor([1.0], np.zeros((1, 3)), np.zeros((1, 3)), grid, dx)
    np.testing.assert_array_equal(_np(u), 0.0)
    assert history == [0.0]


def test_invalid_inputs(by):
    grid, dx = by.cell_centered_grid(num_points=8, half_width=4.0)
    with pytest.raises(ValueError, match="punctures"):
        by.brill_lindquist_conformal_factor(np.ones(17), np.zeros((17, 3)), grid)
    with pytest.raises(ValueError, match="three cells"):
        by.solve_conformal_factor([1.0], np.zeros((1, 3)), np.zeros((1, 3)), grid[:2], dx)
    with pytest.raises(ValueError, match="share one shape"):
        by.hamiltonian_source(np.ones((3, 3, 3)), np.ones((3, 3, 4)))
