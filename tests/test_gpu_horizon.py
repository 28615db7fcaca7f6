"""The apparent-horizon finder on the GPU against the oracle and the reference
suite's analytic answers (tests/test_apparent_horizon.py).

Pieces computed in the reference's operation order (angular derivatives,
the angular regrid) agree with the oracle to an ulp; the geometry sampling and
the expansion to rounding of the interpolation sums (1e-12 relative); the
Jacobian, formed by central differences on both sides, to the rounding those
differences amplify (1e-6 of its scale); the band LU solve with the dense
solve of the same Jacobian to 1e-9.  Whole solves land on the same surface as
the oracle's to far below the Newton tolerance.
"""

import numpy as np
import pytest
import torch

from oracle import horizon as H

from .horizon_cases import MASS, layout_case, schwarzschild_line, schwarzschild_plane, schwarzschild_volume

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ah(cuda, native):
    from jax_bssn_gb300.utilities import apparent_horizon
    return apparent_horizon


def _wavy(n_theta, n_phi, base=1.1, amp=.03):
    theta, phi, _ = H.angular_grid(n_theta, n_phi)
    return base + amp * np.sin(theta[:, None]) ** 2 * np.cos(2 * phi[None, :])


# ---------------------------------------------------------------------------
# the reference suite's cases through the CUDA path
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("layout", ["line", "plane", "volume"])
@pytest.mark.parametrize("slicing", ["isotropic", "kerr_schild"])
def test_exact_mass_all_layouts(ah, layout, slicing):
    axes, gamma, kij, mass, exact = layout_case(layout, slicing)
    horizon = ah.find_apparent_horizon(axes, gamma, kij, center=(0, 0, 0), initial_radius=1.15 * exact, n_theta=6,
                                       n_phi=12, max_angular=24)
    np.testing.assert_allclose(horizon["mass"], mass, rtol=1.e-3)
    np.testing.assert_allclose(horizon["radius"], exact, atol=.002)
    assert horizon["radius"].shape[1] > 1
    assert horizon["residual"] < 1.e-8
    assert horizon["audit_residual"] < 1.e-4
    assert len(horizon["convergence"]) >= 2
    # the oracle lands on the same surface
    ref = H.find_apparent_horizon(axes, gamma, kij, center=(0, 0, 0), initial_radius=1.15 * exact, n_theta=6,
                                  n_phi=12, max_angular=24)
    assert horizon["radius"].shape == ref["radius"].shape
    np.testing.assert_allclose(horizon["radius"], ref["radius"], rtol=0, atol=2.e-7 * exact)
    np.testing.assert_allclose(horizon["mass"], ref["mass"], rtol=1.e-7)


def _horizon_golden():
    from .helpers import GOLDEN
    with np.load(GOLDEN / "horizon.npz") as data:
        return {k: data[k] for k in data.files}


# Pins from the reference's own finder code, run unmodified under the NumPy
# jax stand-in (tests/golden/make_golden.py, horizon section).  There the
# metric derivative (jax.jacfwd) is a Richardson-extrapolated difference of
# the piecewise-cubic Hermite interpolant, good to about 1e-11, hence the
# 1e-9 bounds on the derivative and the expansion; the rest is exact
# arithmetic in the reference's order.

@pytest.mark.parametrize("layout", ["line", "plane", "volume"])
def test_sample_matches_reference_code(ah, layout):
    """build_geometry / sample (JAX_BSSN/utilities/apparent_horizon.py:22-98)."""
    import json
    data = _horizon_golden()
    grid = json.loads(str(data["grid"]))
    axes, gamma, kij, _, _ = layout_case(layout, "kerr_schild", **grid)
    table, sample = ah.build_geometry(axes, gamma, kij)
    pts = data["sample.points"]
    g, dg, k, valid = (t.cpu().numpy() for t in sample(table, pts))
    ovalid = data[f"sample.{layout}.valid"].astype(bool)
    np.testing.assert_array_equal(valid.astype(bool), ovalid)
    for got, key, tol in ((g, "gamma", 1e-12), (dg, "d_gamma", 1e-9), (k, "curvature", 1e-12)):
        want = data[f"sample.{layout}.{key}"]
        scale = np.max(np.abs(want[ovalid]))
        np.testing.assert_allclose(got[ovalid], want[ovalid], rtol=0, atol=tol * scale, err_msg=key)


@pytest.mark.parametrize("layout", ["line", "plane", "volume"])
@pytest.mark.parametrize("slicing", ["isotropic", "kerr_schild"])
def test_surface_matches_reference_code(ah, layout, slicing):
    """surface (apparent_horizon.py:160-236): expansion and area density of a
    non-spherical surface about an off-axis centre."""
    import json
    data = _horizon_golden()
    grid = json.loads(str(data["grid"]))
    axes, gamma, kij, _, _ = layout_case(layout, slicing, **grid)
    table, _ = ah.build_geometry(axes, gamma, kij)
    key = f"surface.{layout}_{slicing}"
    exp, dens, usable = ah.surface(torch.as_tensor(data[f"{key}.radius"]).cuda(), data[f"{key}.center"], table)
    assert bool(usable) == bool(data[f"{key}.usable"])
    want = data[f"{key}.expansion"]
    np.testing.assert_allclose(exp.cpu().numpy(), want, rtol=0, atol=1e-8 * np.max(np.abs(want)) + 1e-12)
    np.testing.assert_allclose(dens.cpu().numpy(), data[f"{key}.density"], rtol=1e-12)


def test_angular_operators_match_reference_code(ah):
    """angular_derivatives (:125-144) and interpolate_angular (:147-157)."""
    data = _horizon_golden()
    field = data["angular.field"]
    got = [d.cpu().numpy() for d in ah.angular_derivatives(torch.as_tensor(field).cuda())]
    for k, g in enumerate(got):
        w = data[f"angular.derivative{k}"]
        np.testing.assert_allclose(g, w, rtol=1e-15, atol=1e-15 * np.max(np.abs(w)))
    theta, phi, _ = ah.angular_grid(22, 42)
    regrid = ah.interpolate_angular(torch.as_tensor(field).cuda(), theta, phi)
    regrid = regrid.cpu().numpy() if hasattr(regrid, "cpu") else np.asarray(regrid)
    np.testing.assert_allclose(regrid, data["angular.regrid"], rtol=1e-14)


@pytest.mark.parametrize("slicing", ["isotropic", "kerr_schild"])
def test_find_matches_reference_finder(ah, slicing):
    """Complete finds of the reference's find_apparent_horizon (:246-338) on
    the radial-line layout: 6 x 12, refined once to 12 x 24, Newton tolerance
    1e-9.  Both finders stop once mean(h) max|Theta| < 1e-9, so the surfaces
    agree to about that over |dTheta/dh|."""
    import json
    data = _horizon_golden()
    grid = json.loads(str(data["grid"]))
    options = json.loads(str(data["find_options"]))
    axes, gamma, kij, _, exact = layout_case("line", slicing, **grid)
    key = f"find.line_{slicing}"
    got = ah.find_apparent_horizon(axes, gamma, kij, center=(0, 0, 0),
                                   initial_radius=float(data[f"{key}.guess"]) * exact, **options)
    ref = data[f"{key}.radius"]
    assert got["radius"].shape == ref.shape
    err = float(np.max(np.abs(got["radius"] - ref))) / exact
    mass_err = abs(got["mass"] - float(data[f"{key}.mass"])) / float(data[f"{key}.mass"])
    print(slicing, f"radius {err:.1e} of r, mass {mass_err:.1e}")
    assert err < 1e-7
    assert mass_err < 1e-7
    np.testing.assert_allclose(np.asarray(got["convergence"])[:, 2], data[f"{key}.convergence"][:, 2], rtol=1e-7)


def test_nonspherical_guess_and_fixed_displaced_center(ah):
    center = (0., 0., .15)
    x, z, gamma, kij = schwarzschild_plane(stretch=1.3, center_z=center[2], dx=.03)
    theta, phi, _ = ah.angular_grid(12, 24)
    guess = 1.1 + .05 * np.sin(theta[:, None]) ** 2 * np.cos(2 * phi[None, :])
    h = ah.find_apparent_horizon((x, z), gamma, kij, center=center, initial_radius=guess)
    np.testing.assert_array_equal(h["center"], center)
    np.testing.assert_allclose(h["mass"], MASS, rtol=.002)
    norm = h["radius"] * np.sqrt(np.sin(h["theta"][:, None]) ** 2 + (1.3 * np.cos(h["theta"][:, None])) ** 2)
    np.testing.assert_allclose(norm, 1., atol=.003)
    assert "recenter_shift" not in h and "seed_radius" not in h


def test_triaxial_volume(ah):
    scale = (1., 1.25, 1.5)
    x, y, z, gamma, kij = schwarzschild_volume(dx=.04, scale=scale)
    h = ah.find_apparent_horizon((x, y, z), gamma, kij, center=(0, 0, 0), initial_radius=.9)
    theta, phi = h["theta"][:, None], h["phi"][None, :]
    norm = h["radius"] * np.sqrt((scale[0] * np.sin(theta) * np.cos(phi)) ** 2
                                 + (scale[1] * np.sin(theta) * np.sin(phi)) ** 2 + (scale[2] * np.cos(theta)) ** 2)
    np.testing.assert_allclose(norm, 1., atol=.003)
    np.testing.assert_allclose(h["mass"], MASS, rtol=.002)
    assert np.ptp(h["radius"], axis=1).max() > .1


def test_spatial_convergence(ah):
    errors = []
    for dx in (.12, .06):
        r, gamma, kij = schwarzschild_line(dx=dx)
        h = ah.find_apparent_horizon((r,), gamma, kij, center=(0, 0, 0), initial_radius=1.1, n_theta=6, n_phi=12,
                                     max_angular=12)
        errors.append(abs(h["mass"] - MASS))
    assert errors[1] < errors[0] / 4


def test_pole_stencil_and_angular_convergence(ah):
    errors = []
    for n in (12, 24):
        theta, phi, _ = ah.angular_grid(n, 2 * n)
        field = np.sin(theta[:, None]) * np.cos(phi[None, :])
        dt, dtt, dp, dpp, dtp = (d.cpu().numpy() for d in ah.angular_derivatives(torch.as_tensor(field).cuda()))
        errors.append(float(np.max(np.abs(dt - np.cos(theta[:, None]) * np.cos(phi[None, :])))))
        np.testing.assert_allclose(dpp, -field, atol=.001)
    assert errors[1] < errors[0] / 12


def test_dense_jacobian_matches_finite_difference(ah):
    r, gamma, kij = schwarzschild_line()
    table, sample = ah.build_geometry((r,), gamma, kij)
    h = torch.as_tensor(_wavy(6, 12)).cuda()
    residual = ah.ExpansionResidual(np.zeros(3), table)
    jacobian = ah.dense_jacobian(residual, h).cpu().numpy()
    direction = torch.as_tensor(np.random.default_rng(4).normal(size=h.shape)).cuda()
    eps = 1.e-6
    fd = ((residual(h + eps * direction) - residual(h - eps * direction)) / (2 * eps)).cpu().numpy()
    np.testing.assert_allclose(jacobian @ direction.cpu().numpy().reshape(-1), fd, rtol=1.e-6, atol=1.e-8)
    # a plain callable is differentiated column by column
    generic = ah.dense_jacobian(lambda q: residual(q), h).cpu().numpy()
    np.testing.assert_allclose(generic, jacobian, rtol=1.e-5, atol=1.e-7)


def test_residual_on_both_sides_of_spatial_cell_boundary(ah):
    r, gamma, kij = schwarzschild_line()
    table, sample = ah.build_geometry((r,), gamma, kij)
    residual = ah.ExpansionResidual(np.zeros(3), table)
    direction = torch.ones((6, 12), dtype=torch.float64, device="cuda")
    knot = r[55]
    for side in (-1., 1.):
        h = direction * (knot + side * 1.e-5)
        jac = ah.dense_jacobian(residual, h)
        derivative = (jac @ direction.reshape(-1)).cpu().numpy()
        eps = 1.e-7
        fd = ((residual(h + eps * direction) - residual(h - eps * direction)) / (2 * eps)).cpu().numpy()
        np.testing.assert_allclose(derivative, fd, rtol=1.e-5, atol=1.e-7)
    below = residual(direction * (knot - 1.e-7)).cpu().numpy()
    above = residual(direction * (knot + 1.e-7)).cpu().numpy()
    np.testing.assert_allclose(below, above, atol=1.e-6)


def test_failures_do_not_search_for_another_seed(ah):
    r, gamma, kij = schwarzschild_line()
    flat = np.broadcast_to(np.eye(3)[:, :, None], gamma.shape)
    with pytest.raises(RuntimeError, match="Newton"):
        ah.find_apparent_horizon((r,), flat, kij, center=(0, 0, 0), initial_radius=1., n_theta=6, n_phi=12,
                                 max_angular=12, max_iterations=2)
    with pytest.raises(RuntimeError, match="resolved domain"):
        ah.find_apparent_horizon((r,), gamma, kij, center=(0, 0, 0), initial_radius=20.)
    with pytest.raises(RuntimeError, match="Newton did not converge"):
        ah.find_apparent_horizon((r,), gamma, kij, center=(0, 0, 0), initial_radius=1.2, max_iterations=0)
    bad = gamma.copy()
    bad[0, 0] *= -1
    with pytest.raises(RuntimeError, match="nonphysical"):
        ah.find_apparent_horizon((r,), bad, kij, center=(0, 0, 0), initial_radius=1.)


@pytest.mark.parametrize("guess", [np.ones(12), np.ones((12, 13)), -1., np.full((6, 12), np.nan)])
def test_bad_initial_surface(ah, guess):
    r, gamma, kij = schwarzschild_line()
    with pytest.raises(ValueError):
        ah.find_apparent_horizon((r,), gamma, kij, center=(0, 0, 0), initial_radius=guess)


def test_center_and_guess_are_required(ah):
    r, gamma, kij = schwarzschild_line()
    with pytest.raises(TypeError):
        ah.find_apparent_horizon((r,), gamma, kij)


def test_geometry_validation(ah):
    r, gamma, kij = schwarzschild_line()
    with pytest.raises(ValueError, match="uniform axes"):
        ah.build_geometry((r[:8],), gamma[..., :8], kij[..., :8])
    with pytest.raises(ValueError, match="shape"):
        ah.build_geometry((r,), gamma[..., :-1], kij)
    skew = gamma.copy()
    skew[0, 1] += 1.e-3
    with pytest.raises(ValueError, match="symmetric"):
        ah.build_geometry((r,), skew, kij)
    off = gamma.copy()
    off[0, 1] = off[1, 0] = 1.e-3
    with pytest.raises(ValueError, match="diagonal"):
        ah.build_geometry((r,), off, kij)
    x, z, g2, k2 = schwarzschild_plane()
    with pytest.raises(ValueError, match="signed x-z plane"):
        ah.build_geometry((x - x[0] + 1., z), g2, k2)
    with pytest.raises(ValueError, match="margin"):
        ah.build_geometry((r,), gamma, kij, margin=1)


# ---------------------------------------------------------------------------
# parity of each piece with the oracle
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("layout", ["line", "plane", "volume"])
def test_sample_matches_oracle(ah, layout):
    axes, gamma, kij, _, _ = layout_case(layout, "kerr_schild", volume_dx=.1, volume_extent=3.)
    table, sample = ah.build_geometry(axes, gamma, kij)
    rng = np.random.default_rng(7)
    pts = rng.normal(size=(500, 3))
    pts *= (rng.uniform(1.2, 2.8, size=500) / np.linalg.norm(pts, axis=1))[:, None]
    pts[:5] = [[0, 0, 2.0], [2.0, 0, 0], [0, 2.0, 0], [1e-12, 0, 2.0], [0, 0, 40.0]]
    g, dg, k, valid = (t.cpu().numpy() for t in sample(table, pts))
    og, odg, ok, ovalid = H.build_geometry(axes, gamma, kij)(pts)
    np.testing.assert_array_equal(valid, ovalid)
    for got, want in ((g, og), (dg, odg), (k, ok)):
        scale = np.max(np.abs(want[ovalid]))
        np.testing.assert_allclose(got[ovalid], want[ovalid], rtol=0, atol=1.e-12 * scale)


def test_angular_derivatives_match_oracle(ah):
    field = _wavy(10, 20) + .01 * np.random.default_rng(3).normal(size=(10, 20))
    got = [d.cpu().numpy() for d in ah.angular_derivatives(torch.as_tensor(field).cuda())]
    for g, w in zip(got, H.angular_derivatives(field)):
        np.testing.assert_allclose(g, w, rtol=1.e-15, atol=1.e-15 * np.max(np.abs(w)))


@pytest.mark.parametrize("layout", ["line", "plane", "volume"])
@pytest.mark.parametrize("slicing", ["isotropic", "kerr_schild"])
def test_surface_matches_oracle(ah, layout, slicing):
    axes, gamma, kij, _, exact = layout_case(layout, slicing, volume_dx=.1, volume_extent=3.)
    table, sample = ah.build_geometry(axes, gamma, kij)
    h = _wavy(8, 16, base=1.1 * exact, amp=.03 * exact)
    center = np.array([0., 0., .02]) if layout != "line" else np.zeros(3)
    exp, dens, usable = ah.surface(torch.as_tensor(h).cuda(), center, table)
    oexp, odens, ousable = H.surface(h, center, H.build_geometry(axes, gamma, kij))
    assert usable and ousable
    np.testing.assert_allclose(exp.cpu().numpy(), oexp, rtol=0, atol=1.e-11 * np.max(np.abs(oexp)) + 1.e-12)
    np.testing.assert_allclose(dens.cpu().numpy(), odens, rtol=1.e-12)


@pytest.mark.parametrize("layout", ["line", "plane", "volume"])
def test_jacobian_matches_oracle(ah, layout):
    axes, gamma, kij, _, exact = layout_case(layout, "kerr_schild", volume_dx=.1, volume_extent=3.)
    table, _ = ah.build_geometry(axes, gamma, kij)
    h = _wavy(6, 12, base=1.1 * exact, amp=.03 * exact)
    center = np.zeros(3)
    got = ah.dense_jacobian(ah.ExpansionResidual(center, table), torch.as_tensor(h).cuda()).cpu().numpy()
    want = H.jacobian(h, center, H.build_geometry(axes, gamma, kij))
    np.testing.assert_allclose(got, want, rtol=0, atol=1.e-6 * np.max(np.abs(want)))
    pattern = np.eye(h.size, dtype=bool) | np.any(H._stencil_matrices(*h.shape) != 0, axis=0)
    assert not np.any(got[~pattern])


# (6, 126): band too wide for the panel kernel (column steps with the folded
# pivot search); (6, 130): too wide for those too (plain column steps);
# (6, 200): upper band too wide for the shared-memory back substitution
@pytest.mark.parametrize("shape", [(6, 12), (8, 16), (12, 24), (24, 48), (6, 126), (6, 130), (6, 200)])
def test_band_solve_matches_dense_solve(ah, shape):
    axes, gamma, kij, _, exact = layout_case("plane", "kerr_schild")
    table, _ = ah.build_geometry(axes, gamma, kij)
    h = torch.as_tensor(_wavy(*shape, base=1.1 * exact, amp=.05 * exact)).cuda()
    S = ah._Surfaces(table, np.array([0., 0., .03]), *shape)
    S.measure(h)
    largest, nonfinite = S.direction(h)
    assert nonfinite == 0
    jac = S.jacobian(h).cpu().numpy()
    want = np.linalg.solve(jac, -S.expansion.cpu().numpy().reshape(-1))
    got = S.delta.cpu().numpy().reshape(-1)
    np.testing.assert_allclose(got, want, rtol=0, atol=1.e-9 * np.max(np.abs(want)))
    assert largest == pytest.approx(np.max(np.abs(got)), rel=0, abs=0)


def test_regrid_matches_oracle(ah):
    radius = _wavy(12, 24) + .01 * np.random.default_rng(5).normal(size=(12, 24))
    for nt, nphi in ((26, 50), (24, 48), (7, 10)):
        theta, phi, _ = H.angular_grid(nt, nphi)
        got = ah.interpolate_angular(torch.as_tensor(radius).cuda(), theta, phi).cpu().numpy()
        np.testing.assert_allclose(got, H.interpolate_angular(radius, theta, phi), rtol=1.e-15, atol=0)


def test_surface_summary(ah):
    axes, gamma, kij, _, exact = layout_case("line", "isotropic")
    table, _ = ah.build_geometry(axes, gamma, kij)
    h = _wavy(12, 24, base=1.1 * exact, amp=.02 * exact)
    S = ah._Surfaces(table, np.zeros(3), 12, 24)
    total, peak, bad, area = S.measure(torch.as_tensor(h).cuda())
    exp, dens, _ = H.surface(h, np.zeros(3), H.build_geometry(axes, gamma, kij))
    _, _, weights = H.angular_grid(12, 24)
    assert bad == 0
    assert total == pytest.approx(h.sum(), rel=1.e-14)
    assert peak == pytest.approx(np.max(np.abs(exp)), rel=1.e-11)
    assert area == pytest.approx(float(np.sum(weights[:, None] * dens) * (2 * np.pi / 24)), rel=1.e-12)


def test_invalid_surfaces_raise(ah):
    dev = torch.device("cuda")
    with pytest.raises(ValueError, match="six nodes"):
        ah.angular_derivatives(torch.ones((5, 12), dtype=torch.float64, device=dev))
    with pytest.raises(ValueError, match="even n_phi"):
        ah.angular_derivatives(torch.ones((6, 13), dtype=torch.float64, device=dev))
    with pytest.raises(ValueError, match="output grid"):
        ah.interpolate_angular(torch.ones((6, 12), dtype=torch.float64, device=dev), np.zeros(0), np.zeros(3))
    r, gamma, kij = schwarzschild_line()
    table, _ = ah.build_geometry((r,), gamma, kij)
    with pytest.raises(ValueError, match="six nodes"):
        ah.surface(torch.ones((6, 7), dtype=torch.float64, device=dev), np.zeros(3), table)


def test_horizon_of_puncture_data_matches_oracle(ah):
    """Brill-Lindquist data from the GPU puncture kernels, physical metric
    psi^4 delta_ij and K = 0, searched about one of two punctures; the oracle
    runs the same finder on the oracle's own puncture data."""
    from jax_bssn_gb300.utilities import bowen_york_solver as by
    from oracle import puncture as op
    masses, positions = [0.5, 0.5], [[0.0, 0.0, -1.0], [0.0, 0.0, 1.0]]
    grid, dx = by.cell_centered_grid(96, 1.5)
    psi = by.brill_lindquist_conformal_factor(masses, positions, grid)
    gamma = psi[None, None] ** 4 * torch.eye(3, dtype=torch.float64, device=psi.device)[:, :, None, None, None]
    kij = torch.zeros_like(gamma)
    axis = grid[:, 0, 0, 0].cpu().numpy()
    # the horizon sits 8 cells from a 1/r puncture: the C1 geometry limits the
    # angular audit to a few 1e-4, so its tolerance is loosened
    options = dict(center=(0.0, 0.0, -1.0), initial_radius=0.3, n_theta=6, n_phi=12, max_angular=24,
                   audit_tolerance=2.e-3)
    got = ah.find_apparent_horizon((axis, axis, axis), gamma.contiguous(), kij, **options)
    hgrid, _ = op.cell_centered_grid(96, 1.5)
    hpsi = op.brill_lindquist_conformal_factor(masses, positions, hgrid)
    hgamma = hpsi[None, None] ** 4 * np.eye(3)[:, :, None, None, None]
    want = H.find_apparent_horizon((axis, axis, axis), hgamma, np.zeros_like(hgamma), **options)
    assert got["residual"] < 1.e-8 and got["audit_residual"] < 2.e-3
    assert got["radius"].shape == want["radius"].shape
    np.testing.assert_allclose(got["radius"], want["radius"], rtol=0, atol=1.e-7)
    np.testing.assert_allclose(got["mass"], want["mass"], rtol=1.e-7)
    # an isolated hole of mass 0.5 would have area mass 0.5 at coordinate radius 0.25;
    # the companion raises both a little
    assert 0.5 < got["mass"] < 0.6 and 0.2 < got["radius"].mean() < 0.35
