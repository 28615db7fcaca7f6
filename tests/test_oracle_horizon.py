"""The apparent-horizon oracle against the reference suite's analytic answers.

JAX is absent, so the reference finder cannot run here; its own tests pin
the answers (tests/test_apparent_horizon.py): the Schwarzschild horizon mass
and coordinate radius in every storage layout, the pole stencil's order, the
spatial convergence of the mass and the failure modes.
"""

import numpy as np
import pytest

from oracle import horizon as H
from tests.horizon_cases import MASS, layout_case, schwarzschild_line


@pytest.mark.parametrize("layout", ["line", "plane"])
@pytest.mark.parametrize("slicing", ["isotropic", "kerr_schild"])
def test_oracle_exact_mass(layout, slicing):
    axes, gamma, kij, mass, exact = layout_case(layout, slicing)
    h = H.find_apparent_horizon(axes, gamma, kij, center=(0, 0, 0), initial_radius=1.15 * exact, n_theta=6,
                                n_phi=12, max_angular=24)
    np.testing.assert_allclose(h["mass"], mass, rtol=1.e-3)
    np.testing.assert_allclose(h["radius"], exact, atol=.002)
    assert h["residual"] < 1.e-8
    assert h["audit_residual"] < 1.e-4
    assert len(h["convergence"]) >= 2


def test_oracle_spatial_convergence():
    errors = []
    for dx in (.12, .06):
        r, gamma, kij = schwarzschild_line(dx=dx)
        h = H.find_apparent_horizon((r,), gamma, kij, center=(0, 0, 0), initial_radius=1.1, n_theta=6, n_phi=12,
                                    max_angular=12)
        errors.append(abs(h["mass"] - MASS))
    assert errors[1] < errors[0] / 4


def test_oracle_pole_stencil_order():
    errors = []
    for n in (12, 24):
        theta, phi, _ = H.angular_grid(n, 2 * n)
        field = np.sin(theta[:, None]) * np.cos(phi[None, :])
        dt, dtt, dp, dpp, dtp = H.angular_derivatives(field)
        errors.append(float(np.max(np.abs(dt - np.cos(theta[:, None]) * np.cos(phi[None, :])))))
        np.testing.assert_allclose(dpp, -field, atol=.001)
    assert errors[1] < errors[0] / 12


def test_oracle_jacobian_matches_finite_difference():
    r, gamma, kij = schwarzschild_line()
    sample = H.build_geometry((r,), gamma, kij)
    theta, phi, _ = H.angular_grid(6, 12)
    h = 1.1 + .03 * np.sin(theta[:, None]) ** 2 * np.cos(2 * phi[None, :])
    jac = H.jacobian(h, np.zeros(3), sample)
    direction = np.random.default_rng(4).normal(size=h.shape)
    eps = 1.e-6

    def residual(x):
        return H.surface(x, np.zeros(3), sample)[0].reshape(-1)
    fd = (residual(h + eps * direction) - residual(h - eps * direction)) / (2 * eps)
    np.testing.assert_allclose(jac @ direction.reshape(-1), fd, rtol=1.e-6, atol=1.e-8)


def test_oracle_failures():
    r, gamma, kij = schwarzschild_line()
    flat = np.broadcast_to(np.eye(3)[:, :, None], gamma.shape)
    with pytest.raises(RuntimeError, match="Newton"):
        H.find_apparent_horizon((r,), flat, kij, center=(0, 0, 0), initial_radius=1., n_theta=6, n_phi=12,
                                max_angular=12, max_iterations=2)
    with pytest.raises(RuntimeError, match="resolved domain"):
        H.find_apparent_horizon((r,), gamma, kij, center=(0, 0, 0), initial_radius=20.)
    bad = gamma.copy()
    bad[0, 0] *= -1
    with pytest.raises(RuntimeError, match="nonphysical"):
        H.find_apparent_horizon((r,), bad, kij, center=(0, 0, 0), initial_radius=1.)


# ---------------------------------------------------------------------------
# against the reference's own finder code (tests/golden/horizon.npz, made by
# tests/golden/make_golden.py running JAX_BSSN/utilities/apparent_horizon.py
# unmodified under the NumPy jax stand-in; its jacfwd is a Richardson
# difference good to about 1e-11)
# ---------------------------------------------------------------------------

def _golden():
    from tests.helpers import GOLDEN
    with np.load(GOLDEN / "horizon.npz") as data:
        return {k: data[k] for k in data.files}


@pytest.mark.parametrize("layout", ["line", "plane", "volume"])
def test_oracle_sample_and_surface_match_reference_code(layout):
    import json
    data = _golden()
    grid = json.loads(str(data["grid"]))
    axes, gamma, kij, _, _ = layout_case(layout, "kerr_schild", **grid)
    g, dg, k, valid = H.build_geometry(axes, gamma, kij)(data["sample.points"])
    ovalid = data[f"sample.{layout}.valid"].astype(bool)
    np.testing.assert_array_equal(np.asarray(valid).astype(bool), ovalid)
    for got, key, tol in ((g, "gamma", 1e-12), (dg, "d_gamma", 1e-9), (k, "curvature", 1e-12)):
        want = data[f"sample.{layout}.{key}"]
        np.testing.assert_allclose(np.asarray(got)[ovalid], want[ovalid], rtol=0,
                                   atol=tol * np.max(np.abs(want[ovalid])), err_msg=key)
    for slicing in ("isotropic", "kerr_schild"):
        axes, gamma, kij, _, _ = layout_case(layout, slicing, **grid)
        key = f"surface.{layout}_{slicing}"
        exp, dens, usable = H.surface(data[f"{key}.radius"], data[f"{key}.center"], H.build_geometry(axes, gamma, kij))
        assert bool(usable) == bool(data[f"{key}.usable"])
        want = data[f"{key}.expansion"]
        np.testing.assert_allclose(exp, want, rtol=0, atol=1e-8 * np.max(np.abs(want)) + 1e-12)
        np.testing.assert_allclose(dens, data[f"{key}.density"], rtol=1e-12)


def test_oracle_angular_operators_match_reference_code():
    data = _golden()
    field = data["angular.field"]
    for k, got in enumerate(H.angular_derivatives(field)):
        want = data[f"angular.derivative{k}"]
        np.testing.assert_allclose(got, want, rtol=1e-15, atol=1e-15 * np.max(np.abs(want)))
    theta, phi, _ = H.angular_grid(22, 42)
    np.testing.assert_allclose(H.interpolate_angular(field, theta, phi), data["angular.regrid"], rtol=1e-14)


@pytest.mark.parametrize("slicing", ["isotropic", "kerr_schild"])
def test_oracle_find_matches_reference_finder(slicing):
    import json
    data = _golden()
    grid = json.loads(str(data["grid"]))
    options = json.loads(str(data["find_options"]))
    axes, gamma, kij, _, exact = layout_case("line", slicing, **grid)
    key = f"find.line_{slicing}"
    h = H.find_apparent_horizon(axes, gamma, kij, center=(0, 0, 0), initial_radius=float(data[f"{key}.guess"]) * exact,
                                **options)
    assert h["radius"].shape == data[f"{key}.radius"].shape
    assert np.max(np.abs(h["radius"] - data[f"{key}.radius"])) < 1e-7 * exact
    assert abs(h["mass"] / float(data[f"{key}.mass"]) - 1) < 1e-7
