"""Generate golden vectors by running the unmodified reference (uwplasma/JAX_BSSN).

JAX is not installable in this environment, so the reference source is
imported with ``tests/golden/jaxshim`` -- a NumPy stand-in for the part of the
``jax`` API the hot path uses (``jit`` = identity, ``lax.cond`` = Python
branch, single-device collectives) -- placed first on ``sys.path``.  Under it
the reference's own derivative, boundary, FMR and Cartoon test suites pass.

Usage (needs the reference checkout; the GPU machine does not have it):
    python tests/golden/make_golden.py [/path/to/reference] [--no-long] [--only=rhs,...]

Outputs ``tests/golden/*.npz``; each archive stores the inputs, the
parameters (as a JSON string) and the reference outputs.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def _setup(reference: Path):
    sys.path.insert(0, str(HERE / "jaxshim"))
    sys.path.insert(0, str(reference))
    sys.path.insert(0, str(REPO))


def _params_json(params) -> str:
    d = params._asdict()
    return json.dumps({k: (list(v) if isinstance(v, tuple) else v) for k, v in d.items()})


LEAF_NAMES = ("conformal_metric", "conformal_factor", "traceless_K", "trace_K",
              "conformal_connection", "lapse", "shift")


def _state_arrays(prefix, state):
    names = ("conformal_metric", "conformal_factor", "traceless_K", "trace_K",
             "conformal_connection", "lapse", "shift")
    return {f"{prefix}.{n}": np.asarray(v, dtype=np.float64) for n, v in zip(names, state)}


def make_stencils(out: Path):
    from JAX_BSSN.evolution.derivatives import diff1_field, diff1_upwind_field, diff2_field, diff6_field
    rng = np.random.default_rng(814)
    shape = (12, 10, 14)
    f = rng.normal(size=shape)
    coef = rng.normal(size=shape)
    coef[rng.random(shape) < 0.2] = 0.0
    dx = 0.17
    data = {"field": f, "coefficient": coef, "dx": np.float64(dx)}
    cases = {"periodic": (0, 0), "sommerfeld": (1, 1), "left": (1, 0), "right": (0, 1)}
    for cname, (lbc, rbc) in cases.items():
        for q in (1.0, 1.0 / 16.0):
            for axis in range(3):
                key = f"{cname}.q{q:g}.axis{axis}"
                data[f"d1.{key}"] = np.asarray(diff1_field(f, axis, dx, lbc, rbc, mad_q=q))
                data[f"d2.{key}"] = np.asarray(diff2_field(f, axis, dx, lbc, rbc, mad_q=q))
                data[f"up.{key}"] = np.asarray(diff1_upwind_field(f, coef, axis, dx, lbc, rbc, mad_q=q))
                if q == 1.0:
                    data[f"d6.{key}"] = np.asarray(diff6_field(f, axis, dx, lbc, rbc))
    np.savez_compressed(out, **data)


def rhs_cases():
    from jax_bssn_gb300.initial_data import gauge_wave_config, random_smooth_state
    from JAX_BSSN.bssn.variables import BSSNParameters as P
    cases = {}
    state, params = gauge_wave_config(n=12, nu=0.1)
    cases["gauge_wave"] = (state, P(**params._asdict()))
    smooth = random_smooth_state((10, 10, 10), seed=3)
    cases["generic_kappa"] = (smooth, P(eta=2.0, kappa=0.3, nu=0.05, g=0.75, dx=0.1, dt=0.02,
                                         gauge=1, zero_shift=0, x_min=-0.4, y_min=0.1, z_min=0.3))
    cases["sommerfeld"] = (random_smooth_state((10, 9, 11), seed=5),
                           P(eta=1.0, kappa=0.0, nu=0.02, g=0.75, dx=0.1, dt=0.02, gauge=1,
                             xl_bc=1, xr_bc=1, yl_bc=1, yr_bc=1, zl_bc=1, zr_bc=1,
                             x_min=-0.45, y_min=-0.4, z_min=-0.5))
    cases["mad_mixed"] = (random_smooth_state((10, 10, 10), seed=7),
                          P(eta=1.0, kappa=0.1, nu=0.02, g=0.75, dx=0.1, dt=0.02, gauge=0,
                            mad_q=1.0 / 16.0, xl_bc=1, xr_bc=0, x_min=-0.3, y_min=0.2, z_min=-0.1))
    cases["mad_periodic_zero_shift"] = (random_smooth_state((10, 10, 10), seed=9, shift=False),
                                        P(eta=1.0, kappa=0.0, nu=0.02, g=0.75, dx=0.1, dt=0.02, gauge=0,
                                          mad_q=1.0 / 16.0, zero_shift=1))
    # A 1e-6 wave on the flat background carried by a uniform O(1) shift, with
    # no shift damping: the advection of the unit-background fields dominates
    # their RHS, and the shift's own RHS is as small as the wave, so the
    # numerators of every field with a constant background (diagonal metric,
    # W, alpha and the shift) must round as the reference's do.
    weak = random_smooth_state((12, 11, 10), seed=11, amplitude=1e-6)
    beta = np.asarray(weak.shift) + np.array([0.5, -0.3, 0.2])[:, None, None, None]
    cases["boosted_weak_wave"] = (weak._replace(shift=beta),
                                  P(eta=0.0, kappa=0.0, nu=0.02, g=0.75, dx=0.1, dt=0.02, gauge=1,
                                    x_min=-0.55, y_min=-0.5, z_min=-0.45))
    return cases


def make_rhs(out_dir: Path):
    from JAX_BSSN.evolution.time_evolve import compute_bssn_rhs, rk4_step, enforce_algebraic_constraints
    from JAX_BSSN.bssn.constraints import compute_all_constraints
    for name, (state, params) in rhs_cases().items():
        data = {"params": np.asarray(_params_json(params))}
        data.update(_state_arrays("input", state))
        data.update(_state_arrays("rhs", compute_bssn_rhs(state, params)))
        data.update(_state_arrays("project", enforce_algebraic_constraints(state)))
        step = rk4_step(state, params)
        data.update(_state_arrays("rk4_1", step))
        data.update(_state_arrays("rk4_2", rk4_step(step, params)))
        c = compute_all_constraints(state, params)
        for field in c._fields:
            data[f"constraints.{field}"] = np.asarray(getattr(c, field))
        np.savez_compressed(out_dir / f"rhs_{name}.npz", **data)


def make_long_runs(out_dir: Path):
    """Multi-step reference runs on the headline parity workloads."""
    from JAX_BSSN.evolution.time_evolve import rk4_step
    from JAX_BSSN.bssn.variables import BSSNParameters as P
    from jax_bssn_gb300.initial_data import gauge_wave_config, teukolsky_config
    # 32^3 periodic gauge wave, A=0.1, harmonic, zero shift, CFL 0.25, nu=0.1: 1 and 100 steps
    state, params = gauge_wave_config(n=32, nu=0.1)
    params = P(**params._asdict())
    data = {"params": np.asarray(_params_json(params))}
    data.update(_state_arrays("input", state))
    for n in range(1, 101):
        state = rk4_step(state, params)
        if n in (1, 10, 100):
            data.update(_state_arrays(f"rk4_{n}", state))
    np.savez_compressed(out_dir / "run_gauge_wave32.npz", **data)
    # linearised Teukolsky wave on 24^3 (Sommerfeld, 1+log, Gamma-driver): 1 and 10 steps
    state, params = teukolsky_config(n=24)
    params = P(**params._asdict())
    data = {"params": np.asarray(_params_json(params))}
    data.update(_state_arrays("input", state))
    for n in range(1, 11):
        state = rk4_step(state, params)
        if n in (1, 10):
            data.update(_state_arrays(f"rk4_{n}", state))
    np.savez_compressed(out_dir / "run_teukolsky24.npz", **data)


def _owned_arrays(prefix, states, guard_first=0):
    """Owned samples of tiled states (tile axes dropped)."""
    out = {}
    for patch, state in enumerate(states):
        for name, leaf in zip(LEAF_NAMES, state):
            a = np.asarray(leaf)
            a = a.reshape(a.shape[:-6] + a.shape[-3:])
            g = 4
            out[f"{prefix}.{patch}.{name}"] = a[..., g:-g, g:-g, g:-g]
    return out


def _padded_arrays(prefix, state, patch):
    out = {}
    for name, leaf in zip(LEAF_NAMES, state):
        a = np.asarray(leaf)
        out[f"{prefix}.{patch}.{name}"] = a.reshape(a.shape[:-6] + a.shape[-3:])
    return out


def fmr_cases():
    from JAX_BSSN.bssn.variables import BSSNParameters as P, BSSNVariables as V
    from JAX_BSSN.fmr import FMRHierarchySpec, FMRPatchSpec
    from jax_bssn_gb300.initial_data import gauge_wave_state

    def smooth(coordinates, params):
        x, y, z = np.broadcast_arrays(*[np.asarray(c) for c in coordinates])
        phase = x + 0.03 * np.sin(2 * np.pi * y) * np.cos(2 * np.pi * z)
        state = gauge_wave_state(phase, y, z, amplitude=0.01)
        shift = np.stack((0.1 + 0.01 * np.sin(2 * np.pi * y), -0.05 + 0.005 * np.cos(2 * np.pi * z),
                          0.025 + 0.003 * np.sin(2 * np.pi * x)))
        return V(*state[:-1], shift)

    cases = {}
    cases["three_level_mad"] = (smooth, P(dx=1 / 12, dt=0.0005, eta=0.0, g=0.0, nu=0.005,
                                          x_min=-0.5, y_min=-0.5, z_min=-0.5), (12, 12, 12),
                                FMRHierarchySpec((FMRPatchSpec((3,) * 3, (8,) * 3), FMRPatchSpec((2,) * 3, (4,) * 3))))
    cases["sommerfeld_kappa"] = (smooth, P(dx=1 / 14, dt=0.001, eta=1.0, g=0.75, nu=0.02, kappa=0.1, gauge=1,
                                           xl_bc=1, xr_bc=1, yl_bc=1, yr_bc=1, zl_bc=1, zr_bc=1,
                                           x_min=-0.45, y_min=-0.45, z_min=-0.45), (14, 14, 14),
                                 FMRHierarchySpec((FMRPatchSpec((5,) * 3, (8,) * 3),)))
    cases["siblings_no_mad"] = (smooth, P(dx=1 / 12, dt=0.0005, eta=0.5, g=0.5, nu=0.01,
                                          x_min=-0.5, y_min=-0.5, z_min=-0.5), (12, 12, 12),
                                FMRHierarchySpec((FMRPatchSpec((2,) * 3, (4,) * 3),
                                                  FMRPatchSpec((6, 2, 3), (9, 5, 6), parent=0)), use_mad=False))
    return cases


def make_fmr(out_dir: Path):
    from JAX_BSSN.fmr import initialize_tiled_fmr, fmr_stage, fmr_rk4_step, fmr_constraint_norms
    for name, (initial, params, shape, hierarchy) in fmr_cases().items():
        states, parameters, layouts = initialize_tiled_fmr(initial, params, shape, hierarchy)
        data = {"hierarchy": np.asarray(json.dumps({
            "patches": [[list(s.coarse_lo), list(s.coarse_hi), s.parent] for s in hierarchy.patches],
            "use_mad": hierarchy.use_mad})), "root_params": np.asarray(_params_json(params)),
            "root_shape": np.asarray(shape)}
        data.update(_owned_arrays("initial", states))
        prepared, rhs = fmr_stage(states, parameters, hierarchy, layouts=layouts)
        data.update(_owned_arrays("stage1_rhs", rhs))
        last = len(states) - 1
        data.update(_padded_arrays("stage1_prepared", prepared[last], last))
        one = fmr_rk4_step(states, parameters, hierarchy, layouts=layouts)
        data.update(_owned_arrays("rk4_1", one))
        data.update(_padded_arrays("rk4_1_padded", one[last], last))
        two = fmr_rk4_step(one, parameters, hierarchy, layouts=layouts)
        data.update(_owned_arrays("rk4_2", two))
        norms = fmr_constraint_norms(two, parameters, hierarchy, layouts=layouts)
        data["norms"] = np.asarray(json.dumps({k: float(v) for k, v in norms.items()}))
        np.savez_compressed(out_dir / f"fmr_{name}.npz", **data)


def cartoon_cases():
    """Generic smooth data on the compact Cartoon grids (every component set)."""
    from JAX_BSSN.bssn.variables import BSSNParameters as P, BSSNVariables as V
    rng = np.random.default_rng(44)
    nrho, nz = 12, 20
    dx = 0.1
    x = (np.arange(nrho + 4) - 3.5) * dx
    z = -0.5 * (nz - 1) * dx + dx * np.arange(nz)
    X, Z = np.meshgrid(x, z, indexing="ij")

    def f2d(amp):
        c = rng.normal(size=5)
        return amp * (c[0] * np.cos(1.3 * X + c[1]) * np.sin(0.9 * Z + c[2]) + c[3] * np.cos(2.1 * Z + c[4]))

    def axi_field(rank, base):
        shape = (3,) * rank
        out = np.zeros(shape + (nrho + 4, 1, nz))
        for idx in np.ndindex(*shape):
            if rank == 2 and idx[0] > idx[1]:
                continue
            val = f2d(0.05) + (base if (rank == 0 or (rank == 2 and idx[0] == idx[1])) else 0.0)
            out[idx + (slice(None), 0, slice(None))] = val
            if rank == 2:
                out[(idx[1], idx[0]) + (slice(None), 0, slice(None))] = val
        return out

    axi = V(axi_field(2, 1.0), axi_field(0, 1.0), axi_field(2, 0.0), axi_field(0, 0.0), axi_field(1, 0.0),
            axi_field(0, 1.0), axi_field(1, 0.0))
    axi_params = P(eta=2.0, kappa=0.002, nu=0.02, g=0.75, dx=dx, dt=0.2 * dx, gauge=1, zero_shift=0,
                   xl_bc=0, xr_bc=1, yl_bc=0, yr_bc=0, zl_bc=1, zr_bc=1, x_min=-3.5 * dx, y_min=-4.0 * dx,
                   z_min=float(z[0]))
    nr = 16
    r = (np.arange(nr + 4) - 3.5) * dx

    def f1d(amp):
        c = rng.normal(size=3)
        return amp * (c[0] * np.cos(1.7 * r + c[1]) + c[2] * np.exp(-r * r))

    def sph_field(rank, base):
        shape = (3,) * rank
        out = np.zeros(shape + (nr + 4, 1, 1))
        if rank == 0:
            out[:, 0, 0] = base + f1d(0.05)
        elif rank == 1:
            out[0, :, 0, 0] = f1d(0.05)
        else:
            out[0, 0, :, 0, 0] = base + f1d(0.05)
            t = base + f1d(0.05)
            out[1, 1, :, 0, 0] = t
            out[2, 2, :, 0, 0] = t
        return out

    sph = V(sph_field(2, 1.0), sph_field(0, 1.0), sph_field(2, 0.0), sph_field(0, 0.0), sph_field(1, 0.0),
            sph_field(0, 1.0), sph_field(1, 0.0))
    sph_params = P(eta=2.0, kappa=0.0, nu=0.02, g=0.75, dx=dx, dt=0.2 * dx, gauge=1, zero_shift=0,
                   xl_bc=0, xr_bc=1, x_min=-3.5 * dx, y_min=-4.0 * dx, z_min=-4.0 * dx)
    return {"axisymmetric": (axi, axi_params), "spherical": (sph, sph_params)}


def matter_fields(shape, seed):
    """Smooth seeded matter sources rho (n), S_i (3, n), symmetric S_ij (3, 3, n)."""
    rng = np.random.default_rng(seed)
    axes = [np.linspace(0.0, 2.0 * np.pi, n, endpoint=False) for n in shape]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")

    def field(amp):
        c = rng.normal(size=6)
        return amp * (c[0] * np.sin(X + c[1]) + c[2] * np.cos(2.0 * Y + c[3]) + c[4] * np.sin(Z + X + c[5]))

    rho = 0.02 + field(0.01) ** 2
    S_i = np.stack([field(0.01) for _ in range(3)])
    S_ij = np.zeros((3, 3) + tuple(shape))
    for i in range(3):
        for j in range(i, 3):
            S_ij[i, j] = S_ij[j, i] = (0.01 if i == j else 0.0) + field(0.005)
    return rho, S_i, S_ij


def make_matter(out_dir: Path):
    """compute_bssn_rhs_with_matter (time_evolve.py:60-91) on three RHS cases:
    kappa != 0 (momentum-constraint damping with the matter momentum), Sommerfeld
    faces, and MAD weights."""
    from JAX_BSSN.evolution.time_evolve import compute_bssn_rhs_with_matter
    cases = rhs_cases()
    for name, seed in (("generic_kappa", 71), ("sommerfeld", 72), ("mad_mixed", 73)):
        state, params = cases[name]
        shape = np.asarray(state.conformal_factor).shape
        rho, S_i, S_ij = matter_fields(shape, seed)
        data = {"params": np.asarray(_params_json(params))}
        data.update(_state_arrays("input", state))
        data["matter.energy_density"] = rho
        data["matter.momentum_density"] = S_i
        data["matter.spatial_stress"] = S_ij
        data.update(_state_arrays("rhs", compute_bssn_rhs_with_matter(state, params, rho, S_i, S_ij)))
        np.savez_compressed(out_dir / f"matter_{name}.npz", **data)


def wave_tree():
    """A branching patch tree with synthetic level fields for the composite
    wave norms: two siblings under the root and a grandchild under the first."""
    from JAX_BSSN.fmr import FMRHierarchySpec, FMRPatchSpec
    hierarchy = FMRHierarchySpec((FMRPatchSpec((2, 2, 2), (5, 5, 4), parent=0),
                                  FMRPatchSpec((7, 2, 2), (9, 5, 5), parent=0),
                                  FMRPatchSpec((1, 1, 1), (3, 3, 3), parent=1)))
    rng = np.random.default_rng(2024)
    shapes = [(12, 10, 9)] + [tuple(2 * (h - l) + 1 for l, h in zip(s.coarse_lo, s.coarse_hi))
                              for s in hierarchy.patches]
    amplitude, wavelength, time = 1.0e-3, 2.0, 0.3
    levels, coords = [], []
    for shape in shapes:
        x = np.broadcast_to(rng.uniform(-1.0, 1.0, shape[0])[:, None, None], shape).copy()
        h = amplitude * np.sin(2.0 * np.pi * (x - time) / wavelength) + 1e-6 * rng.normal(size=shape)
        levels.append({"h_plus": h, "hamiltonian_constraint": rng.normal(size=shape),
                       "momentum_constraint": tuple(rng.normal(size=shape) for _ in range(3))})
        coords.append(x)
    return hierarchy, levels, coords, time, amplitude, wavelength


def make_waves(out_dir: Path):
    """h_plus and diagnostic_fields (diagnostics/waves.py:11-39) on the
    Sommerfeld RHS case, and composite_wave_diagnostics (:43-91) on a branching
    tree, with active and guard-padded level fields."""
    from JAX_BSSN.diagnostics.waves import composite_wave_diagnostics, diagnostic_fields, h_plus
    state, params = rhs_cases()["sommerfeld"]
    data = {"params": np.asarray(_params_json(params))}
    data.update(_state_arrays("input", state))
    data["h_plus"] = np.asarray(h_plus(state))
    fields = diagnostic_fields(state, params)
    data["hamiltonian"] = np.asarray(fields["hamiltonian_constraint"])
    data["momentum"] = np.stack([np.asarray(m) for m in fields["momentum_constraint"]])
    hierarchy, levels, coords, time, amplitude, wavelength = wave_tree()
    for i, (lv, x) in enumerate(zip(levels, coords)):
        data[f"tree.{i}.h_plus"] = lv["h_plus"]
        data[f"tree.{i}.hamiltonian"] = lv["hamiltonian_constraint"]
        data[f"tree.{i}.momentum"] = np.stack(lv["momentum_constraint"])
        data[f"tree.{i}.x"] = x
    data["tree.hierarchy"] = np.asarray(json.dumps([[list(s.coarse_lo), list(s.coarse_hi), s.parent]
                                                    for s in hierarchy.patches]))
    data["tree.scalars"] = np.array([time, amplitude, wavelength])
    active = composite_wave_diagnostics(tuple(levels), tuple(coords), hierarchy, time, amplitude, wavelength,
                                        active_fields=True)
    data["tree.active"] = np.array([active[k] for k in sorted(active)])
    # the same fields inside guard-padded arrays for every level below the root
    padded, padded_x = [levels[0]], [coords[0]]
    for lv, x, spec in zip(levels[1:], coords[1:], hierarchy.patches):
        g = spec.ghost_width
        pad = lambda a: np.pad(a, g, constant_values=999.0)  # noqa: E731
        padded.append({"h_plus": pad(lv["h_plus"]), "hamiltonian_constraint": pad(lv["hamiltonian_constraint"]),
                       "momentum_constraint": tuple(pad(m) for m in lv["momentum_constraint"])})
        padded_x.append(pad(x))
    guarded = composite_wave_diagnostics(tuple(padded), tuple(padded_x), hierarchy, time, amplitude, wavelength)
    data["tree.guarded"] = np.array([guarded[k] for k in sorted(guarded)])
    data["tree.keys"] = np.asarray(json.dumps(sorted(active)))
    np.savez_compressed(out_dir / "waves.npz", **data)


def puncture_cases():
    """Bowen-York solves: the reference suite's two boosted single punctures
    (tests/test_bowen_york.py:57-110), a generic boosted binary on a Cartesian
    grid, the axisymmetric collision's setup at reduced resolution
    (demos/axisymmetric_blackhole_collision, tolerances 1e-12) and a
    zero-momentum meridional grid (analytic Brill-Lindquist data)."""
    return {
        "cart_single": dict(axi=False, grid=(10, 5.0), masses=[1.0], positions=[[0.0, 0.0, 0.0]],
                            momenta=[[0.0, 0.0, 0.2]], tol=(1.0e-9, 12, 1.0e-11, 1000)),
        "cart_binary": dict(axi=False, grid=(20, 6.0), masses=[0.5, 0.4],
                            positions=[[0.05, -0.12, -1.07], [-0.08, 0.11, 1.21]],
                            momenta=[[0.1, -0.05, 0.2], [-0.1, 0.03, -0.15]], tol=(1.0e-10, 12, 1.0e-10, 1000)),
        "axi_single": dict(axi=True, grid=(12, 5.0), masses=[1.0], positions=[[0.0, 0.0, 0.0]],
                           momenta=[[0.0, 0.0, 0.2]], tol=(1.0e-9, 12, 1.0e-11, 1000)),
        "axi_binary": dict(axi=True, grid=(32, 8.0), masses=[0.5, 0.5], positions=[[0.0, 0.0, -1.5], [0.0, 0.0, 1.5]],
                           momenta=[[0.0, 0.0, 0.05], [0.0, 0.0, -0.05]], tol=(1.0e-12, 100, 1.0e-12, 1000)),
        "axi_zero": dict(axi=True, grid=(8, 4.0), masses=[1.0], positions=[[0.0, 0.0, 0.0]],
                         momenta=[[0.0, 0.0, 0.0]], tol=(1.0e-10, 12, 1.0e-10, 1000)),
    }


def make_puncture(out_dir: Path):
    """utilities/bowen_york_solver.py: grids, Brill-Lindquist psi, Bowen-York
    curvature, operators on seeded fields, and the Newton solves."""
    import jax.numpy as jnp
    from JAX_BSSN.utilities import bowen_york_solver as by
    data = {}
    for name, case in puncture_cases().items():
        n, extent = case["grid"]
        if case["axi"]:
            grid, dx = by.axisymmetric_cell_centered_grid(n, extent)
            solve = by.solve_axisymmetric_conformal_factor
            kw = dict(newton_tolerance=case["tol"][0], max_newton_iterations=case["tol"][1],
                      linear_tolerance=case["tol"][2], max_linear_iterations=case["tol"][3])
        else:
            grid, dx = by.cell_centered_grid(n, extent)
            solve = by.solve_conformal_factor
            kw = dict(newton_tolerance=case["tol"][0], max_newton_iterations=case["tol"][1],
                      cg_tolerance=case["tol"][2], max_cg_iterations=case["tol"][3])
        masses, positions, momenta = (jnp.asarray(case[k]) for k in ("masses", "positions", "momenta"))
        psi, u, history = solve(masses, positions, momenta, grid, dx, **kw)
        data[f"{name}.case"] = np.asarray(json.dumps(case))
        data[f"{name}.grid"] = np.asarray(grid)
        data[f"{name}.dx"] = np.asarray(dx)
        data[f"{name}.psi_bl"] = np.asarray(by.brill_lindquist_conformal_factor(masses, positions, grid))
        data[f"{name}.curvature"] = np.asarray(by.bowen_york_extrinsic_curvature(momenta, positions, grid))
        data[f"{name}.psi"] = np.asarray(psi)
        data[f"{name}.u"] = np.asarray(u)
        data[f"{name}.history"] = np.asarray(history, dtype=np.float64)
    # operators on seeded fields of the binary cases' grids
    rng = np.random.default_rng(11)
    for name in ("cart_binary", "axi_binary"):
        grid = data[f"{name}.grid"]
        dx = float(data[f"{name}.dx"])
        axi = name.startswith("axi")
        inner = (slice(None, -1), 0, slice(1, -1)) if axi else (slice(1, -1),) * 3
        curvature = jnp.asarray(data[f"{name}.curvature"])
        psi_bl = jnp.asarray(data[f"{name}.psi_bl"])
        a2 = np.asarray(by.contract_conformal_curvature(curvature))
        delta = rng.standard_normal(psi_bl[inner].shape)
        u = np.zeros(psi_bl.shape)
        u[inner] = 0.01 * rng.standard_normal(psi_bl[inner].shape)
        psi = np.asarray(psi_bl)[inner] + u[inner]
        data[f"{name}.a2"] = a2
        data[f"{name}.delta"] = delta
        data[f"{name}.u_probe"] = u
        lap = by.axisymmetric_laplacian if axi else by.laplacian
        lin = by.axisymmetric_linearized_hamiltonian_operator if axi else by.linearized_hamiltonian_operator
        res = by.axisymmetric_hamiltonian_residual if axi else by.hamiltonian_residual
        data[f"{name}.laplacian"] = np.asarray(lap(jnp.asarray(delta), dx))
        data[f"{name}.linearized"] = np.asarray(lin(jnp.asarray(delta), jnp.asarray(psi), jnp.asarray(a2[inner]), dx))
        data[f"{name}.residual"] = np.asarray(res(jnp.asarray(u), psi_bl, curvature, dx))
        data[f"{name}.source"] = np.asarray(by.hamiltonian_source(jnp.asarray(psi), jnp.asarray(a2[inner])))
        data[f"{name}.linearized_source"] = np.asarray(
            by.linearized_hamiltonian_source(jnp.asarray(delta), jnp.asarray(psi), jnp.asarray(a2[inner])))
    np.savez_compressed(out_dir / "puncture.npz", **data)


def make_cartoon(out_dir: Path):
    from JAX_BSSN.cartoon.axisymmetry import (axisymmetric_rk4_step, compute_axisymmetric_rhs,
                                              compute_axisymmetric_constraints, reconstruct_axisymmetric_support,
                                              compute_axisymmetric_constraint_norms, fill_axisymmetric_ghosts)
    from JAX_BSSN.cartoon.spherical_symmetry.evolution import cartoon_rk4_step, compute_cartoon_rhs
    from JAX_BSSN.cartoon.spherical_symmetry.diagnostics import (compute_cartoon_constraint_norms,
                                                                 compute_cartoon_constraints,
                                                                 compute_spherical_symmetry_norms)
    from JAX_BSSN.cartoon.spherical_symmetry.reconstruction import reconstruct_cartoon_support
    cases = cartoon_cases()
    state, params = cases["axisymmetric"]
    state = fill_axisymmetric_ghosts(state)
    data = {"params": np.asarray(_params_json(params))}
    data.update(_state_arrays("input", state))
    data.update(_state_arrays("support", reconstruct_axisymmetric_support(state, params)))
    data.update(_state_arrays("rhs", compute_axisymmetric_rhs(state, params)))
    one = axisymmetric_rk4_step(state, params)
    data.update(_state_arrays("rk4_1", one))
    data.update(_state_arrays("rk4_2", axisymmetric_rk4_step(one, params)))
    violations = compute_axisymmetric_constraints(one, params)
    for field in violations._fields:
        data[f"constraints.{field}"] = np.asarray(getattr(violations, field))
    norms = compute_axisymmetric_constraint_norms(violations, params=params)
    data["norms"] = np.asarray(json.dumps({k: float(v) for k, v in norms.items()}))
    np.savez_compressed(out_dir / "cartoon_axisymmetric.npz", **data)
    state, params = cases["spherical"]
    data = {"params": np.asarray(_params_json(params))}
    data.update(_state_arrays("input", state))
    data.update(_state_arrays("support", reconstruct_cartoon_support(state, params)))
    data.update(_state_arrays("rhs", compute_cartoon_rhs(state, params)))
    one = cartoon_rk4_step(state, params)
    data.update(_state_arrays("rk4_1", one))
    data.update(_state_arrays("rk4_2", cartoon_rk4_step(one, params)))
    violations = compute_cartoon_constraints(one, params)
    for field in violations._fields:
        data[f"constraints.{field}"] = np.asarray(getattr(violations, field))
    norms = compute_cartoon_constraint_norms(violations)
    data["norms"] = np.asarray(json.dumps({k: float(v) for k, v in norms.items()}))
    sym = compute_spherical_symmetry_norms(compute_cartoon_rhs(state, params))
    data["symmetry_norms"] = np.asarray(json.dumps({k: float(v) for k, v in sym.items()}))
    np.savez_compressed(out_dir / "cartoon_spherical.npz", **data)


# Apparent-horizon pins from the reference's own finder code
# (JAX_BSSN/utilities/apparent_horizon.py, hermite_interpolation.py), run
# unmodified under the stand-in.  There, jax.jacfwd (the metric derivative of
# the Hermite interpolant, piecewise cubic) is a Richardson-extrapolated
# central difference, accurate to about 1e-11, and jax.linearize (the Newton
# Jacobian) a central difference that only steers Newton.  A dense Newton step
# re-evaluates every node once per column, minutes per iteration here, so
# complete finds are stored for the radial-line cases; for every layout and
# slicing the pieces of the residual are stored on fixed inputs: sample (the
# interpolated metric, its derivative, K and the resolved flag), surface (the
# expansion and area density of a non-spherical surface), angular_derivatives
# and interpolate_angular.
HORIZON_FIND_OPTIONS = dict(n_theta=6, n_phi=12, max_angular=12, tolerance=1e-9, audit_tolerance=1.0,
                            mass_tolerance=1.0)
HORIZON_GRID = dict(volume_dx=0.1, volume_extent=3.0)


def make_horizon(out_dir: Path):
    import time
    sys.path.insert(0, str(REPO / "tests"))
    from horizon_cases import layout_case
    from JAX_BSSN.utilities.apparent_horizon import (angular_derivatives, angular_grid, build_geometry,
                                                     find_apparent_horizon, interpolate_angular, surface)
    data = {"find_options": np.asarray(json.dumps(HORIZON_FIND_OPTIONS)),
            "grid": np.asarray(json.dumps(HORIZON_GRID))}

    def wavy(n_theta, n_phi, base, amp):
        theta, phi, _ = angular_grid(n_theta, n_phi)
        return base + amp * np.sin(theta[:, None]) ** 2 * np.cos(2 * phi[None, :])

    # sample at seeded points (radii 1.2 .. 2.8, a few on axes and one outside)
    rng = np.random.default_rng(7)
    pts = rng.normal(size=(300, 3))
    pts *= (rng.uniform(1.2, 2.8, size=300) / np.linalg.norm(pts, axis=1))[:, None]
    pts[:5] = [[0, 0, 2.0], [2.0, 0, 0], [0, 2.0, 0], [1e-12, 0, 2.0], [0, 0, 40.0]]
    data["sample.points"] = pts
    for layout in ("line", "plane", "volume"):
        for slicing in ("isotropic", "kerr_schild"):
            axes, gamma, kij, mass, exact = layout_case(layout, slicing, **HORIZON_GRID)
            table, sample = build_geometry(axes, gamma, kij, margin=4)
            key = f"{layout}_{slicing}"
            if slicing == "kerr_schild":
                g, dg, k, valid = (np.asarray(a) for a in sample(table, pts))
                for name, value in (("gamma", g), ("d_gamma", dg), ("curvature", k), ("valid", valid)):
                    data[f"sample.{layout}.{name}"] = value
            h = wavy(8, 16, 1.1 * exact, 0.03 * exact)
            center = np.zeros(3) if layout == "line" else np.array([0.0, 0.0, 0.02])
            expansion, density, usable = surface(h, center, table, sample)
            data[f"surface.{key}.radius"] = h
            data[f"surface.{key}.center"] = center
            data[f"surface.{key}.expansion"] = np.asarray(expansion)
            data[f"surface.{key}.density"] = np.asarray(density)
            data[f"surface.{key}.usable"] = np.asarray(bool(usable))
    field = wavy(10, 20, 1.1, 0.03) + 0.01 * np.random.default_rng(3).normal(size=(10, 20))
    data["angular.field"] = field
    for k, d in enumerate(angular_derivatives(field)):
        data[f"angular.derivative{k}"] = np.asarray(d)
    theta, phi, _ = angular_grid(22, 42)
    data["angular.regrid"] = np.asarray(interpolate_angular(field, theta, phi))
    for slicing, guess in (("isotropic", 1.15), ("kerr_schild", 0.9)):
        axes, gamma, kij, mass, exact = layout_case("line", slicing, **HORIZON_GRID)
        t = time.time()
        found = find_apparent_horizon(axes, gamma, kij, center=(0.0, 0.0, 0.0), initial_radius=guess * exact,
                                      **HORIZON_FIND_OPTIONS)
        print(f"horizon line_{slicing}: mass {found['mass']:.10f} ({time.time() - t:.0f} s)", flush=True)
        key = f"find.line_{slicing}"
        data[f"{key}.guess"] = np.asarray(guess)
        for name in ("radius", "expansion", "convergence"):
            data[f"{key}.{name}"] = np.asarray(found[name])
        for name in ("area", "mass", "residual", "audit_residual"):
            data[f"{key}.{name}"] = np.asarray(found[name])
    np.savez_compressed(out_dir / "horizon.npz", **data)


def main(argv):
    args = [a for a in argv[1:] if not a.startswith("--")]
    reference = Path(args[0]) if args else Path("/root/reference")
    _setup(reference)
    only = [part for a in argv if a.startswith("--only=") for part in a.split("=", 1)[1].split(",")]
    parts = {"stencils": lambda: make_stencils(HERE / "stencils.npz"), "rhs": lambda: make_rhs(HERE),
             "fmr": lambda: make_fmr(HERE), "cartoon": lambda: make_cartoon(HERE),
             "matter": lambda: make_matter(HERE), "waves": lambda: make_waves(HERE),
             "puncture": lambda: make_puncture(HERE), "horizon": lambda: make_horizon(HERE),
             "long": lambda: make_long_runs(HERE)}
    for name, build in parts.items():
        if only and name not in only:
            continue
        if name == "long" and "--no-long" in argv:
            continue
        build()
    for path in sorted(HERE.glob("*.npz")):
        print(f"{path.name}: {path.stat().st_size / 1024:.0f} KiB")


if __name__ == "__main__":
    main(sys.argv)
