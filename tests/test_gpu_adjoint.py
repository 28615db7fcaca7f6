"""Adjoint kernels against central finite differences of the forward path.

The reference never differentiates its evolution, so finite differences of
the (oracle-pinned) forward kernels are the gradient oracle:
  * the RHS VJP in dot-product form, <kbar, J v> = <J^T kbar, v>, with J v
    from central differences of compute_bssn_rhs (JAX_BSSN/evolution/
    time_evolve.py:41-57), one state component at a time, for generic,
    harmonic zero-shift, MAD, signed-shift (upwind) and Sommerfeld-faced
    configurations (the one-sided closure rows and the radial face condition,
    JAX_BSSN/evolution/boundaries.py:150-171);
  * one RK4 step (time_evolve.py:144-217) the same way, periodic and
    Sommerfeld-faced;
  * the gradient of a loss after several steps of a Sommerfeld-faced wave
    against central differences;
  * the gradient of a gauge-wave loss after many steps with respect to a
    seeded conformal-metric perturbation, batched over seeds, against central
    differences (h = 1e-6) along random directions: within 1e-6;
  * checkpoint schedules (segment lengths, stored or recomputed stages) and
    batching change nothing, bit for bit.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FD_TOL = 1e-6


def _batch(states):
    from jax_bssn_gb300.evolution.adjoint import components
    return torch.stack([components(s) for s in states], dim=1).cuda()


def _rhs_batch(u, params):
    from jax_bssn_gb300.evolution.adjoint import components, leaves
    from jax_bssn_gb300.evolution.time_evolve import compute_bssn_rhs
    return torch.stack([components(compute_bssn_rhs(leaves(u[:, i]), params)) for i in range(u.shape[1])], dim=1)


def _configs():
    from jax_bssn_gb300 import BSSNParameters
    from jax_bssn_gb300.initial_data import random_smooth_state
    base = dict(eta=1.5, kappa=0.0, nu=0.06, g=0.75, dx=0.09, dt=0.01)
    shape = (12, 10, 14)
    strong = random_smooth_state(shape, seed=5)
    strong = strong._replace(shift=strong.shift * 6.0)       # |beta| ~ 0.3: upwind sides matter
    # The shift is nonzero in every case: at beta = 0 exactly the upwinded
    # advection beta * U_sign(beta) f has a kink (the one-sided stencils differ
    # from the centred one), where central differences average the two sides
    # and the adjoint, like jax.grad through the reference's selection, takes
    # the centred stencil.
    return [
        ("generic_1+log", [random_smooth_state(shape, seed=s) for s in (1, 2)], BSSNParameters(gauge=1, **base)),
        ("harmonic_frozen_shift", [random_smooth_state(shape, seed=3)],
         BSSNParameters(gauge=0, zero_shift=1, **dict(base, eta=0.0))),
        ("mad", [random_smooth_state(shape, seed=4)], BSSNParameters(gauge=1, mad_q=1.0 / 16.0, **base)),
        ("large_shift", [strong], BSSNParameters(gauge=1, **base)),
        ("sommerfeld", [random_smooth_state(shape, seed=s) for s in (6, 7)],
         BSSNParameters(gauge=1, xl_bc=1, xr_bc=1, yl_bc=1, yr_bc=1, zl_bc=1, zr_bc=1,
                        x_min=-0.5, y_min=-0.45, z_min=-0.6, **base)),
        ("sommerfeld_x_z_periodic_y", [random_smooth_state(shape, seed=8)],
         BSSNParameters(gauge=1, xl_bc=1, xr_bc=1, zl_bc=1, zr_bc=1, x_min=-0.5, y_min=0.0, z_min=-0.6, **base)),
    ]


@pytest.mark.parametrize("case", range(6))
def test_rhs_vjp_dot_product(cuda, native, case):
    from jax_bssn_gb300.evolution.adjoint import rhs_vjp
    name, states, params = _configs()[case]
    u = _batch(states)
    gen = torch.Generator(device="cuda").manual_seed(11 + case)
    kbar = torch.randn(u.shape, generator=gen, device="cuda", dtype=torch.float64)
    ub = rhs_vjp(u, kbar, params)
    worst = 0.0
    for c in range(21):
        v = torch.zeros_like(u)
        v[c] = torch.randn(u[c].shape, generator=gen, device="cuda", dtype=torch.float64)
        h = 1e-6
        jv = (_rhs_batch(u + h * v, params) - _rhs_batch(u - h * v, params)) / (2 * h)
        lhs = float((kbar * jv).sum())
        rhs = float((ub * v).sum())
        scale = float((kbar.abs() * jv.abs()).sum()) + 1e-30
        err = abs(lhs - rhs) / scale
        worst = max(worst, err)
        assert err < FD_TOL, (name, c, lhs, rhs, err)
    print(name, "rhs vjp worst", f"{worst:.2e}")


@pytest.mark.parametrize("case", (0, 4, 5))
def test_rk4_step_vjp_dot_product(cuda, native, case):
    from jax_bssn_gb300.evolution import BatchEvolution
    from jax_bssn_gb300.evolution.adjoint import CheckpointedEvolution, components, leaves
    name, states, params = _configs()[case]
    u = _batch(states)

    def step(x):
        evo = BatchEvolution([leaves(x[:, i]) for i in range(x.shape[1])], params)
        evo.step(1)
        return torch.stack([components(evo.state(i)) for i in range(x.shape[1])], dim=1)

    gen = torch.Generator(device="cuda").manual_seed(5)
    ybar = torch.randn(u.shape, generator=gen, device="cuda", dtype=torch.float64)
    run = CheckpointedEvolution(u, params, 1)
    out = run.forward()
    assert torch.equal(out, step(u))
    ub = run.backward(ybar)
    for c in range(21):
        v = torch.zeros_like(u)
        v[c] = torch.randn(u[c].shape, generator=gen, device="cuda", dtype=torch.float64)
        h = 1e-6
        jv = (step(u + h * v) - step(u - h * v)) / (2 * h)
        lhs, rhs = float((ybar * jv).sum()), float((ub * v).sum())
        scale = float((ybar.abs() * jv.abs()).sum()) + 1e-30
        assert abs(lhs - rhs) / scale < FD_TOL, (c, lhs, rhs)


def _perturbed_gauge_waves(n, seeds, amplitude=1e-3):
    """The gauge wave with a seeded symmetric 1e-3 Gaussian perturbation of gt_ij."""
    from jax_bssn_gb300.evolution.adjoint import components
    from jax_bssn_gb300.initial_data import gauge_wave_config
    state, params = gauge_wave_config(n=n)
    base = components(state).cuda()
    batch = []
    for seed in seeds:
        rng = np.random.default_rng(seed)
        u = base.clone()
        u[0:6] += torch.as_tensor(amplitude * rng.standard_normal((6,) + tuple(base.shape[1:])), device="cuda")
        batch.append(u)
    return torch.stack(batch, dim=1), base, params


def _loss(u_final, w_target):
    return 0.5 * ((u_final[6] - w_target) ** 2).sum()


def _smooth_direction(shape, gen):
    """A random smooth periodic field per conformal-metric component: a few
    low Fourier modes with random amplitudes and phases."""
    n = shape[-3:]
    axes = [torch.arange(m, device="cuda", dtype=torch.float64) * (2 * torch.pi / m) for m in n]
    X, Y, Z = torch.meshgrid(*axes, indexing="ij")
    out = torch.zeros(shape, device="cuda", dtype=torch.float64)
    for c in range(6):
        for i in range(shape[1]):
            r = torch.rand(9, generator=gen, device="cuda", dtype=torch.float64)
            out[c, i] = (r[0] * torch.sin(X + 6 * r[1]) + r[2] * torch.cos(2 * Y + 6 * r[3])
                         + r[4] * torch.sin(Z + X + 6 * r[5]) + r[6] * torch.cos(2 * Z - Y + 6 * r[7]))
    return out


def test_evolution_gradient_matches_finite_differences(cuda, native):
    """The gauge wave with seeded 1e-3 metric perturbations (three seeds in one
    batch), 12 steps: <grad, d> against central differences with h = 1e-6
    along smooth random directions, and along white-noise directions where
    Richardson extrapolation of h and h/2 removes the O(h^2) term."""
    from jax_bssn_gb300.evolution.adjoint import evolve
    steps = 12
    u0, base, params = _perturbed_gauge_waves(16, seeds=(0, 1, 2))
    w_target = evolve(base[:, None].contiguous(), params, steps)[6]
    x = u0.clone().requires_grad_(True)
    loss = _loss(evolve(x, params, steps), w_target)
    loss.backward()
    grad = x.grad
    assert torch.isfinite(grad).all()

    def central(d, h):
        with torch.no_grad():
            lp = float(_loss(evolve(u0 + h * d, params, steps), w_target))
            lm = float(_loss(evolve(u0 - h * d, params, steps), w_target))
        return (lp - lm) / (2 * h)

    gen = torch.Generator(device="cuda").manual_seed(21)
    worst = 0.0
    for trial in range(8):
        d = _smooth_direction(u0.shape, gen)
        fd = central(d, 1e-6)
        ad = float((grad * d).sum())
        err = abs(ad - fd) / abs(fd)
        worst = max(worst, err)
        assert err < FD_TOL, (trial, ad, fd, err)
    print("evolution gradient vs FD (smooth directions) worst", f"{worst:.2e}")
    for trial in range(2):
        d = torch.zeros_like(u0)
        d[0:6] = torch.randn(d[0:6].shape, generator=gen, device="cuda", dtype=torch.float64)
        f1, f2 = central(d, 1e-5), central(d, 5e-6)
        richardson = (4.0 * f2 - f1) / 3.0
        ad = float((grad * d).sum())
        err = abs(ad - richardson) / abs(richardson)
        print("white-noise direction: h=1e-5", f"{abs(ad - f1) / abs(f1):.2e}", "extrapolated", f"{err:.2e}")
        assert err < FD_TOL, (trial, ad, richardson, err)


def test_sommerfeld_evolution_gradient_matches_finite_differences(cuda, native):
    """A Teukolsky wave on a 16^3 grid with Sommerfeld faces (the radial
    condition and the one-sided rows every step) and a uniform shift, two
    instances, 6 steps: the gradient of a loss on the change of the conformal
    factor against central differences along smooth random directions of
    every component."""
    from jax_bssn_gb300.evolution.adjoint import components, evolve
    from jax_bssn_gb300.initial_data import teukolsky_config
    steps = 6
    state, params = teukolsky_config(n=16, amplitude=1e-2)
    base = components(state).cuda()
    # a uniform background shift keeps every shift component away from 0, where
    # the upwinded advection has a kink that central differences average over
    base[18:21] += torch.tensor([0.05, 0.04, 0.03], dtype=torch.float64, device="cuda")[:, None, None, None]
    gen = torch.Generator(device="cuda").manual_seed(3)
    u0 = torch.stack([base, base + 1e-3 * _smooth_direction(base[:, None].shape, gen)[:, 0]], dim=1)
    target = u0[6].clone()   # the loss measures W's change: small, so central differences keep their digits
    x = u0.clone().requires_grad_(True)
    loss = _loss(evolve(x, params, steps), target)
    loss.backward()
    grad = x.grad
    assert torch.isfinite(grad).all()

    def central(d, h):
        with torch.no_grad():
            lp = float(_loss(evolve(u0 + h * d, params, steps), target))
            lm = float(_loss(evolve(u0 - h * d, params, steps), target))
        return (lp - lm) / (2 * h)

    worst = 0.0
    for trial in range(6):
        d = torch.zeros_like(u0)
        smooth = _smooth_direction(u0.shape, gen)
        for c in range(21):
            d[c] = smooth[c % 6] * (0.1 if c >= 6 else 1.0)
        fd = central(d, 1e-6)
        ad = float((grad * d).sum())
        err = abs(ad - fd) / abs(fd)
        worst = max(worst, err)
        assert err < FD_TOL, (trial, ad, fd, err)
    print("Sommerfeld evolution gradient vs FD worst", f"{worst:.2e}")


def test_checkpoint_schedules_and_batching_are_bitwise(cuda, native):
    from jax_bssn_gb300.evolution.adjoint import CheckpointedEvolution
    u0, _, params = _perturbed_gauge_waves(12, seeds=(3, 4))
    gen = torch.Generator(device="cuda").manual_seed(2)
    steps = 7
    ybar = torch.randn(u0.shape, generator=gen, device="cuda", dtype=torch.float64)
    grads = []
    finals = []
    for segment, store in ((0, 1), (0, 0), (1, 1), (3, 0), (7, 1), (0, 2), (2, 2)):
        run = CheckpointedEvolution(u0, params, steps, segment=segment, store_stages=store)
        finals.append(run.forward().clone())
        grads.append(run.backward(ybar))
    for f, g in zip(finals[1:], grads[1:]):
        assert torch.equal(f, finals[0])
        assert torch.equal(g, grads[0])
    for i in range(u0.shape[1]):
        single = CheckpointedEvolution(u0[:, i:i + 1].contiguous(), params, steps)
        single.forward()
        assert torch.equal(single.backward(ybar[:, i:i + 1].contiguous())[:, 0], grads[0][:, i])


def test_adjoint_rejects_unsupported_configurations(cuda, native):
    from jax_bssn_gb300 import BSSNParameters
    from jax_bssn_gb300.evolution.adjoint import rhs_vjp
    u = torch.zeros((21, 1, 10, 10, 10), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError, match="both faces"):
        rhs_vjp(u, u, BSSNParameters(dx=0.1, xl_bc=1))
    with pytest.raises(ValueError, match="kappa"):
        rhs_vjp(u, u, BSSNParameters(dx=0.1, kappa=0.1))
