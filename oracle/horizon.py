"""Apparent-horizon finder restated in NumPy (test infrastructure).

Follows uwplasma/JAX_BSSN/utilities/apparent_horizon.py and
hermite_interpolation.py:
  hermite_weights, interpolate_point       hermite_interpolation.py:12-38
  build_geometry (line / plane / volume)   apparent_horizon.py:22-117
  angular_grid, theta_ghosts,
  angular_derivatives, interpolate_angular  :101-157
  surface (expansion, area density)         :160-236
  find_apparent_horizon                     :253-338

The reference differentiates the metric through the interpolation with
jax.jacfwd and the whole residual with jax.linearize.  Here the metric
derivative is the analytic derivative of the Hermite basis, carried through
the radial projection (line) or the azimuthal rotation (plane) by the chain
rule, and the Newton Jacobian is assembled from central differences of the
pointwise residual with respect to h and its five angular derivatives (the
residual at a node depends on the surface only through those six values).
A converged root does not depend on how the Jacobian was formed.  JAX is not
installed, so the reference cannot be run to pin this restatement; the
reference suite's analytic Schwarzschild answers (tests/test_apparent_horizon.py)
check it.  Only the tests and the bench's CPU legs import this module.
"""

from __future__ import annotations

import functools

import numpy as np

from .cartoon import interpolate as _lagrange6_interpolate


# ---------------------------------------------------------------------------
# Hermite interpolation (hermite_interpolation.py:12-38)
# ---------------------------------------------------------------------------
_LEFT = np.array([1.0, -8.0, 0.0, 8.0, -1.0, 0.0]) / 12
_RIGHT = np.array([0.0, 1.0, -8.0, 0.0, 8.0, -1.0]) / 12


def hermite_weights(index, size):
    """Node indices (n, 6), weights (n, 6) and their index derivatives."""
    index = np.asarray(index, dtype=np.float64)
    cell = np.clip(np.floor(index).astype(int), 2, size - 4)
    t = (index - cell)[..., None]
    h00, h01 = 2 * t ** 3 - 3 * t ** 2 + 1, -2 * t ** 3 + 3 * t ** 2
    h10, h11 = t ** 3 - 2 * t ** 2 + t, t ** 3 - t ** 2
    d00, d01 = 6 * t ** 2 - 6 * t, -6 * t ** 2 + 6 * t
    d10, d11 = 3 * t ** 2 - 4 * t + 1, 3 * t ** 2 - 2 * t
    w = h10 * _LEFT + h11 * _RIGHT
    dw = d10 * _LEFT + d11 * _RIGHT
    w[..., 2] += h00[..., 0]
    w[..., 3] += h01[..., 0]
    dw[..., 2] += d00[..., 0]
    dw[..., 3] += d01[..., 0]
    return cell[..., None] + np.arange(-2, 4), w, dw


def _interpolate(table, indices, spacing):
    """Values (n, f) and spatial derivatives (n, dims, f) of a (f, *grid) table."""
    dims = len(indices)
    parts = [hermite_weights(q, n) for q, n in zip(indices, table.shape[1:])]
    npts = np.asarray(indices[0]).shape[0]
    values = np.zeros((npts, table.shape[0]))
    derivs = np.zeros((npts, dims, table.shape[0]))
    if dims == 1:
        nodes, w, dw = parts[0]
        block = table[:, nodes]                       # (f, n, 6)
        values = np.einsum("fna,na->nf", block, w)
        derivs[:, 0] = np.einsum("fna,na->nf", block, dw) / spacing[0]
        return values, derivs
    if dims == 2:
        (n0, w0, d0), (n1, w1, d1) = parts
        block = table[:, n0[:, :, None], n1[:, None, :]]   # (f, n, 6, 6)
        values = np.einsum("fnab,na,nb->nf", block, w0, w1)
        derivs[:, 0] = np.einsum("fnab,na,nb->nf", block, d0, w1) / spacing[0]
        derivs[:, 1] = np.einsum("fnab,na,nb->nf", block, w0, d1) / spacing[1]
        return values, derivs
    (n0, w0, d0), (n1, w1, d1), (n2, w2, d2) = parts
    block = table[:, n0[:, :, None, None], n1[:, None, :, None], n2[:, None, None, :]]
    values = np.einsum("fnabc,na,nb,nc->nf", block, w0, w1, w2)
    derivs[:, 0] = np.einsum("fnabc,na,nb,nc->nf", block, d0, w1, w2) / spacing[0]
    derivs[:, 1] = np.einsum("fnabc,na,nb,nc->nf", block, w0, d1, w2) / spacing[1]
    derivs[:, 2] = np.einsum("fnabc,na,nb,nc->nf", block, w0, w1, d2) / spacing[2]
    return values, derivs


# ---------------------------------------------------------------------------
# geometry (apparent_horizon.py:22-98)
# ---------------------------------------------------------------------------
def build_geometry(coordinates, gamma, Kij, margin=4):
    if isinstance(coordinates, np.ndarray) and coordinates.ndim == 1:
        coordinates = (coordinates,)
    axes = tuple(np.asarray(a, dtype=float) for a in coordinates)
    dims = len(axes)
    gamma, Kij = np.asarray(gamma, dtype=float), np.asarray(Kij, dtype=float)
    if dims == 1:
        table = np.stack([gamma[0, 0], gamma[1, 1], Kij[0, 0], Kij[1, 1]])
    else:
        shape = tuple(len(a) for a in axes)
        table = np.concatenate((gamma.reshape((9,) + shape), Kij.reshape((9,) + shape)))
    origin = np.array([a[0] for a in axes])
    spacing = np.array([a[1] - a[0] for a in axes])
    sizes = np.array([len(a) for a in axes])

    def sample(points):
        p = np.asarray(points, dtype=float)
        n = p.shape[0]
        eye = np.eye(3)
        if dims == 1:
            r = np.linalg.norm(p, axis=1)
            vals, der = _interpolate(table, ((r - origin[0]) / spacing[0],), spacing)
            nrm = p / np.maximum(r, 1e-30)[:, None]
            rr = nrm[:, :, None] * nrm[:, None, :]
            metric = vals[:, 0, None, None] * rr + vals[:, 1, None, None] * (eye - rr)
            curv = vals[:, 2, None, None] * rr + vals[:, 3, None, None] * (eye - rr)
            dnd = (eye[None] - rr) / np.maximum(r, 1e-30)[:, None, None]   # dn_i/dp_k: (n, i, k)
            grr, gtt = der[:, 0, 0], der[:, 0, 1]
            d = np.zeros((n, 3, 3, 3))                                     # (n, k, i, j)
            for k in range(3):
                drr = dnd[:, :, k][:, :, None] * nrm[:, None, :] + nrm[:, :, None] * dnd[:, :, k][:, None, :]
                d[:, k] = ((grr - gtt) * nrm[:, k])[:, None, None] * rr + (gtt * nrm[:, k])[:, None, None] * eye \
                    + (vals[:, 0] - vals[:, 1])[:, None, None] * drr
            coord0 = r
            index = ((r - origin[0]) / spacing[0])[:, None]
        elif dims == 2:
            rho = np.linalg.norm(p[:, :2], axis=1)
            vals, der = _interpolate(table, ((rho - origin[0]) / spacing[0], (p[:, 2] - origin[1]) / spacing[1]),
                                     spacing)
            M, Kp = vals[:, :9].reshape(n, 3, 3), vals[:, 9:].reshape(n, 3, 3)
            dM_drho, dM_dz = der[:, 0, :9].reshape(n, 3, 3), der[:, 1, :9].reshape(n, 3, 3)
            safe = np.maximum(rho, 1e-30)
            c, s = p[:, 0] / safe, p[:, 1] / safe
            R = np.zeros((n, 3, 3))
            R[:, 0, 0], R[:, 0, 1], R[:, 1, 0], R[:, 1, 1], R[:, 2, 2] = c, -s, s, c, 1.0
            metric = R @ M @ np.swapaxes(R, 1, 2)
            curv = R @ Kp @ np.swapaxes(R, 1, 2)
            dc = np.stack([s * s / safe, -c * s / safe, np.zeros(n)], axis=1)
            ds = np.stack([-c * s / safe, c * c / safe, np.zeros(n)], axis=1)
            drho = np.stack([c, s, np.zeros(n)], axis=1)
            d = np.zeros((n, 3, 3, 3))
            for k in range(3):
                dR = np.zeros((n, 3, 3))
                dR[:, 0, 0], dR[:, 0, 1], dR[:, 1, 0], dR[:, 1, 1] = dc[:, k], -ds[:, k], ds[:, k], dc[:, k]
                dMk = dM_drho * drho[:, k, None, None] + (dM_dz if k == 2 else 0.0)
                d[:, k] = dR @ M @ np.swapaxes(R, 1, 2) + R @ dMk @ np.swapaxes(R, 1, 2) \
                    + R @ M @ np.swapaxes(dR, 1, 2)
            coord0 = rho
            index = np.stack([(rho - origin[0]) / spacing[0], (p[:, 2] - origin[1]) / spacing[1]], axis=1)
        else:
            idx = tuple((p[:, a] - origin[a]) / spacing[a] for a in range(3))
            vals, der = _interpolate(table, idx, spacing)
            metric, curv = vals[:, :9].reshape(n, 3, 3), vals[:, 9:].reshape(n, 3, 3)
            d = der[:, :, :9].reshape(n, 3, 3, 3)
            coord0 = None
            index = np.stack(idx, axis=1)
        inside = np.all((index >= margin) & (index <= sizes - 1 - margin), axis=1)
        if dims < 3:
            inside &= coord0 > 1e-10 * spacing[0]
        return metric, d, curv, inside

    return sample


# ---------------------------------------------------------------------------
# angular tools (apparent_horizon.py:101-157)
# ---------------------------------------------------------------------------
def angular_grid(n_theta, n_phi):
    theta = (np.arange(n_theta) + 0.5) * np.pi / n_theta
    phi = np.arange(n_phi) * 2 * np.pi / n_phi
    modes = np.arange(n_theta)
    integrals = np.zeros(n_theta)
    even = modes[modes % 2 == 0]
    integrals[even] = 2 / (1 - even ** 2)
    integrals[1:] *= 2
    weights = integrals @ np.cos(np.outer(modes, theta)) / n_theta
    return theta, phi, weights


def theta_ghosts(field, width):
    shift = field.shape[1] // 2
    low = np.flip(np.roll(field[:width], shift, axis=1), axis=0)
    high = np.flip(np.roll(field[-width:], shift, axis=1), axis=0)
    return np.concatenate((low, field, high), axis=0)


_FIRST = (1 / 12, -2 / 3, 0.0, 2 / 3, -1 / 12)
_SECOND = (-1 / 12, 4 / 3, -2.5, 4 / 3, -1 / 12)


def angular_derivatives(field):
    n_theta, n_phi = field.shape

    def polar(values, stencil, power):
        ext = theta_ghosts(values, 2)
        return sum(w * ext[k:k + n_theta] for k, w in enumerate(stencil) if w) / (np.pi / n_theta) ** power

    def azimuthal(values, stencil, power):
        return sum(w * np.roll(values, 2 - k, axis=1) for k, w in enumerate(stencil) if w) / (2 * np.pi / n_phi) ** power

    h_phi = azimuthal(field, _FIRST, 1)
    return polar(field, _FIRST, 1), polar(field, _SECOND, 2), h_phi, azimuthal(field, _SECOND, 2), polar(h_phi, _FIRST, 1)


def interpolate_angular(radius, theta, phi):
    n_theta, n_phi = radius.shape
    field = theta_ghosts(radius, 3)
    field = _lagrange6_interpolate(field, np.asarray(theta) * n_theta / np.pi - 0.5 + 3, 0)
    field = np.concatenate((field[:, -3:], field, field[:, :3]), axis=1)
    return _lagrange6_interpolate(field, np.asarray(phi) * n_phi / (2 * np.pi) + 3, 1)


# ---------------------------------------------------------------------------
# expansion (apparent_horizon.py:160-236), pointwise in (h, its five angular
# derivatives) once the geometry is sampled at the surface point
# ---------------------------------------------------------------------------
def _frames(n_theta, n_phi):
    theta, phi, _ = angular_grid(n_theta, n_phi)
    t, p = np.meshgrid(theta, phi, indexing="ij")
    st, ct, sp, cp = np.sin(t), np.cos(t), np.sin(p), np.cos(p)
    radial = np.stack([st * cp, st * sp, ct], axis=-1).reshape(-1, 3)
    polar = np.stack([ct * cp, ct * sp, -st], axis=-1).reshape(-1, 3)
    azimuthal = np.stack([-sp, cp, np.zeros_like(t)], axis=-1).reshape(-1, 3)
    return radial, polar, azimuthal, st.reshape(-1), (ct / st).reshape(-1)


def _pointwise(h, ht, htt, hp, hpp, htp, frames, gamma, d_gamma, curvature):
    radial, polar, azimuthal, sine, cot = frames
    sym = lambda a, b: a[:, :, None] * b[:, None, :] + b[:, :, None] * a[:, None, :]  # noqa: E731
    gradient = radial - (ht / h)[:, None] * polar - (hp / (h * sine))[:, None] * azimuthal
    hess = (ht / h ** 2)[:, None, None] * sym(radial, polar)
    hess = hess + (hp / (h ** 2 * sine))[:, None, None] * sym(radial, azimuthal)
    hess = hess + (1 / h - htt / h ** 2)[:, None, None] * sym(polar, polar) / 2
    hess = hess + ((cot * hp - htp) / (h ** 2 * sine))[:, None, None] * sym(polar, azimuthal)
    hess = hess + (1 / h - cot * ht / h ** 2 - hpp / (h ** 2 * sine ** 2))[:, None, None] * sym(azimuthal, azimuthal) / 2
    with np.errstate(invalid="ignore"):
        inverse = np.linalg.inv(gamma)
    up = np.einsum("nij,nj->ni", inverse, gradient)
    norm = np.sqrt(np.sum(gradient * up, axis=1))
    normal = up / norm[:, None]
    projector = inverse - normal[:, :, None] * normal[:, None, :]
    cg = 0.5 * np.einsum("nl,nijl->nij", up, d_gamma.transpose(0, 1, 3, 2) + d_gamma.transpose(0, 3, 1, 2)
                         - d_gamma.transpose(0, 2, 3, 1))
    divergence = np.einsum("nij,nij->n", projector, hess - cg) / norm
    expansion = divergence + np.einsum("nij,ni,nj->n", curvature, normal, normal) \
        - np.einsum("nij,nij->n", inverse, curvature)
    tt = ht[:, None] * radial + h[:, None] * polar
    tp = (hp / sine)[:, None] * radial + h[:, None] * azimuthal
    mtt = np.einsum("ni,nij,nj->n", tt, gamma, tt)
    mpp = np.einsum("ni,nij,nj->n", tp, gamma, tp)
    mtp = np.einsum("ni,nij,nj->n", tt, gamma, tp)
    density = np.sqrt(mtt * mpp - mtp ** 2)
    return expansion, density


def surface(radius, center, sample):
    n_theta, n_phi = radius.shape
    frames = _frames(n_theta, n_phi)
    derivs = [d.reshape(-1) for d in angular_derivatives(radius)]
    h = radius.reshape(-1)
    points = np.asarray(center)[None, :] + h[:, None] * frames[0]
    gamma, d_gamma, curvature, resolved = sample(points)
    with np.errstate(invalid="ignore", divide="ignore"):
        physical = bool(np.all(np.linalg.eigvalsh(gamma) > 0)) if np.all(np.isfinite(gamma)) else False
        expansion, density = _pointwise(h, *derivs, frames, gamma, d_gamma, curvature)
    usable = bool(np.all(resolved) and physical and np.all(np.isfinite(expansion)) and np.all(np.isfinite(density))
                  and np.all(h > 0))
    return expansion.reshape(radius.shape), density.reshape(radius.shape), usable


@functools.lru_cache(maxsize=8)
def _stencil_matrices(n_theta, n_phi):
    """The five angular-derivative operators as dense (N, N) matrices."""
    n = n_theta * n_phi
    mats = np.zeros((5, n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        for m, d in enumerate(angular_derivatives(e.reshape(n_theta, n_phi))):
            mats[m, :, j] = d.reshape(-1)
    return mats


def jacobian(radius, center, sample, step=1e-6):
    """dTheta_i/dh_j from central differences of the pointwise residual in
    h_i (geometry resampled) and in each angular derivative (geometry fixed)."""
    n_theta, n_phi = radius.shape
    frames = _frames(n_theta, n_phi)
    h = radius.reshape(-1)
    derivs = [d.reshape(-1) for d in angular_derivatives(radius)]

    def at(hh, dd, geom=None):
        if geom is None:
            geom = sample(np.asarray(center)[None, :] + hh[:, None] * frames[0])[:3]
        return _pointwise(hh, *dd, frames, *geom)[0]
    geom = sample(np.asarray(center)[None, :] + h[:, None] * frames[0])[:3]
    dh = step * np.maximum(np.abs(h), 1.0)
    partial_h = (at(h + dh, derivs) - at(h - dh, derivs)) / (2 * dh)
    jac = np.diag(partial_h)
    for m, S in enumerate(_stencil_matrices(n_theta, n_phi)):
        scale = step * np.maximum(np.abs(derivs[m]), 1.0)
        up = list(derivs)
        dn = list(derivs)
        up[m] = derivs[m] + scale
        dn[m] = derivs[m] - scale
        partial = (at(h, up, geom) - at(h, dn, geom)) / (2 * scale)
        jac = jac + partial[:, None] * S
    return jac


def find_apparent_horizon(coordinates, gamma, Kij, *, center, initial_radius, n_theta=12, n_phi=24,
                          max_angular=48, tolerance=1.e-8, audit_tolerance=1.e-4, mass_tolerance=1.e-3,
                          max_iterations=50, margin=4):
    sample = build_geometry(coordinates, gamma, Kij, margin=margin)
    center = np.asarray(center, dtype=float)
    initial = np.asarray(initial_radius, dtype=float)
    if initial.ndim == 0:
        initial = np.full((n_theta, n_phi), float(initial))
    radius = initial.copy()
    history, previous_mass = [], None
    while True:
        for iteration in range(max_iterations + 1):
            expansion, density, usable = surface(radius, center, sample)
            residual_norm = float(np.mean(radius) * np.max(np.abs(expansion)))
            if not usable:
                raise RuntimeError("Surface leaves the resolved domain or has nonphysical geometry")
            if residual_norm < tolerance:
                break
            if iteration == max_iterations:
                raise RuntimeError(f"Newton did not converge after {max_iterations} iterations: {residual_norm:.3e}")
            delta = np.linalg.solve(jacobian(radius, center, sample), -expansion.reshape(-1)).reshape(radius.shape)
            step = min(1.0, float(0.1 * np.mean(radius) / np.max(np.abs(delta))))
            for _ in range(20):
                trial = radius + step * delta
                te, _, tu = surface(trial, center, sample)
                tn = float(np.mean(trial) * np.max(np.abs(te)))
                if tu and tn < residual_norm * (1 - 1.e-4 * step):
                    radius = trial
                    break
                step *= 0.5
            else:
                raise RuntimeError(f"Newton line search stalled at residual {residual_norm:.3e}")
        nt, nphi = radius.shape
        theta, phi, weights = angular_grid(nt, nphi)
        area = float(np.sum(weights[:, None] * density) * (2 * np.pi / nphi))
        mass = np.sqrt(area / (16 * np.pi))
        at_, ap_, _ = angular_grid(2 * nt + 2, 2 * nphi + 2)
        audit_radius = interpolate_angular(radius, at_, ap_)
        audit_expansion, _, audit_usable = surface(audit_radius, center, sample)
        if not audit_usable:
            raise RuntimeError("Angular audit leaves the resolved domain or has nonphysical geometry")
        audit = float(np.mean(audit_radius) * np.max(np.abs(audit_expansion)))
        mass_change = np.inf if previous_mass is None else abs(mass / previous_mass - 1)
        history.append((nt, nphi, mass, residual_norm, audit, iteration))
        if previous_mass is not None and audit < audit_tolerance and mass_change < mass_tolerance:
            return dict(theta=theta, phi=phi, radius=radius, center=center, expansion=expansion, area=area,
                        mass=float(mass), residual=residual_norm, audit_residual=audit,
                        mass_relative_change=mass_change, convergence=np.asarray(history),
                        iterations=sum(int(row[5]) for row in history))
        if 2 * nt > max_angular:
            raise RuntimeError(f"Angular convergence failed: audit={audit:.3e}, mass change={mass_change:.3e}")
        theta, phi, _ = angular_grid(2 * nt, 2 * nphi)
        radius = interpolate_angular(radius, theta, phi)
        previous_mass = mass
