"""Cartoon reconstructions and steppers, restated in NumPy (test infrastructure).

Axisymmetric (z axis) Cartoon, uwplasma/JAX_BSSN:
  parity ghosts / compact storage        JAX_BSSN/cartoon/axisymmetry/reconstruction.py:34-143
  1/r outer buffer, support geometry     reconstruction.py:146-178
  six-node non-periodic Lagrange         JAX_BSSN/cartoon/interpolation.py:9-87
  rotation onto the nine y planes        reconstruction.py:206-289
  centre-plane projection of the RHS     reconstruction.py:292-300
  RK4 with per-stage preparation         JAX_BSSN/cartoon/axisymmetry/evolution.py:18-65
  constraints and |rho|-weighted norms   JAX_BSSN/cartoon/axisymmetry/diagnostics.py:22-78
Spherical Cartoon:
  symmetric-subspace projection          JAX_BSSN/cartoon/spherical_symmetry/reconstruction.py:147-189
  radial profiles, 9x9 support           reconstruction.py:192-385
  RK4                                    JAX_BSSN/cartoon/spherical_symmetry/evolution.py:17-72
  constraints, norms                     JAX_BSSN/cartoon/spherical_symmetry/diagnostics.py:21-111
Sums over the six interpolation nodes and the rotation contractions are
accumulated in the reference's order (see tests/golden/make_golden.py).
"""

from __future__ import annotations

import numpy as np

from . import bssn as ob
from .state import BSSNVariables

GHOSTS = 4
SUPPORT = 9
CENTER = 4
BUFFER = 3
AXI_PARITY = (-1.0, -1.0, 1.0)
SPH_PARITY = (-1.0, 1.0, 1.0)
ASYMPTOTES = ("flat", 1.0, 0.0, 0.0, 0.0, 1.0, 0.0)


def _parity(rank, signs):
    p = np.asarray(signs)
    if rank == 0:
        return np.asarray(1.0)
    if rank == 1:
        return p
    return p[:, None] * p[None, :]


def _rank(leaf, spatial=3):
    return np.ndim(leaf) - spatial


def _seq_sum(arrays):
    acc = arrays[0]
    for a in arrays[1:]:
        acc = acc + a
    return acc


def _reflect(positive, parity, axis, count=None):
    """Mirror the first ``count`` samples (all when None) across the origin."""
    axis = axis % positive.ndim
    parity = np.asarray(parity)
    parity = parity.reshape(parity.shape + (1,) * (positive.ndim - parity.ndim))
    index = [slice(None)] * positive.ndim
    index[axis] = slice(None, count)
    mirrored = np.flip(positive[tuple(index)], axis=axis) * parity
    return np.concatenate((mirrored, positive), axis=axis)


def lagrange6(q, size):
    """Nodes and weights of the clipped six-node stencil (interpolation.py:9-57)."""
    q = np.asarray(q)
    base = np.floor(q).astype(np.int32)
    start = np.clip(base - 2, 0, size - 6)
    nodes = start[..., None] + np.arange(6, dtype=np.int32)
    w = np.ones(nodes.shape)
    for k in range(6):
        for m in range(6):
            if k != m:
                w[..., k] = w[..., k] * ((q - nodes[..., m]) / (nodes[..., k] - nodes[..., m]))
    return nodes, w


def interpolate(source, q, axis):
    """lagrange6_nonperiodic along ``axis`` with NaN outside the samples."""
    axis = axis % source.ndim
    size = source.shape[axis]
    nodes, w = lagrange6(q, size)
    moved = np.moveaxis(source, axis, -1)
    gathered = np.take(moved, nodes, axis=-1)
    lead = moved.shape[:-1]
    prod = gathered * w.reshape((1,) * len(lead) + w.shape)
    value = _seq_sum([prod[..., k] for k in range(6)])
    tdim = nodes.ndim - 1
    perm = tuple(range(axis)) + tuple(range(source.ndim - 1, source.ndim - 1 + tdim)) + \
        tuple(range(axis, source.ndim - 1))
    value = np.transpose(value, perm)
    valid = (q >= 0) & (q <= size - 1)
    vshape = (1,) * axis + valid.shape + (1,) * (source.ndim - axis - 1)
    return np.where(valid.reshape(vshape), value, np.nan)


def _rotate_tensor(R, T):
    out = np.empty(R.shape[:2] + np.broadcast_shapes(R.shape[2:], T.shape[2:]))
    for i in range(3):
        for j in range(3):
            out[i, j] = _seq_sum([(R[i, a] * R[j, b]) * T[a, b] for a in range(3) for b in range(3)])
    return out


def _rotate_vector(R, v):
    return np.stack([_seq_sum([R[i, j] * v[j] for j in range(3)]) for i in range(3)])


# ----------------------------------------------------------------------------
# axisymmetric Cartoon
# ----------------------------------------------------------------------------

def axi_positive(field):
    return np.asarray(field)[..., GHOSTS:, 0, :]


def axi_compact(positive, parity):
    return np.expand_dims(_reflect(positive, parity, axis=-2, count=GHOSTS), axis=-2)


def axi_fill_ghosts(v):
    return BSSNVariables(*(axi_compact(axi_positive(f), _parity(_rank(f), AXI_PARITY)) for f in v))


def _axi_outer_buffer(reference, asymptotic, p):
    nx, nz = reference.shape[-2:]
    dx = np.float64(p.dx)
    rho_edge = (nx - GHOSTS - 0.5) * dx
    z = np.float64(p.z_min) + dx * np.arange(nz, dtype=np.float64)
    rho_buffer = rho_edge + dx * np.arange(1, BUFFER + 1, dtype=np.float64)
    r_edge = np.sqrt(rho_edge * rho_edge + z * z)
    r_buffer = np.sqrt(rho_buffer[:, None] * rho_buffer[:, None] + z[None, :] * z[None, :])
    ratio = r_edge[None, :] / r_buffer
    asymptotic = np.asarray(asymptotic, dtype=np.float64)
    lead = reference.ndim - 2
    asymptotic = asymptotic.reshape(asymptotic.shape + (1, 1))
    buffer = asymptotic + (reference[..., -1:, :] - asymptotic) * ratio.reshape((1,) * lead + ratio.shape)
    return np.concatenate((reference, buffer), axis=-2)


def axi_geometry(num_x, p):
    dx = np.float64(p.dx)
    x = (np.arange(num_x, dtype=np.float64) - 3.5) * dx
    y = (np.arange(SUPPORT, dtype=np.float64) - 4.0) * dx
    X, Y = np.broadcast_arrays(x[:, None], y[None, :])
    return np.sqrt(X * X + Y * Y), X, Y


def axi_rotation(X, Y):
    rho = np.sqrt(X * X + Y * Y)
    on_axis = rho <= 0.0
    safe = np.where(on_axis, 1.0, rho)
    c = np.where(on_axis, 1.0, X / safe)
    s = np.where(on_axis, 0.0, Y / safe)
    zero, one = np.zeros_like(X), np.ones_like(X)
    return np.stack((np.stack((c, s, zero)), np.stack((-s, c, zero)), np.stack((zero, zero, one))), axis=1)


def axi_radial_interpolate(positive, rho, p, parity, asymptotic):
    plane = _reflect(positive, parity, axis=-2, count=GHOSTS)
    source = _axi_outer_buffer(plane, asymptotic, p)
    q = rho / np.float64(p.dx) + GHOSTS - 0.5
    return interpolate(source, q, axis=-2)


def axi_reconstruct(v, p):
    num_x = np.asarray(v.conformal_factor).shape[0]
    rho, X, Y = axi_geometry(num_x, p)
    R = axi_rotation(X[..., None], Y[..., None])
    out = []
    for f, asym in zip(v, ASYMPTOTES):
        rank = _rank(f)
        parity = _parity(rank, AXI_PARITY)
        asym = np.eye(3) if asym == "flat" else (np.zeros((3,) * rank) + asym if rank else asym)
        prof = axi_radial_interpolate(axi_positive(f), rho, p, parity, asym)
        if rank == 2:
            prof = _rotate_tensor(R, prof)
        elif rank == 1:
            prof = _rotate_vector(R, prof)
        out.append(prof)
    return BSSNVariables(*out)


def axi_project_rhs(rhs):
    return BSSNVariables(*(axi_compact(np.asarray(f)[..., GHOSTS:, CENTER, :], _parity(_rank(f), AXI_PARITY))
                           for f in rhs))


def axi_rhs(v, p):
    return axi_project_rhs(ob.compute_rhs(axi_reconstruct(v, p), p))


def _prepare(v):
    return axi_fill_ghosts(ob.project(v))


def _add(v, k, scale):
    return BSSNVariables(*(a + scale * b for a, b in zip(v, k)))


def axi_rk4_step(v, p):
    dt = p.dt
    v = _prepare(v)
    k1 = axi_rhs(v, p)
    k2 = axi_rhs(_prepare(_add(v, k1, 0.5 * dt)), p)
    k3 = axi_rhs(_prepare(_add(v, k2, 0.5 * dt)), p)
    k4 = axi_rhs(_prepare(_add(v, k3, dt)), p)
    new = BSSNVariables(*(f + (dt / 6.0) * (a + 2.0 * b + 2.0 * c + d) for f, a, b, c, d in zip(v, k1, k2, k3, k4)))
    return _prepare(new)


def axi_constraints(v, p):
    support = axi_reconstruct(v, p)
    H, M, det, trA, gam = ob.constraints(support, p)

    def project(f, rank):
        return axi_compact(np.asarray(f)[..., GHOSTS:, CENTER, :], _parity(rank, AXI_PARITY))

    return project(H, 0), project(M, 1), project(det, 0), project(trA, 0), project(gam, 1)


def axi_constraint_norms(violations, exclude_outer_rho=4, exclude_z=4, p=None):
    names = ("hamiltonian", "momentum", "det_gamma", "trace_A", "gamma")

    def physical(f):
        f = np.asarray(f)[..., GHOSTS:, 0, :]
        if exclude_outer_rho:
            f = f[..., :-exclude_outer_rho, :]
        if exclude_z:
            f = f[..., exclude_z:-exclude_z]
        return f

    H = violations[0]
    if p is not None:
        nx = np.asarray(H).shape[0]
        rho = np.float64(p.x_min) + np.float64(p.dx) * (np.arange(nx, dtype=np.float64) + 0.0)
        full = np.broadcast_to(np.abs(rho)[:, None], (nx, np.asarray(H).shape[-1]))
        weight_full = physical(full[:, None, :])
    out = {}
    for name, f in zip(names, violations):
        f = physical(f)
        nrho, nz = f.shape[-2:]
        w = np.broadcast_to((np.arange(nrho, dtype=np.float64) + 0.5)[:, None], (nrho, nz)) if p is None \
            else weight_full
        comps = int(np.prod(f.shape[:-2])) if f.ndim > 2 else 1
        out[name + "_l2"] = float(np.sqrt(np.sum(w * f ** 2) / (np.sum(w) * comps)))
        out[name + "_linf"] = float(np.max(np.abs(f)))
    return out


# ----------------------------------------------------------------------------
# spherical Cartoon
# ----------------------------------------------------------------------------

def sph_positive(field):
    f = np.asarray(field)
    line = f[..., :, 0, 0] if f.shape[-2:] == (1, 1) else f[..., :, CENTER, CENTER]
    return line[..., GHOSTS:]


def sph_compact(positive, parity):
    return _reflect(positive, parity, axis=-1, count=GHOSTS)[..., :, None, None]


def _symmetric_subspace(pos):
    rank = pos.ndim - 1
    if rank == 0:
        return pos
    zero = np.zeros_like(pos[(0,) * rank])
    if rank == 1:
        return np.stack((pos[0], zero, zero))
    t = pos[1, 1]
    return np.stack((np.stack((pos[0, 0], zero, zero)), np.stack((zero, t, zero)), np.stack((zero, zero, t))))


def sph_enforce_symmetry(v):
    return BSSNVariables(*(sph_compact(_symmetric_subspace(sph_positive(f)), _parity(_rank(f), SPH_PARITY))
                           for f in v))


def _sph_buffer(axis, asymptotic, dx):
    spacing = np.float64(dx)
    asym = np.broadcast_to(np.asarray(asymptotic, dtype=np.float64), axis.shape[:-1])[..., None]
    outer = (axis.shape[-1] - GHOSTS - 0.5) * spacing
    radius = outer + spacing * np.arange(1, BUFFER + 1, dtype=np.float64)
    buffer = asym + (axis[..., -1:] - asym) * (outer / radius)
    return np.concatenate((axis, buffer), axis=-1)


def sph_radial_interpolate(positive, radius, dx, parity, asymptotic):
    axis = _reflect(positive, parity, axis=-1, count=GHOSTS)
    axis = _sph_buffer(axis, asymptotic, dx)
    q = radius / np.float64(dx) + GHOSTS - 0.5
    return interpolate(axis, q, axis=-1)


def sph_geometry(num_x, dx):
    spacing = np.float64(dx)
    x = (np.arange(num_x, dtype=np.float64) - GHOSTS + 0.5) * spacing
    t = (np.arange(SUPPORT, dtype=np.float64) - CENTER) * spacing
    X, Y, Z = np.broadcast_arrays(x[:, None, None], t[None, :, None], t[None, None, :])
    return np.sqrt(X * X + Y * Y + Z * Z), X, Y, Z


def sph_rotation(x, y, z):
    r = np.sqrt(x * x + y * y + z * z)
    rho = np.sqrt(x * x + y * y)
    safe = np.where(rho > 0.0, rho, 1.0)
    zero, one = np.zeros_like(x), np.ones_like(x)
    off = (rho > 0.0)[None]
    radial = np.stack((x / r, y / r, z / r))
    azimuthal = np.where(off, np.stack((-y / safe, x / safe, zero)), np.stack((zero, one, zero)))
    polar = np.where(off, np.stack((-x * z / (r * safe), -y * z / (r * safe), rho / r)),
                     np.stack((-z / r, zero, zero)))
    return np.stack((radial, azimuthal, polar), axis=1)


def sph_reconstruct(v, p):
    num_x = np.asarray(v.conformal_factor).shape[0]
    radius, X, Y, Z = sph_geometry(num_x, p.dx)
    R = sph_rotation(X, Y, Z)

    def prof(field, asym, parity=1.0):
        return sph_radial_interpolate(sph_positive(field), radius, p.dx, parity, asym)

    def tensor(radial, tangential):
        zero = np.zeros_like(radial)
        T = np.stack((np.stack((radial, zero, zero)), np.stack((zero, tangential, zero)),
                      np.stack((zero, zero, tangential))))
        return _rotate_tensor(R, T)

    def vector(radial):
        zero = np.zeros_like(radial)
        return _rotate_vector(R, np.stack((radial, zero, zero)))

    g, A = np.asarray(v.conformal_metric), np.asarray(v.traceless_K)
    return BSSNVariables(
        tensor(prof(g[0, 0], 1.0), prof(g[1, 1], 1.0)),
        prof(v.conformal_factor, 1.0),
        tensor(prof(A[0, 0], 0.0), prof(A[1, 1], 0.0)),
        prof(v.trace_K, 0.0),
        vector(prof(np.asarray(v.conformal_connection)[0], 0.0, SPH_PARITY[0])),
        prof(v.lapse, 1.0),
        vector(prof(np.asarray(v.shift)[0], 0.0, SPH_PARITY[0])),
    )


def sph_project_rhs(rhs):
    return BSSNVariables(*(sph_compact(np.asarray(f)[..., GHOSTS:, CENTER, CENTER], _parity(_rank(f), SPH_PARITY))
                           for f in rhs))


def sph_rhs(v, p):
    return sph_project_rhs(ob.compute_rhs(sph_reconstruct(v, p), p))


def _sph_prepare(v):
    return ob.project(sph_enforce_symmetry(v))


def sph_rk4_step(v, p):
    dt = p.dt
    v = _sph_prepare(v)
    k1 = sph_rhs(v, p)
    k2 = sph_rhs(_sph_prepare(_add(v, k1, 0.5 * dt)), p)
    k3 = sph_rhs(_sph_prepare(_add(v, k2, 0.5 * dt)), p)
    k4 = sph_rhs(_sph_prepare(_add(v, k3, dt)), p)
    new = BSSNVariables(*(f + (dt / 6.0) * (a + 2.0 * b + 2.0 * c + d) for f, a, b, c, d in zip(v, k1, k2, k3, k4)))
    return _sph_prepare(new)


def sph_constraints(v, p):
    """compute_cartoon_constraints (spherical_symmetry/diagnostics.py:21-37)."""
    support = sph_reconstruct(v, p)
    H, M, det, trA, gam = ob.constraints(support, p)

    def project(f, rank):
        return sph_compact(np.asarray(f)[..., GHOSTS:, CENTER, CENTER], _parity(rank, SPH_PARITY))

    return project(H, 0), project(M, 1), project(det, 0), project(trA, 0), project(gam, 1)


def _radius_norms(fields, exclude_outer):
    out = {}
    for name, f in fields.items():
        f = sph_positive(f)
        if exclude_outer:
            f = f[..., :-exclude_outer]
        out[name + "_l2"] = float(np.sqrt(np.mean(f ** 2)))
        out[name + "_linf"] = float(np.max(np.abs(f)))
    return out


def sph_constraint_norms(violations, exclude_outer=4):
    """compute_cartoon_constraint_norms (spherical_symmetry/diagnostics.py:40-65)."""
    names = ("hamiltonian", "momentum", "det_gamma", "trace_A", "gamma")
    return _radius_norms(dict(zip(names, violations)), exclude_outer)


def sph_symmetry_norms(v, exclude_outer=0):
    """compute_spherical_symmetry_norms (spherical_symmetry/diagnostics.py:68-111)."""
    g, A = np.asarray(v.conformal_metric), np.asarray(v.traceless_K)
    beta, gam = np.asarray(v.shift), np.asarray(v.conformal_connection)
    errors = {"metric_tangential": g[1, 1] - g[2, 2], "A_tangential": A[1, 1] - A[2, 2],
              "metric_xy": g[0, 1], "metric_xz": g[0, 2], "metric_yz": g[1, 2],
              "A_xy": A[0, 1], "A_xz": A[0, 2], "A_yz": A[1, 2],
              "shift_y": beta[1], "shift_z": beta[2], "connection_y": gam[1], "connection_z": gam[2]}
    return _radius_norms(errors, exclude_outer)
