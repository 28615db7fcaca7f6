"""Stage-synchronous FMR on one device, restated in NumPy (test infrastructure).

Follows uwplasma/JAX_BSSN for a (1, 1, 1) tile topology -- every patch is a
single padded array of (n + 2g)^3 samples with g = 4 guards:
  patch spacing/origin/MAD policy       JAX_BSSN/fmr/tiled.py:39-48, 105-143
  halo refresh (self-wrap, linear exterior)   JAX_BSSN/parallel/evolution.py:74-92, communication.py:36-106
  tile-local parameters                 JAX_BSSN/parallel/evolution.py:19-38
  six-node Lagrange prolongation        JAX_BSSN/fmr/transfer.py:57-142, 197-244
  injection                             JAX_BSSN/fmr/transfer.py:145-171, 247-252
  prepare / stage / RK4 step            JAX_BSSN/fmr/tiled.py:146-209
  composite constraint norms            JAX_BSSN/fmr/tiled.py:212-246
Fields are BSSNVariables whose leaves have shape (..., n+2g, n+2g, n+2g); the
reference's three singleton tile axes are dropped.
"""

from __future__ import annotations

import math
from typing import NamedTuple

import numpy as np

from . import bssn as ob
from .state import BSSNParameters, BSSNVariables

GUARD = 4
FACE_NAMES = ("xl_bc", "xr_bc", "yl_bc", "yr_bc", "zl_bc", "zr_bc")


class FMRPatchSpec(NamedTuple):
    coarse_lo: tuple
    coarse_hi: tuple
    refinement_ratio: int = 2
    ghost_width: int = 4
    parent: int | None = None


class FMRHierarchySpec(NamedTuple):
    patches: tuple
    use_mad: bool = True


def parents_of(hierarchy):
    parents = [-1]
    for child, spec in enumerate(hierarchy.patches, start=1):
        parents.append(child - 1 if spec.parent is None else spec.parent)
    return tuple(parents)


def fine_active_shape(spec):
    return tuple(2 * (h - l) + 1 for l, h in zip(spec.coarse_lo, spec.coarse_hi))


def evolution_parameters(parameters, hierarchy):
    """mad_q = (dx_finest/dx)^4 per patch; child faces periodic (tiled.py:39-48)."""
    finest = min(p.dx for p in parameters)
    out = []
    for patch, p in enumerate(parameters):
        changes = dict(mad_q=(finest / p.dx) ** 4 if hierarchy.use_mad else 1.0)
        if patch:
            changes.update({name: 0 for name in FACE_NAMES})
        out.append(p._replace(**changes))
    return tuple(out)


def patch_parameters(root_params, root_shape, hierarchy):
    """Per-patch spacing and active origins (tiled.py:120-127)."""
    parents = parents_of(hierarchy)
    reduced = (tuple(n == 1 for n in root_shape) if root_params.reduced_axes is None
               else root_params.reduced_axes)
    params = [root_params._replace(guard_cells=0, owned_shape=None, reduced_axes=reduced)]
    shapes = [tuple(root_shape)]
    for child, spec in enumerate(hierarchy.patches, start=1):
        parent = params[parents[child]]
        origin = tuple(getattr(parent, name) + lo * parent.dx
                       for name, lo in zip(("x_min", "y_min", "z_min"), spec.coarse_lo))
        params.append(parent._replace(dx=parent.dx / 2, x_min=origin[0], y_min=origin[1], z_min=origin[2],
                                      **{name: 0 for name in FACE_NAMES}))
        shapes.append(fine_active_shape(spec))
    return evolution_parameters(tuple(params), hierarchy), tuple(shapes)


def local_parameters(p, shape):
    """Tile-local parameters of a single padded patch (parallel/evolution.py:19-38)."""
    minima = tuple(origin + (0 - GUARD) * p.dx for origin in (p.x_min, p.y_min, p.z_min))
    reduced = p.reduced_axes if p.reduced_axes is not None else tuple(n == 1 for n in shape)
    return p._replace(x_min=minima[0], y_min=minima[1], z_min=minima[2], guard_cells=GUARD,
                      owned_shape=tuple(shape), owned_faces=(True,) * 6, reduced_axes=reduced)


# ----------------------------------------------------------------------------
# halo refresh of one patch (parallel/evolution.py:74-92; communication.py:36-106, count == 1)
# ----------------------------------------------------------------------------

def _plane(axis, index):
    s = [slice(None)] * 3
    s[axis] = index
    return (Ellipsis,) + tuple(s)


def refresh_field(a, codes, n):
    a = np.array(a, copy=True)
    g = GUARD
    for axis in range(3):
        spatial_axis = a.ndim - 3 + axis
        size = a.shape[spatial_axis]
        nodes = g + (np.arange(size) - g) % n[axis]
        a = np.take(a, nodes, axis=spatial_axis)
        for side in (0, 1):
            if not codes[2 * axis + side]:
                continue
            boundary = g if side == 0 else g + n[axis] - 1
            targets = np.arange(g) if side == 0 else np.arange(g + n[axis], n[axis] + 2 * g)
            base = np.take(a, [boundary], axis=spatial_axis)
            inward = boundary + (1 if side == 0 else -1)
            neighbour = np.take(a, [inward], axis=spatial_axis)
            slope = neighbour - base if side == 0 else base - neighbour
            shape = [1] * a.ndim
            shape[spatial_axis] = g
            values = base + (targets - boundary).reshape(shape) * slope
            a[_plane(axis, slice(int(targets[0]), int(targets[-1]) + 1))] = values
    return a


def refresh(state, p, n):
    codes = tuple(int(getattr(p, name)) for name in FACE_NAMES)
    return BSSNVariables(*(refresh_field(np.asarray(f), codes, n) for f in state))


# ----------------------------------------------------------------------------
# prolongation and injection (transfer.py)
# ----------------------------------------------------------------------------

def lagrange_weights(targets, nodes):
    """Degree-5 Lagrange basis at targets for each row of six nodes (transfer.py:57-69)."""
    coefficient = np.ones(nodes.shape)
    for k in range(6):
        for m in range(6):
            if k != m:
                coefficient[:, k] *= (targets - nodes[:, m]) / (nodes[:, k] - nodes[:, m])
    return coefficient


def _axis_segments(spec, axis, child_n):
    """Per child padded index along one axis: (segment id, parent local target)."""
    out = []
    for local in range(child_n + 2 * GUARD):
        fine = local - GUARD
        target = spec.coarse_lo[axis] + fine / 2
        exterior = -1 if fine < 0 else (1 if fine >= child_n else 0)
        out.append((exterior, target + GUARD))
    return out


def _sequential_sum(values, axis):
    """Sum along a short axis left to right (the order XLA's reduce loop uses)."""
    moved = np.moveaxis(values, axis, 0)
    acc = moved[0]
    for k in range(1, moved.shape[0]):
        acc = acc + moved[k]
    return acc


def prolong(parent, child, spec, child_n):
    """Replace the child's exterior shell by separable six-node Lagrange
    interpolation of the prepared parent (transfer.py:114-142, 205-244)."""
    segs = [_axis_segments(spec, a, child_n[a]) for a in range(3)]
    out = [np.array(np.asarray(c), copy=True) for c in child]
    groups = []
    for a in range(3):
        ids = {}
        for local, (ext, t) in enumerate(segs[a]):
            ids.setdefault(ext, []).append((local, t))
        groups.append(ids)
    for ex in groups[0]:
        for ey in groups[1]:
            for ez in groups[2]:
                if ex == 0 and ey == 0 and ez == 0:
                    continue
                pts = (groups[0][ex], groups[1][ey], groups[2][ez])
                for leaf, (p_leaf, c_leaf) in enumerate(zip(parent, out)):
                    window = np.asarray(p_leaf)
                    lead = window.ndim - 3
                    for a in range(3):
                        targets = np.asarray([t for _, t in pts[a]])
                        nodes = np.floor(targets).astype(np.int64)[:, None] + np.arange(-2, 4)
                        weights = lagrange_weights(targets, nodes)
                        gathered = np.take(window, nodes, axis=lead + a)      # (..., T, 6, ...)
                        wshape = [1] * gathered.ndim
                        wshape[lead + a:lead + a + 2] = weights.shape
                        window = _sequential_sum(gathered * weights.reshape(wshape), lead + a + 1)
                    idx = tuple(np.asarray([l for l, _ in pts[a]]) for a in range(3))
                    c_leaf[(Ellipsis,) + np.ix_(*idx)] = window
    return BSSNVariables(*out)


def inject(parent, child, spec, child_n):
    """Copy coincident owned fine vertices into the parent (transfer.py:145-171)."""
    out = [np.array(np.asarray(p), copy=True) for p in parent]
    src = [np.arange(0, child_n[a], 2) + GUARD for a in range(3)]
    dst = [spec.coarse_lo[a] + np.arange(0, child_n[a], 2) // 2 + GUARD for a in range(3)]
    for o, c in zip(out, child):
        o[(Ellipsis,) + np.ix_(*dst)] = np.asarray(c)[(Ellipsis,) + np.ix_(*src)]
    return BSSNVariables(*out)


# ----------------------------------------------------------------------------
# stages and the RK4 step (tiled.py:146-209)
# ----------------------------------------------------------------------------

def _owned(shape_n):
    return tuple(slice(GUARD, GUARD + n) for n in shape_n)


def project_owned(state, n):
    sl = (Ellipsis,) + _owned(n)
    proj = ob.project(BSSNVariables(*(np.asarray(f)[sl] for f in state)))
    out = []
    for f, q in zip(state, proj):
        f = np.array(f, copy=True)
        f[sl] = q
        out.append(f)
    return BSSNVariables(*out)


def prepare(states, params, shapes, hierarchy, project=True):
    parents = parents_of(hierarchy)
    prepared = []
    for patch, (state, p, n) in enumerate(zip(states, params, shapes)):
        if project:
            state = project_owned(state, n)
        state = refresh(state, p, n)
        if patch:
            state = prolong(prepared[parents[patch]], state, hierarchy.patches[patch - 1], n)
        prepared.append(state)
    return tuple(prepared)


def rhs(states, params, shapes):
    return tuple(ob.compute_rhs(state, local_parameters(p, n)) for state, p, n in zip(states, params, shapes))


def stage(states, params, shapes, hierarchy):
    prepared = prepare(states, params, shapes, hierarchy)
    return prepared, rhs(prepared, params, shapes)


def _combine(a, b, fn):
    return tuple(BSSNVariables(*(fn(x, y) for x, y in zip(sa, sb))) for sa, sb in zip(a, b))


def rk4_step(states, params, shapes, hierarchy):
    dt = params[0].dt
    s0, k1 = stage(states, params, shapes, hierarchy)
    _, k2 = stage(_combine(s0, k1, lambda q, k: q + dt * k / 2), params, shapes, hierarchy)
    _, k3 = stage(_combine(s0, k2, lambda q, k: q + dt * k / 2), params, shapes, hierarchy)
    _, k4 = stage(_combine(s0, k3, lambda q, k: q + dt * k), params, shapes, hierarchy)
    result = []
    for q, a, b, c, d in zip(s0, k1, k2, k3, k4):
        result.append(BSSNVariables(*(qq + dt * (aa + 2 * bb + 2 * cc + dd) / 6
                                      for qq, aa, bb, cc, dd in zip(q, a, b, c, d))))
    result = [project_owned(s, n) for s, n in zip(result, shapes)]
    parents = parents_of(hierarchy)
    for child in range(len(result) - 1, 0, -1):
        parent = parents[child]
        result[parent] = inject(result[parent], result[child], hierarchy.patches[child - 1], shapes[child])
        result[parent] = project_owned(result[parent], shapes[parent])
    return prepare(tuple(result), params, shapes, hierarchy, project=False)


def constraint_norms(states, params, shapes, hierarchy):
    """Composite point-count L2/Linf over uncovered owned vertices (tiled.py:212-246)."""
    prepared = prepare(states, params, shapes, hierarchy, project=False)
    parents = parents_of(hierarchy)
    names = ("hamiltonian", "momentum", "det_gamma", "trace_A", "gamma")
    totals = {name: [0, 0.0, 0.0] for name in names}
    for patch, (state, p, n) in enumerate(zip(prepared, params, shapes)):
        values = ob.constraints(state, local_parameters(p, n))
        mask = np.zeros(np.asarray(state.lapse).shape, dtype=bool)
        mask[_owned(n)] = True
        for child, spec in enumerate(hierarchy.patches, start=1):
            if parents[child] != patch:
                continue
            cover = tuple(slice(GUARD + lo, GUARD + hi + 1) for lo, hi in zip(spec.coarse_lo, spec.coarse_hi))
            mask[cover] = False
        for name, field in zip(names, values):
            comps = math.prod(field.shape[:-3])
            totals[name][0] += int(mask.sum()) * comps
            totals[name][1] += float(np.sum(np.where(mask, field ** 2, 0.0)))
            totals[name][2] = max(totals[name][2], float(np.max(np.where(mask, np.abs(field), 0.0))))
    out = {}
    for name, (count, square, peak) in totals.items():
        out[name + "_l2"] = math.sqrt(square / count)
        out[name + "_linf"] = peak
    return out
