"""Stage-synchronous FMR on GB300 (mirrors JAX_BSSN/fmr/tiled.py).

Same names and arguments as the reference: ``initialize_tiled_fmr``,
``validate_hierarchy``, ``prepare_fmr_states``, ``fmr_stage``,
``fmr_rk4_step`` and ``fmr_constraint_norms`` take and return tuples of
``BSSNVariables`` in the reference's tiled layout -- leaves shaped
(..., 1, 1, 1, n+8, n+8, n+8) for the single-device tile topology a GPU
serves -- and the per-patch ``BSSNParameters``.  The work runs in
``libbssn_gb300.so`` (``bssn_fmr_*``).  ``FMREvolution`` keeps the patches
resident in the kernels' 21-component layout for repeated steps.
"""

from __future__ import annotations

import ctypes
import math
from typing import NamedTuple

import numpy as np
import torch

from .. import _device, _native
from .._graph import GraphSteps
from ..bssn.variables import BSSNParameters, BSSNVariables
from .refinement import fine_active_shape, hierarchy_parents

FACE_NAMES = ("xl_bc", "xr_bc", "yl_bc", "yr_bc", "zl_bc", "zr_bc")
GUARD = 4
NCOMP = 21
CONSTRAINT_NAMES = ("hamiltonian", "momentum", "det_gamma", "trace_A", "gamma")
CONSTRAINT_COMPONENTS = (1, 3, 1, 1, 3)


class TileLayout(NamedTuple):
    """One patch on one device: owned extent and guard depth
    (JAX_BSSN/parallel/layout.py:29-89 with a (1, 1, 1) mesh)."""
    tile_shape: tuple
    guard_cells: int = GUARD
    upper_endpoints: tuple = (False, False, False)

    @property
    def counts(self):
        return (1, 1, 1)

    @property
    def active_shape(self):
        return tuple(int(n) + int(e) for n, e in zip(self.tile_shape, self.upper_endpoints))

    @property
    def allocated_shape(self):
        return tuple(int(n) + 2 * self.guard_cells for n in self.tile_shape)


def patch_layout(shape, mesh=None):
    if mesh is not None and tuple(getattr(mesh, "devices", np.empty((1, 1, 1))).shape) != (1, 1, 1):
        raise ValueError("the GB300 FMR path runs every patch as a single tile on one GPU")
    return TileLayout(tuple(int(n) for n in shape), GUARD, (False, False, False))


def _layout_shape(layout):
    counts = tuple(getattr(layout, "counts", (1, 1, 1)))
    if counts != (1, 1, 1):
        raise ValueError("the GB300 FMR path runs every patch as a single tile on one GPU")
    if int(layout.guard_cells) != GUARD or any(layout.upper_endpoints):
        raise ValueError("FMR patches need exactly four guards and no owned upper endpoint")
    return tuple(int(n) for n in layout.tile_shape)


def evolution_parameters(parameters, hierarchy):
    """Finest spacing for MAD, bulk equations on children (tiled.py:39-48)."""
    finest = min(p.dx for p in parameters)
    out = []
    for patch, p in enumerate(parameters):
        changes = dict(mad_q=(finest / p.dx) ** 4 if hierarchy.use_mad else 1.0)
        if patch:
            changes.update({name: 0 for name in FACE_NAMES})
        out.append(p._replace(**changes))
    return tuple(out)


def validate_hierarchy(states, parameters, hierarchy, layouts):
    """Host-side checks of the reference (tiled.py:51-102), before any launch."""
    parents = hierarchy_parents(hierarchy)
    if not parameters or not len(parameters) == len(layouts) == len(parents):
        raise ValueError("FMR requires one parameter tuple and one layout per patch")
    if states is not None and len(states) != len(parents):
        raise ValueError("FMR requires one state per patch")
    dt = float(parameters[0].dt)
    if not math.isfinite(dt) or dt <= 0:
        raise ValueError("the shared FMR timestep must be finite and positive")
    root_codes = tuple(int(getattr(parameters[0], name)) for name in FACE_NAMES)
    if any(code not in (0, 1) for code in root_codes):
        raise ValueError("FMR root boundaries support periodic and Sommerfeld codes")
    shapes = [_layout_shape(layout) for layout in layouts]
    for axis in range(3):
        if 1 in root_codes[2 * axis:2 * axis + 2] and shapes[0][axis] < 8:
            raise ValueError("Sommerfeld/KO closures require eight accessible inward samples")
    for child, (params, shape) in enumerate(zip(parameters, shapes)):
        if states is not None:
            expected = tuple(n + 2 * GUARD for n in shape)
            if any(tuple(leaf.shape[-3:]) != expected for leaf in states[child]):
                raise ValueError("FMR state shape does not match its tiled layout")
        if not math.isclose(float(params.dt), dt, rel_tol=1e-5, abs_tol=1e-8):
            raise ValueError("stage-synchronous FMR requires identical timesteps")
        if child:
            parent = parents[child]
            spec = hierarchy.patches[child - 1]
            if shape != fine_active_shape(spec):
                raise ValueError("FMR child active shape does not match its parent bounds")
            if not math.isclose(float(params.dx) * 2, float(parameters[parent].dx), rel_tol=1e-5, abs_tol=1e-8):
                raise ValueError("successive FMR spacings must differ by exactly two")
            parent_shape = shapes[parent]
            if any(lo <= 0 or hi >= n - 1 for lo, hi, n in zip(spec.coarse_lo, spec.coarse_hi, parent_shape)):
                raise ValueError("every child patch must be strictly inside its parent")
            for axis, name in enumerate(("x_min", "y_min", "z_min")):
                origin = getattr(parameters[parent], name) + spec.coarse_lo[axis] * parameters[parent].dx
                if not math.isclose(float(getattr(params, name)), float(origin), rel_tol=1e-5, abs_tol=1e-8):
                    raise ValueError("FMR child active origin is inconsistent with its parent")
            if parent == 0:
                for axis in range(3):
                    lo, hi, n = spec.coarse_lo[axis], spec.coarse_hi[axis], parent_shape[axis]
                    if (lo - 4 < 0 and root_codes[2 * axis] != 0) or (hi + 5 >= n and root_codes[2 * axis + 1] != 0):
                        raise ValueError("FMR interpolation stencil crosses a physical root boundary")
    return shapes


# ----------------------------------------------------------------------------
# C structs and layout conversion
# ----------------------------------------------------------------------------

def _plan(parameters, hierarchy, shapes, precision=None):
    parents = hierarchy_parents(hierarchy)
    n = len(shapes)
    patches = (_native.BssnFmrPatch * n)()
    cparams = (_native.BssnParams * n)()
    for p, shape in enumerate(shapes):
        for a in range(3):
            patches[p].n[a] = shape[a]
        patches[p].parent = parents[p]
        if p:
            spec = hierarchy.patches[p - 1]
            for a in range(3):
                patches[p].coarse_lo[a] = spec.coarse_lo[a]
                patches[p].coarse_hi[a] = spec.coarse_hi[a]
        cparams[p] = _device.to_params(parameters[p], precision)
    return patches, cparams


def _padded(shape):
    return tuple(n + 2 * GUARD for n in shape)


def _to_components(state, shape, device):
    """Tiled reference-layout leaves -> one 21 x (n+8)^3 component buffer."""
    P = _padded(shape)
    leaves = []
    for leaf, lead in zip(state, _device.LEAF_SHAPES):
        t = leaf if isinstance(leaf, torch.Tensor) else torch.as_tensor(np.asarray(leaf))
        leaves.append(t.to(device=device, dtype=torch.float64).reshape(lead + P).contiguous())
    u = torch.empty(NCOMP * math.prod(P), dtype=torch.float64, device=device)
    lib = _native.load()
    _native.check(lib.bssn_fields_to_components(_device.fields_struct(leaves), u.data_ptr(), _device.shape3(P),
                                                _device.stream_handle()), "bssn_fields_to_components")
    return u


def _from_components(u, shape, device, tiled=True):
    P = _padded(shape)
    out = _device.empty_state(P, device)
    lib = _native.load()
    _native.check(lib.bssn_components_to_fields(u.data_ptr(), _device.fields_struct(out), _device.shape3(P),
                                                _device.stream_handle()), "bssn_components_to_fields")
    if tiled:
        out = BSSNVariables(*(leaf.reshape(lead + (1, 1, 1) + P) for leaf, lead in zip(out, _device.LEAF_SHAPES)))
    return out


def _pointers(buffers):
    arr = (ctypes.c_void_p * len(buffers))()
    for i, b in enumerate(buffers):
        arr[i] = b.data_ptr()
    return arr


def _is_host(states):
    leaf = states[0].lapse
    return not (isinstance(leaf, torch.Tensor) and leaf.is_cuda)


def _finish(states, host):
    if host:
        return tuple(_device.to_host(s) for s in states)
    return tuple(states)


# ----------------------------------------------------------------------------
# reference API
# ----------------------------------------------------------------------------

def initialize_tiled_fmr(initial, root_params, root_shape, hierarchy, *, mesh=None):
    """Patches from a common ``initial(coordinates, params)`` callback (tiled.py:105-143).

    The callback receives broadcast Cartesian coordinates of a patch's owned
    samples and parameters describing that patch, and returns BSSNVariables
    of owned samples (NumPy or torch).  ``None`` initialises flat spacetime.
    """
    device = _device.require_cuda()
    root_shape = tuple(int(n) for n in root_shape)
    parents = hierarchy_parents(hierarchy)
    layouts = [patch_layout(root_shape, mesh)]
    reduced = (tuple(n == 1 for n in root_shape) if root_params.reduced_axes is None
               else root_params.reduced_axes)
    parameters = [root_params._replace(guard_cells=0, owned_shape=None, reduced_axes=reduced)]
    for child, spec in enumerate(hierarchy.patches, start=1):
        parent = parameters[parents[child]]
        origin = tuple(getattr(parent, name) + lo * parent.dx
                       for name, lo in zip(("x_min", "y_min", "z_min"), spec.coarse_lo))
        parameters.append(parent._replace(dx=parent.dx / 2, x_min=origin[0], y_min=origin[1], z_min=origin[2],
                                          **{name: 0 for name in FACE_NAMES}))
        layouts.append(patch_layout(fine_active_shape(spec), mesh))
    parameters = evolution_parameters(tuple(parameters), hierarchy)
    layouts = tuple(layouts)
    shapes = validate_hierarchy(None, parameters, hierarchy, layouts)
    states = []
    for p, shape in zip(parameters, shapes):
        P = _padded(shape)
        axes = [p.x_min + p.dx * (np.arange(n, dtype=np.float64) + 0.0) for n in shape]
        coords = (axes[0][:, None, None], axes[1][None, :, None], axes[2][None, None, :])
        local = p._replace(guard_cells=0, owned_shape=shape, owned_faces=(True,) * 6)
        if initial is None:
            one = np.ones(shape)
            value = BSSNVariables(np.eye(3)[:, :, None, None, None] * one, one, np.zeros((3, 3) + shape),
                                  np.zeros(shape), np.zeros((3,) + shape), one, np.zeros((3,) + shape))
        else:
            value = initial(coords, local)
        leaves = []
        for leaf, lead in zip(value, _device.LEAF_SHAPES):
            a = leaf.detach().cpu().numpy() if isinstance(leaf, torch.Tensor) else np.asarray(leaf)
            if a.shape != lead + shape:
                raise ValueError("Initial-data callback must return the owned tile shape")
            full = np.zeros(lead + P)
            full[(Ellipsis,) + tuple(slice(GUARD, GUARD + n) for n in shape)] = a
            leaves.append(torch.as_tensor(full, device=device).reshape(lead + (1, 1, 1) + P))
        states.append(BSSNVariables(*leaves))
    states = prepare_fmr_states(tuple(states), parameters, hierarchy, layouts=layouts, project=False)
    return states, parameters, layouts


def prepare_fmr_states(states, parameters, hierarchy, *, layouts, project=True):
    """Project owned samples, refresh halos, prolong child shells (tiled.py:146-166)."""
    shapes = validate_hierarchy(states, parameters, hierarchy, layouts)
    host = _is_host(states)
    device = _device.require_cuda()
    buffers = [_to_components(s, n, device) for s, n in zip(states, shapes)]
    patches, cparams = _plan(parameters, hierarchy, shapes)
    lib = _native.load()
    _native.check(lib.bssn_fmr_prepare(_pointers(buffers), patches, cparams, len(shapes), int(bool(project)),
                                       _device.stream_handle()), "prepare_fmr_states")
    return _finish([_from_components(u, n, device) for u, n in zip(buffers, shapes)], host)


def fmr_stage(states, parameters, hierarchy, *, layouts):
    """Matching stage states and RHS values (tiled.py:169-179).

    The RHS is defined on owned samples; its guard samples are zero."""
    parameters = evolution_parameters(parameters, hierarchy)
    shapes = validate_hierarchy(states, parameters, hierarchy, layouts)
    host = _is_host(states)
    device = _device.require_cuda()
    buffers = [_to_components(s, n, device) for s, n in zip(states, shapes)]
    rhs = [torch.zeros_like(u) for u in buffers]
    patches, cparams = _plan(parameters, hierarchy, shapes)
    lib = _native.load()
    nbytes = lib.bssn_fmr_workspace_bytes(patches, cparams, len(shapes))
    ws = _device.workspace(nbytes, device, tag="fmr")
    _native.check(lib.bssn_fmr_stage_rhs(_pointers(buffers), _pointers(rhs), patches, cparams, len(shapes),
                                         ws.data_ptr(), ws.numel(), _device.stream_handle()), "fmr_stage")
    prepared = _finish([_from_components(u, n, device) for u, n in zip(buffers, shapes)], host)
    rates = _finish([_from_components(u, n, device) for u, n in zip(rhs, shapes)], host)
    return prepared, rates


def fmr_rk4_step(states, parameters, hierarchy, *, layouts):
    """Advance every patch with the same four RK stages and timestep (tiled.py:182-209)."""
    return fmr_rk4_steps(states, parameters, hierarchy, 1, layouts=layouts)


def fmr_rk4_steps(states, parameters, hierarchy, steps, *, layouts):
    states, parameters = tuple(states), tuple(parameters)
    validate_hierarchy(states, parameters, hierarchy, layouts)
    parameters = evolution_parameters(parameters, hierarchy)
    shapes = [_layout_shape(layout) for layout in layouts]
    host = _is_host(states)
    device = _device.require_cuda()
    buffers = [_to_components(s, n, device) for s, n in zip(states, shapes)]
    patches, cparams = _plan(parameters, hierarchy, shapes)
    lib = _native.load()
    nbytes = lib.bssn_fmr_workspace_bytes(patches, cparams, len(shapes))
    ws = _device.workspace(nbytes, device, tag="fmr")
    _native.check(lib.bssn_fmr_rk4_step(_pointers(buffers), patches, cparams, len(shapes), int(steps),
                                        ws.data_ptr(), ws.numel(), _device.stream_handle()), "fmr_rk4_step")
    return _finish([_from_components(u, n, device) for u, n in zip(buffers, shapes)], host)


def _norms_from_stats(stats, parameters, hierarchy, shapes):
    parents = hierarchy_parents(hierarchy)
    points = 0
    for patch, shape in enumerate(shapes):
        owned = math.prod(shape)
        for child, spec in enumerate(hierarchy.patches, start=1):
            if parents[child] == patch:
                owned -= math.prod(h - l + 1 for l, h in zip(spec.coarse_lo, spec.coarse_hi))
        points += owned
    out = {}
    for q, (name, comps) in enumerate(zip(CONSTRAINT_NAMES, CONSTRAINT_COMPONENTS)):
        out[name + "_l2"] = math.sqrt(float(stats[2 * q]) / (points * comps))
        out[name + "_linf"] = float(stats[2 * q + 1])
    return out


def fmr_constraint_norms(states, parameters, hierarchy, *, layouts):
    """Composite point-count norms over uncovered owned vertices (tiled.py:212-246)."""
    parameters = evolution_parameters(parameters, hierarchy)
    shapes = validate_hierarchy(states, parameters, hierarchy, layouts)
    device = _device.require_cuda()
    buffers = [_to_components(s, n, device) for s, n in zip(states, shapes)]
    return _stats(buffers, parameters, hierarchy, shapes, device)


def _stats(buffers, parameters, hierarchy, shapes, device):
    patches, cparams = _plan(parameters, hierarchy, shapes)
    lib = _native.load()
    need = 0
    for shape in shapes:
        cs = math.prod(_padded(shape))
        need = max(need, (3 * 11 + 24) * cs + 9 * math.prod(shape) + 10 * 304)
    ws = _device.workspace(need * 8, device, tag="fmr_stats")
    stats = torch.zeros(10, dtype=torch.float64, device=device)
    _native.check(lib.bssn_fmr_constraint_stats(_pointers(buffers), patches, cparams, len(shapes),
                                                stats.data_ptr(), ws.data_ptr(), ws.numel(),
                                                _device.stream_handle()), "fmr_constraint_norms")
    return _norms_from_stats(stats.cpu().numpy(), parameters, hierarchy, shapes)


class FMREvolution(GraphSteps):
    """All patches resident in the 21-component layout; ``step(n)`` runs n
    stage-synchronous RK4 steps without leaving the device."""

    def __init__(self, states, parameters, hierarchy, layouts, precision=None):
        self.parameters = evolution_parameters(tuple(parameters), hierarchy)
        self.hierarchy = hierarchy
        self.layouts = tuple(layouts)
        self.shapes = validate_hierarchy(tuple(states), self.parameters, hierarchy, self.layouts)
        self.device = _device.require_cuda()
        self.buffers = [_to_components(s, n, self.device) for s, n in zip(states, self.shapes)]
        self.patches, self.cparams = _plan(self.parameters, hierarchy, self.shapes, precision)
        self.lib = _native.load()
        nbytes = self.lib.bssn_fmr_workspace_bytes(self.patches, self.cparams, len(self.shapes))
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self.ptrs = _pointers(self.buffers)

    @property
    def points(self) -> int:
        return sum(math.prod(shape) for shape in self.shapes)

    def _advance(self, steps: int) -> None:
        _native.check(self.lib.bssn_fmr_rk4_step(self.ptrs, self.patches, self.cparams, len(self.shapes),
                                                 int(steps), self.ws.data_ptr(), self.ws.numel(),
                                                 _device.stream_handle()), "fmr_rk4_step")

    def tune(self, margin: float = 0.98) -> str:
        """Autotune the RHS launch shapes of every patch (each patch's padded
        extent is a single patch's, so the tuned shapes apply to its launches
        inside the FMR step)."""
        reports = []
        for p, (u, n) in enumerate(zip(self.buffers, self.shapes)):
            scratch = u.clone()     # tuning wraps the guards periodically; a child's are prolonged
            reports.append(_native.tune_launch_shapes(scratch.data_ptr(), n, 1, self.cparams[p], self.device,
                                                        margin=margin))
        return " | ".join(reports)

    def states(self):
        return tuple(_from_components(u, n, self.device) for u, n in zip(self.buffers, self.shapes))

    def constraint_norms(self):
        return _stats(self.buffers, self.parameters, self.hierarchy, self.shapes, self.device)
