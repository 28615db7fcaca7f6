"""Output staging for openPMD writers (mirrors the array side of
JAX_BSSN/diagnostics/openpmd.py).

The reference's writers strip ghost cells (``_strip_ghost_cells``, :51-71) or
copy owned tile samples (``tiled_output_fields``, :254-285) and hand host
arrays to openPMD-api.  Here every owned box of a level is gathered on the
device into one contiguous staging buffer by one kernel
(``bssn_gather_boxes``) and crosses to the host in a single pinned copy; the
returned NumPy arrays are views of that pinned buffer.  The openPMD-api
writers themselves (``OpenPMDWriter``, ``FMRPatchSeriesWriter``) are not part
of this package: openPMD-api is not installed here, and the staged arrays are
what they consume.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from .. import _device, _native


def _integer_3tuple(value, name):
    values = tuple(int(v) for v in (value if isinstance(value, (tuple, list)) else (value,) * 3))
    if len(values) != 3:
        raise ValueError(f"{name} must be a scalar or a 3-tuple")
    return values


def _is_vector(field):
    return isinstance(field, (tuple, list)) and len(field) == 3


def _components(field_map):
    """[(name, component index or None, array)] in map order."""
    out = []
    for name, field in field_map.items():
        if _is_vector(field):
            out.extend((name, c, component) for c, component in enumerate(field))
        else:
            out.append((name, None, field))
    return out


def _gather(items, device):
    """items: [(source tensor, lo, extent)] -> one flat device buffer and offsets."""
    lib = _native.load()
    sizes = [math.prod(ext) for _, _, ext in items]
    offsets = np.concatenate(([0], np.cumsum(sizes))).astype(np.int64)
    flat = torch.empty(int(offsets[-1]), dtype=torch.float64, device=device)
    stream = _device.stream_handle()
    for start in range(0, len(items), _native.MAX_GATHER_BOXES):
        chunk = items[start:start + _native.MAX_GATHER_BOXES]
        boxes = (_native.BssnBox * len(chunk))()
        for b, (src, lo, ext) in enumerate(chunk):
            boxes[b].src = src.data_ptr()
            for a in range(3):
                boxes[b].shape[a] = int(src.shape[a])
                boxes[b].lo[a] = int(lo[a])
                boxes[b].extent[a] = int(ext[a])
        dst = flat[int(offsets[start]):]
        _native.check(lib.bssn_gather_boxes(len(chunk), ctypes.addressof(boxes), dst.data_ptr(), stream),
                      "gather_boxes")
    return flat, offsets


def _device_component(array, name, device):
    t = _device.as_device(array, tuple(array.shape), device, name)
    if t.dim() != 3:
        raise ValueError(f"field {name!r} must have three-dimensional components")
    return t


def _staged(field_map, boxes_of, to_host):
    device = _device.require_cuda()
    comps = _components(field_map)
    items, shapes = [], []
    for name, c, array in comps:
        t = _device_component(array, name, device)
        lo, ext = boxes_of(name, t)
        if any(n < 1 for n in ext):
            raise ValueError(f"ghost stripping leaves field {name!r} with an empty axis")
        items.append((t, lo, ext))
        shapes.append(tuple(ext))
    for name in field_map:
        if _is_vector(field_map[name]):
            sh = {s for (n, _, _), s in zip(comps, shapes) if n == name}
            if len(sh) != 1:
                raise ValueError(f"vector field {name!r} has components with different active shapes")
    flat, offsets = _gather(items, device)
    if to_host:
        pinned = torch.empty(flat.numel(), dtype=torch.float64, pin_memory=True)
        pinned.copy_(flat, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        flat = pinned.numpy()
    pieces = [flat[int(offsets[i]):int(offsets[i + 1])].reshape(s) for i, s in enumerate(shapes)]
    out, i = {}, 0
    for name, field in field_map.items():
        if _is_vector(field):
            out[name] = tuple(pieces[i:i + 3])
            i += 3
        else:
            out[name] = pieces[i]
            i += 1
    return out


def strip_ghost_cells(field_map, ghost_cells):
    """Interior boxes of scalar and 3-vector fields, compact on the device
    (openpmd.py:51-71)."""
    g = _integer_3tuple(ghost_cells, "ghost_cells")
    if any(w < 0 for w in g):
        raise ValueError("ghost_cells must be a non-negative scalar or 3-tuple")
    return _staged(field_map, lambda name, t: (g, tuple(n - 2 * w for n, w in zip(t.shape, g))), to_host=False)


def stage_output_fields(field_map, ghost_cells=0):
    """Ghost-stripped fields as host NumPy arrays, all gathered by one kernel
    and copied by one pinned transfer (the arrays a writer hands to
    openPMD-api; openpmd.py:39-71)."""
    g = _integer_3tuple(ghost_cells, "ghost_cells")
    if any(w < 0 for w in g):
        raise ValueError("ghost_cells must be a non-negative scalar or 3-tuple")
    return _staged(field_map, lambda name, t: (g, tuple(n - 2 * w for n, w in zip(t.shape, g))), to_host=True)


def tiled_output_fields(field_map, layout):
    """Owned tile samples of a patch as host arrays (openpmd.py:254-285).

    Fields carry the tile axes first, ``counts + allocated_shape``; the GB300
    FMR path keeps each patch as one tile on one GPU."""
    counts = tuple(int(c) for c in getattr(layout, "counts", (1, 1, 1)))
    if counts != (1, 1, 1):
        raise ValueError("the GB300 FMR path runs every patch as a single tile on one GPU")
    g = int(layout.guard_cells)
    allocated = tuple(int(n) for n in layout.allocated_shape)
    active = tuple(int(n) for n in layout.active_shape)
    flat_map = {}
    for name, field in field_map.items():
        def strip(v):
            if tuple(v.shape) != counts + allocated:
                raise ValueError("output field does not match its tile layout")
            return v.reshape(allocated)
        flat_map[name] = tuple(strip(c) for c in field) if _is_vector(field) else strip(field)
    return _staged(flat_map, lambda name, t: ((g, g, g), active), to_host=True)
