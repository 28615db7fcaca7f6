"""Patch transfers on GB300 (mirrors JAX_BSSN/fmr/transfer.py:237-252)."""

from __future__ import annotations

from .. import _device, _native
from .tiled import _finish, _from_components, _is_host, _layout_shape, _to_components


def fill_tiled_fine_ghosts(parent, child, spec, *, parent_layout, child_layout,
                           parent_boundary_codes=(0,) * 6, parent_is_root=True):
    """Replace only the child's exterior shell by six-node Lagrange
    interpolation of the prepared parent (transfer.py:237-244)."""
    pshape, cshape = _layout_shape(parent_layout), _layout_shape(child_layout)
    if parent_is_root:
        for axis in range(3):
            lo, hi, n = spec.coarse_lo[axis], spec.coarse_hi[axis], pshape[axis]
            if (lo - 4 < 0 and parent_boundary_codes[2 * axis]) or (hi + 5 >= n and parent_boundary_codes[2 * axis + 1]):
                raise ValueError("FMR interpolation stencil crosses a physical root boundary")
    host = _is_host((child,))
    device = _device.require_cuda()
    up, uc = _to_components(parent, pshape, device), _to_components(child, cshape, device)
    lib = _native.load()
    _native.check(lib.bssn_fmr_prolong(up.data_ptr(), _device.shape3(pshape), uc.data_ptr(), _device.shape3(cshape),
                                       _device.shape3(spec.coarse_lo), _device.stream_handle()),
                  "fill_tiled_fine_ghosts")
    return _finish([_from_components(uc, cshape, device)], host)[0]


def restrict_tiled_to_coarse(parent, child, spec, *, parent_layout, child_layout):
    """Inject owned coincident child vertices into the parent (transfer.py:247-252)."""
    pshape, cshape = _layout_shape(parent_layout), _layout_shape(child_layout)
    host = _is_host((parent,))
    device = _device.require_cuda()
    up, uc = _to_components(parent, pshape, device), _to_components(child, cshape, device)
    lib = _native.load()
    _native.check(lib.bssn_fmr_inject(up.data_ptr(), _device.shape3(pshape), uc.data_ptr(), _device.shape3(cshape),
                                      _device.shape3(spec.coarse_lo), _device.stream_handle()),
                  "restrict_tiled_to_coarse")
    return _finish([_from_components(up, pshape, device)], host)[0]
