"""Six-node Lagrange interpolation of the Cartoon reconstructions
(mirrors JAX_BSSN/cartoon/interpolation.py:9-87).

The reconstruction kernels (``bssn_cartoon_reconstruct``) carry this
interpolation inline; these device-tensor versions serve callers that
interpolate their own profiles.  Weights are the product formula with the
factors taken in node order; the six products are summed left to right.
"""

from __future__ import annotations

import torch

from .symmetry import _back, _dev


def lagrange6_weights(q, nodes):
    """Degree-five Lagrange weights of ``q`` for six nodes (interpolation.py:9-23)."""
    qt, host = _dev(q)
    nt = torch.as_tensor(nodes, device=qt.device)
    nf = nt.to(torch.float64)
    w = torch.ones(nt.shape, dtype=torch.float64, device=qt.device)
    for k in range(6):
        for m in range(6):
            if k != m:
                w[..., k] = w[..., k] * ((qt - nf[..., m]) / (nf[..., k] - nf[..., m]))
    return _back(w, host)


def lagrange6_stencil(q, source_size: int):
    """The six clipped source indices of every target (interpolation.py:49-58)."""
    if source_size < 6:
        raise ValueError("six-point Lagrange interpolation needs six samples")
    qt, host = _dev(q)
    start = torch.clamp(torch.floor(qt).to(torch.int32) - 2, 0, source_size - 6)
    nodes = start[..., None] + torch.arange(6, dtype=torch.int32, device=qt.device)
    return nodes.cpu().numpy() if host else nodes


def lagrange6_nonperiodic(array, q, axis: int = -1):
    """Interpolate along ``axis`` at fractional indices ``q``; NaN outside
    [0, size-1] instead of extrapolating (interpolation.py:61-87)."""
    a, host = _dev(array)
    qt, _ = _dev(q)
    axis = axis % a.ndim
    size = a.shape[axis]
    nodes = lagrange6_stencil(qt, size)
    w = lagrange6_weights(qt, nodes)
    moved = torch.movedim(a, axis, -1)
    lead = moved.shape[:-1]
    gathered = moved[..., nodes.long()]                  # lead + targets + (6,)
    prod = gathered * w.reshape((1,) * len(lead) + tuple(w.shape))
    value = prod[..., 0]
    for k in range(1, 6):
        value = value + prod[..., k]
    tdim = nodes.ndim - 1
    perm = tuple(range(axis)) + tuple(range(a.ndim - 1, a.ndim - 1 + tdim)) + tuple(range(axis, a.ndim - 1))
    value = value.permute(perm)
    valid = (qt >= 0) & (qt <= size - 1)
    valid = valid.reshape((1,) * axis + tuple(valid.shape) + (1,) * (a.ndim - axis - 1))
    out = torch.where(valid, value, torch.full_like(value, float("nan")))
    return _back(out, host)


__all__ = ["lagrange6_nonperiodic", "lagrange6_stencil", "lagrange6_weights"]
