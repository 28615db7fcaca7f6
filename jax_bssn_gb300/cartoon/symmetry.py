"""Parity tables and field mapping of the Cartoon modes (mirrors JAX_BSSN/cartoon/symmetry.py:15-71).

A Cartoon mode stores one authoritative half of a reflection-symmetric grid;
a field's reflection sign depends only on its tensor rank and on the mode's
vector parity table (axisymmetric (-1,-1,+1), spherical (-1,+1,+1)).  These
helpers act on CUDA tensors; host arrays are moved to the device first and the
result is returned as NumPy.
"""

from __future__ import annotations

import numpy as np
import torch

from .. import _device
from ..bssn.variables import BSSNVariables

SCALAR_PARITY = 1.0


def _dev(a) -> tuple[torch.Tensor, bool]:
    if isinstance(a, torch.Tensor) and a.is_cuda:
        return a.to(torch.float64), False
    device = _device.require_cuda()
    return torch.as_tensor(np.asarray(a, dtype=np.float64), device=device), True


def _back(t: torch.Tensor, host: bool):
    return t.cpu().numpy() if host else t


def vector_parity(signs, dtype=torch.float64, device=None) -> torch.Tensor:
    """Per-component reflection signs of a Cartesian vector (symmetry.py:18-21)."""
    return torch.as_tensor(signs, dtype=dtype, device=device)


def tensor_parity(signs, dtype=torch.float64, device=None) -> torch.Tensor:
    """Outer product of the vector signs (symmetry.py:24-28)."""
    p = vector_parity(signs, dtype, device)
    return p[:, None] * p[None, :]


def field_parity(field, signs, spatial_ndim: int = 3):
    """Reflection parity implied by the tensor rank (symmetry.py:31-41)."""
    rank = field.ndim - spatial_ndim
    device = field.device if isinstance(field, torch.Tensor) else None
    if rank == 0:
        return torch.tensor(SCALAR_PARITY, dtype=torch.float64, device=device)
    if rank == 1:
        return vector_parity(signs, device=device)
    if rank == 2:
        return tensor_parity(signs, device=device)
    raise ValueError(f"unsupported tensor rank {rank} for reflection parity")


def map_bssn_fields(vars: BSSNVariables, transform, signs, spatial_ndim: int = 3) -> BSSNVariables:
    """Apply ``transform(field, parity)`` to every field in order (symmetry.py:44-52)."""
    return BSSNVariables(*(transform(f, field_parity(f, signs, spatial_ndim)) for f in vars))


def reflect_tensor(positive: torch.Tensor, parity, axis: int = -1, count: int | None = None) -> torch.Tensor:
    axis = axis % positive.ndim
    parity = torch.as_tensor(parity, dtype=positive.dtype, device=positive.device)
    parity = parity.reshape(tuple(parity.shape) + (1,) * (positive.ndim - parity.ndim))
    n = positive.shape[axis] if count is None else min(count, positive.shape[axis])
    mirrored = torch.flip(positive.narrow(axis, 0, n), dims=(axis,)) * parity
    return torch.cat((mirrored, positive), dim=axis)


def reflect(positive, parity, axis: int = -1, count: int | None = None):
    """Mirror the first ``count`` samples (all when None) across the origin with
    the given parity and prepend them (symmetry.py:55-71)."""
    t, host = _dev(positive)
    return _back(reflect_tensor(t, parity, axis, count), host)


__all__ = ["SCALAR_PARITY", "field_parity", "map_bssn_fields", "reflect", "tensor_parity", "vector_parity"]
