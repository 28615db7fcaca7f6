"""Device plumbing for the drop-in API: tensors, parameters, workspaces, streams.

PyTorch supplies CUDA memory and the current stream; the arithmetic happens
in ``libbssn_gb300.so``.  Inputs may be CUDA tensors (returned as CUDA
tensors) or host arrays (copied in and the results copied back as NumPy).
"""

from __future__ import annotations

import contextlib
import contextvars
import ctypes
import math
import threading

import numpy as np
import torch

from . import _native
from .bssn.variables import BSSNVariables

FACE_NAMES = ("xl_bc", "xr_bc", "yl_bc", "yr_bc", "zl_bc", "zr_bc")
LEAF_SHAPES = ((3, 3), (), (3, 3), (), (3,), (), (3,))


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("jax_bssn_gb300 runs on a CUDA GPU; none is visible")
    return torch.device("cuda", torch.cuda.current_device())


# Arithmetic of the RHS kernels for calls made in this context: "fp64" (plain
# float64, the default), "fp32" (float RHS arithmetic on a float64 state) or
# "fp32_paired" (the same with the second-derivative fields as float pairs).
PRECISIONS = {"fp64": _native.PRECISION_F64, "fp32": _native.PRECISION_F32,
              "fp32_paired": _native.PRECISION_F32_PAIRED}
_ARITHMETIC = contextvars.ContextVar("jax_bssn_gb300_arithmetic", default="fp64")


def _checked(name: str) -> str:
    if name not in PRECISIONS:
        raise ValueError(f"arithmetic must be one of {sorted(PRECISIONS)}, got {name!r}")
    return name


def current_arithmetic() -> str:
    return _ARITHMETIC.get()


def set_arithmetic(name: str) -> None:
    """Select the RHS arithmetic for subsequent calls in this context."""
    _ARITHMETIC.set(_checked(name))


@contextlib.contextmanager
def arithmetic(name: str):
    """``with arithmetic("fp32"): ...`` -- the RHS arithmetic inside the block."""
    token = _ARITHMETIC.set(_checked(name))
    try:
        yield
    finally:
        _ARITHMETIC.reset(token)


def to_params(params, precision: str | None = None) -> _native.BssnParams:
    """BSSNParameters -> the C struct (JAX_BSSN/bssn/variables.py:19-46).

    ``precision`` ("fp64" / "fp32" / "fp32_paired") overrides the context's arithmetic."""
    p = _native.BssnParams()
    p.precision = PRECISIONS[_checked(precision) if precision is not None else _ARITHMETIC.get()]
    p.eta, p.kappa, p.nu, p.g = float(params.eta), float(params.kappa), float(params.nu), float(params.g)
    p.dx, p.dt = float(params.dx), float(params.dt)
    p.zero_shift, p.gauge = int(params.zero_shift), int(params.gauge)
    for f, name in enumerate(FACE_NAMES):
        p.bc[f] = int(getattr(params, name))
    p.xmin[0], p.xmin[1], p.xmin[2] = float(params.x_min), float(params.y_min), float(params.z_min)
    p.mad_q = float(params.mad_q)
    p.guard_cells = int(params.guard_cells)
    owned = params.owned_shape
    for d in range(3):
        p.owned_shape[d] = -1 if owned is None else int(owned[d])
    for f in range(6):
        p.owned_faces[f] = 1 if bool(params.owned_faces[f]) else 0
    for d in range(3):
        p.reduced_axes[d] = -1 if params.reduced_axes is None else int(bool(params.reduced_axes[d]))
    return p


def spatial_shape(state) -> tuple[int, int, int]:
    shape = tuple(int(n) for n in state.conformal_factor.shape)
    if len(shape) != 3:
        raise ValueError("BSSN fields must end with three spatial axes")
    return shape


def as_device(leaf, shape, device, name: str = "field") -> torch.Tensor:
    """A contiguous float64 CUDA tensor of the given shape (host arrays are copied in)."""
    if isinstance(leaf, torch.Tensor):
        t = leaf.to(device=device, dtype=torch.float64)
    else:
        t = torch.as_tensor(np.asarray(leaf, dtype=np.float64), device=device)
    if tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(t.shape)}; expected {tuple(shape)}")
    return t.contiguous()



def device_state(state) -> tuple[BSSNVariables, bool]:
    """All seven leaves as contiguous float64 CUDA tensors, and whether the
    caller passed host arrays (so results go back to NumPy)."""
    device = require_cuda()
    shape = spatial_shape(state)
    host = not isinstance(state.conformal_factor, torch.Tensor) or not state.conformal_factor.is_cuda
    leaves = tuple(as_device(leaf, lead + shape, device) for leaf, lead in zip(state, LEAF_SHAPES))
    return BSSNVariables(*leaves), host


def empty_state(shape, device) -> BSSNVariables:
    return BSSNVariables(*(torch.empty(lead + tuple(shape), dtype=torch.float64, device=device)
                           for lead in LEAF_SHAPES))


def to_host(state) -> BSSNVariables:
    return BSSNVariables(*(leaf.detach().cpu().numpy() for leaf in state))


def fields_struct(state) -> _native.BssnFields:
    f = _native.BssnFields()
    for name, leaf in zip(_native.BssnFields._fields_, state):
        setattr(f, name[0], leaf.data_ptr())
    return f


def stream_handle() -> int:
    return torch.cuda.current_stream().cuda_stream


class _Workspaces(threading.local):
    def __init__(self):
        self.buffers: dict[tuple, torch.Tensor] = {}


_WS = _Workspaces()


def workspace(nbytes: int, device, tag: str = "main") -> torch.Tensor:
    """A cached uint8 device buffer of at least ``nbytes`` (grown on demand)."""
    key = (tag, device.index)
    buf = _WS.buffers.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)
        _WS.buffers[key] = buf
    return buf


def shape3(shape) -> ctypes.Array:
    return _native.Shape3(*[int(n) for n in shape])


def prod(shape) -> int:
    return int(math.prod(shape))
