"""Minimal NumPy-backed ``jax`` stand-in for running the reference on a CPU.

Test infrastructure only (golden-vector generation in this directory); no
product code imports it.  ``jit`` is the identity, ``lax.cond`` branches in
Python, and the single-device ``shard_map``/``ppermute``/``psum`` collectives
act on the local (whole) array.  Only the API surface the reference's hot
path touches is provided.
"""

import functools as _functools

import numpy as _np

from . import numpy  # noqa: F401
from . import lax  # noqa: F401
from . import sharding  # noqa: F401
from . import tree  # noqa: F401
from . import scipy  # noqa: F401
from .numpy import ndarray as Array

__version__ = "0.0-numpy-shim"


class _Config:
    def update(self, name, value):
        setattr(self, name, value)

    jax_enable_x64 = True
    x64_enabled = True


config = _Config()


def jit(fun=None, *, static_argnames=None, static_argnums=None, donate_argnums=None,
        donate_argnames=None, **unused):
    if fun is None:
        return lambda f: f
    return fun


def vmap(fun, in_axes=0, out_axes=0):
    """Vectorise ``fun`` over one mapped axis of each argument."""

    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        if fun is numpy.linalg.det and len(args) == 1:
            # Batched determinant over the mapped axis.
            stacked = _np.moveaxis(_np.asarray(args[0]), axes[0], 0)
            return numpy.asarray(_np.moveaxis(_np.asarray(fun(stacked)), 0, out_axes))
        size = None
        moved = []
        for arg, axis in zip(args, axes):
            if axis is None:
                moved.append(None)
            else:
                value = _np.moveaxis(_np.asarray(arg), axis, 0)
                size = value.shape[0]
                moved.append(value)
        results = []
        for index in range(size):
            call = [arg if m is None else m[index] for arg, m in zip(args, moved)]
            results.append(fun(*call))
        if isinstance(results[0], tuple):       # several outputs: stack each
            return tuple(numpy.asarray(_np.moveaxis(_np.stack([_np.asarray(r[k]) for r in results]), 0, out_axes))
                         for k in range(len(results[0])))
        return numpy.asarray(_np.moveaxis(_np.stack([_np.asarray(r) for r in results]), 0, out_axes))

    return mapped


class _Device:
    platform = "cpu"
    id = 0

    def __repr__(self):
        return "CpuDevice(id=0)"


_DEVICE = _Device()


def devices(backend=None):
    return [_DEVICE]


def device_count():
    return 1


def local_device_count():
    return 1


def process_count():
    return 1


def process_index():
    return 0


def device_get(x):
    return x


def device_put(x, device=None):
    return x


def block_until_ready(x):
    return x


class _Mesh:
    def __init__(self, shape, axis_names, devices_):
        self.devices = _np.empty(shape, dtype=object)
        flat = list(devices_)
        for index, position in enumerate(_np.ndindex(*shape)):
            self.devices[position] = flat[index]
        self.axis_names = tuple(axis_names)
        self.shape = dict(zip(axis_names, shape))

    def __eq__(self, other):
        return (isinstance(other, _Mesh) and self.axis_names == other.axis_names
                and self.devices.shape == other.devices.shape)

    def __hash__(self):
        return hash((self.axis_names, self.devices.shape))


def make_mesh(axis_shapes, axis_names, *, devices=None, axis_types=None):
    axis_shapes = tuple(int(n) for n in axis_shapes)
    if int(_np.prod(axis_shapes)) != 1:
        raise ValueError("the NumPy jax shim provides a single device")
    return _Mesh(axis_shapes, axis_names, devices or [_DEVICE])


def shard_map(fun, *, mesh=None, in_specs=None, out_specs=None, check_vma=True,
              check_rep=True, axis_names=None):
    """On one device every shard is the whole array: call ``fun`` directly."""

    @_functools.wraps(fun)
    def mapped(*args):
        return fun(*args)

    return mapped


def make_array_from_callback(shape, sharding_, data_callback, dtype=None):
    index = tuple(slice(0, n) for n in shape)
    value = _np.asarray(data_callback(index))
    if dtype is not None:
        value = value.astype(dtype)
    return numpy.asarray(value.reshape(shape))


def named_call(fun, name=None):
    return fun


# Forward-mode derivatives by central differences.  JAX differentiates
# exactly; these stand-ins are used where the result steers an iteration (the
# horizon finder's Newton Jacobian) or enters a residual to about 1e-11 (the
# metric derivative of the Hermite interpolant, piecewise cubic, by a
# Richardson-extrapolated difference), so a converged answer still comes from
# the reference's own residual.

def linearize(fun, *primals):
    """(fun(*primals), jvp) with jvp(tangent) a central difference of step
    1e-6 relative to the primal's scale (one primal)."""
    if len(primals) != 1:
        raise NotImplementedError("the NumPy shim linearizes functions of one argument")
    x = _np.asarray(primals[0], dtype=_np.float64)
    scale = max(float(_np.max(_np.abs(x))), 1.0)
    value = fun(numpy.asarray(x))

    def jvp(tangent):
        t = _np.asarray(tangent, dtype=_np.float64)
        h = 1.0e-6 * scale / max(float(_np.max(_np.abs(t))), 1e-300)
        plus = _np.asarray(fun(numpy.asarray(x + h * t)))
        minus = _np.asarray(fun(numpy.asarray(x - h * t)))
        return numpy.asarray((plus - minus) / (2.0 * h))

    return value, jvp


def jacfwd(fun, argnums=0):
    """Jacobian by Richardson-extrapolated central differences (steps h and
    h/2, h = 1e-5 max(|x|, 1)), one column per input element; shape fun's
    output + input.  Exact to roundoff for polynomials of degree four."""

    def central(args, x, index, h):
        up, down = x.copy(), x.copy()
        up[index] += h
        down[index] -= h
        call = list(args)
        call[argnums] = numpy.asarray(up)
        plus = _np.asarray(fun(*call))
        call[argnums] = numpy.asarray(down)
        minus = _np.asarray(fun(*call))
        return (plus - minus) / (up[index] - down[index])

    def jac(*args):
        x = _np.asarray(args[argnums], dtype=_np.float64)
        columns = []
        for index in _np.ndindex(*x.shape):
            h = 1.0e-5 * max(abs(float(x[index])), 1.0)
            coarse, fine = central(args, x, index, h), central(args, x, index, 0.5 * h)
            columns.append((4.0 * fine - coarse) / 3.0)
        out_shape = columns[0].shape
        return numpy.asarray(_np.stack(columns, axis=-1).reshape(out_shape + x.shape))

    return jac


class nn:
    @staticmethod
    def one_hot(x, num_classes, dtype=_np.float64):
        x = _np.asarray(x)
        return numpy.asarray((x[..., None] == _np.arange(num_classes)).astype(dtype))
