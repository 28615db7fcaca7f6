"""``jax.lax`` stand-in: Python control flow and single-device collectives."""

import numpy as _np

from .. import numpy as _jnp

_MISSING = object()


def cond(pred, true_fun, false_fun, *operands, operand=_MISSING):
    if operand is not _MISSING:
        operands = (operand,)
    branch = true_fun if bool(_np.asarray(pred)) else false_fun
    return branch(*operands)


def select(pred, on_true, on_false):
    return _jnp.where(pred, on_true, on_false)


def fori_loop(lower, upper, body_fun, init_val):
    value = init_val
    for index in range(int(lower), int(upper)):
        value = body_fun(index, value)
    return value


def while_loop(cond_fun, body_fun, init_val):
    value = init_val
    while bool(cond_fun(value)):
        value = body_fun(value)
    return value


def scan(f, init, xs, length=None):
    carry = init
    outputs = []
    count = length if xs is None else len(xs)
    for index in range(count):
        carry, out = f(carry, None if xs is None else xs[index])
        outputs.append(out)
    return carry, outputs


def map(f, xs):
    return _jnp.stack([f(x) for x in xs])


def _starts(operand, start_indices):
    return tuple(int(_np.asarray(s)) for s in start_indices)


def dynamic_slice(operand, start_indices, slice_sizes):
    operand = _np.asarray(operand)
    starts = _starts(operand, start_indices)
    # JAX clamps each start so the slice stays in bounds.
    starts = tuple(min(max(s, 0), n - size) for s, n, size in zip(starts, operand.shape, slice_sizes))
    index = tuple(slice(s, s + size) for s, size in zip(starts, slice_sizes))
    return _jnp.asarray(operand[index])


def dynamic_update_slice(operand, update, start_indices):
    out = _np.array(operand, copy=True)
    update = _np.asarray(update)
    starts = _starts(operand, start_indices)
    starts = tuple(min(max(s, 0), n - size) for s, n, size in zip(starts, out.shape, update.shape))
    index = tuple(slice(s, s + size) for s, size in zip(starts, update.shape))
    out[index] = update
    return _jnp.asarray(out)


def dynamic_slice_in_dim(operand, start_index, slice_size, axis=0):
    operand = _np.asarray(operand)
    axis = axis % operand.ndim
    starts = [0] * operand.ndim
    sizes = list(operand.shape)
    starts[axis] = start_index
    sizes[axis] = slice_size
    return dynamic_slice(operand, starts, sizes)


def dynamic_update_slice_in_dim(operand, update, start_index, axis):
    operand = _np.asarray(operand)
    axis = axis % operand.ndim
    starts = [0] * operand.ndim
    starts[axis] = start_index
    return dynamic_update_slice(operand, update, starts)


def axis_index(axis_name):
    return 0


def ppermute(x, axis_name, perm):
    for source, destination in perm:
        if source != destination:
            raise ValueError("the NumPy jax shim has a single device")
    return x


def psum(x, axis_name):
    return x


def pmax(x, axis_name):
    return x


def pmin(x, axis_name):
    return x


def stop_gradient(x):
    return x
