"""``jax.numpy.linalg`` stand-in backed by NumPy/LAPACK (test infrastructure)."""

import numpy as _np


def _wrap(value):
    from . import ndarray
    return _np.asarray(value).view(ndarray)


def det(a):
    """JAX evaluates 3x3 determinants in closed form (Sarrus), not by LU."""
    a = _np.asarray(a)
    if a.shape[-2:] == (3, 3):
        return _wrap(a[..., 0, 0] * a[..., 1, 1] * a[..., 2, 2]
                     + a[..., 0, 1] * a[..., 1, 2] * a[..., 2, 0]
                     + a[..., 0, 2] * a[..., 1, 0] * a[..., 2, 1]
                     - a[..., 0, 2] * a[..., 1, 1] * a[..., 2, 0]
                     - a[..., 0, 0] * a[..., 1, 2] * a[..., 2, 1]
                     - a[..., 0, 1] * a[..., 1, 0] * a[..., 2, 2])
    return _wrap(_np.linalg.det(a))


def inv(a):
    return _wrap(_np.linalg.inv(_np.asarray(a)))


def solve(a, b):
    return _wrap(_np.linalg.solve(_np.asarray(a), _np.asarray(b)))


def cholesky(a):
    return _wrap(_np.linalg.cholesky(_np.asarray(a)))


def norm(x, ord=None, axis=None, keepdims=False):
    return _wrap(_np.linalg.norm(_np.asarray(x), ord=ord, axis=axis, keepdims=keepdims))
