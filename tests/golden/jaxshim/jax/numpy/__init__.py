"""NumPy-backed stand-in for the ``jax.numpy`` surface the reference uses.

Test infrastructure only: it lets the unmodified JAX_BSSN source run on the
CPU of a machine without JAX so that golden vectors can be generated from
the reference itself.  Every array is a float64-by-default NumPy array with
an ``.at[...]`` property that returns updated copies, as ``jax.Array`` does.
"""

import numpy as _np

from . import linalg  # noqa: F401  (jnp.linalg.*)


class _AtIndexer:
    def __init__(self, array, index):
        self._array = array
        self._index = index

    def set(self, value):
        out = _np.array(self._array, copy=True)
        out[self._index] = _np.asarray(value)
        return out.view(ndarray)

    def add(self, value):
        out = _np.array(self._array, copy=True)
        out[self._index] += _np.asarray(value)
        return out.view(ndarray)

    def multiply(self, value):
        out = _np.array(self._array, copy=True)
        out[self._index] *= _np.asarray(value)
        return out.view(ndarray)

    def get(self):
        return _wrap(self._array[self._index])


class _At:
    def __init__(self, array):
        self._array = array

    def __getitem__(self, index):
        return _AtIndexer(self._array, index)


class ndarray(_np.ndarray):
    """NumPy array with JAX's functional ``.at`` updates."""

    @property
    def at(self):
        return _At(self)

    def block_until_ready(self):
        return self

    def __pow__(self, other):
        return power(self, other)

    def __rpow__(self, other):
        return power(other, self)


Array = ndarray


def _wrap(value):
    if isinstance(value, _np.ndarray):
        return value.view(ndarray)
    if isinstance(value, (_np.generic, float, int, bool, complex)):
        return _np.asarray(value).view(ndarray)
    return value


def _w(fn):
    def wrapped(*args, **kwargs):
        return _wrap(fn(*args, **kwargs))
    wrapped.__name__ = getattr(fn, "__name__", "wrapped")
    return wrapped


float64 = _np.float64
float32 = _np.float32
int32 = _np.int32
int64 = _np.int64
bool_ = _np.bool_
complex128 = _np.complex128
pi = _np.pi
nan = _np.nan
inf = _np.inf
newaxis = None
dtype = _np.dtype
integer = _np.integer
floating = _np.floating


def _default_float(dtype_):
    return _np.float64 if dtype_ is None else dtype_


def asarray(a, dtype=None):
    return _np.asarray(a, dtype=dtype).view(ndarray)


def array(a, dtype=None, copy=True):
    return _np.array(a, dtype=dtype, copy=copy).view(ndarray)


def zeros(shape, dtype=None):
    return _np.zeros(shape, dtype=_default_float(dtype)).view(ndarray)


def ones(shape, dtype=None):
    return _np.ones(shape, dtype=_default_float(dtype)).view(ndarray)


def full(shape, fill_value, dtype=None):
    return _np.full(shape, fill_value, dtype=dtype).view(ndarray)


def zeros_like(a, dtype=None):
    return _np.zeros_like(_np.asarray(a), dtype=dtype).view(ndarray)


def ones_like(a, dtype=None):
    return _np.ones_like(_np.asarray(a), dtype=dtype).view(ndarray)


def full_like(a, fill_value, dtype=None):
    return _np.full_like(_np.asarray(a), fill_value, dtype=dtype).view(ndarray)


def eye(n, m=None, dtype=None):
    return _np.eye(n, m, dtype=_default_float(dtype)).view(ndarray)


def arange(*args, dtype=None):
    return _np.arange(*args, dtype=dtype).view(ndarray)


def linspace(start, stop, num=50, endpoint=True, dtype=None):
    return _np.linspace(start, stop, num, endpoint=endpoint, dtype=dtype).view(ndarray)


def einsum(subscripts, *operands, **kwargs):
    kwargs.pop("precision", None)
    ops = [_np.asarray(o) for o in operands]
    return _wrap(_np.einsum(subscripts, *ops, **kwargs))


def where(condition, x=None, y=None):
    if x is None and y is None:
        return tuple(_wrap(v) for v in _np.where(condition))
    return _wrap(_np.where(_np.asarray(condition), x, y))


def stack(arrays, axis=0):
    return _wrap(_np.stack([_np.asarray(a) for a in arrays], axis=axis))


def concatenate(arrays, axis=0):
    return _wrap(_np.concatenate([_np.asarray(a) for a in arrays], axis=axis))


def roll(a, shift, axis=None):
    return _wrap(_np.roll(_np.asarray(a), shift, axis=axis))


def take(a, indices, axis=None, mode=None):
    return _wrap(_np.take(_np.asarray(a), _np.asarray(indices), axis=axis))


def moveaxis(a, source, destination):
    return _wrap(_np.moveaxis(_np.asarray(a), source, destination))


def swapaxes(a, axis1, axis2):
    return _wrap(_np.swapaxes(_np.asarray(a), axis1, axis2))


def transpose(a, axes=None):
    return _wrap(_np.transpose(_np.asarray(a), axes))


def broadcast_to(a, shape):
    return _wrap(_np.broadcast_to(_np.asarray(a), shape))


def broadcast_arrays(*args):
    return [_wrap(v) for v in _np.broadcast_arrays(*[_np.asarray(a) for a in args])]


def meshgrid(*xi, indexing="xy"):
    return [_wrap(v) for v in _np.meshgrid(*[_np.asarray(x) for x in xi], indexing=indexing)]


def result_type(*args):
    converted = []
    for arg in args:
        if isinstance(arg, float):
            converted.append(_np.float64)
        elif isinstance(arg, bool):
            converted.append(_np.bool_)
        elif isinstance(arg, int):
            converted.append(_np.int64)
        else:
            converted.append(arg)
    return _np.result_type(*converted)


sqrt = _w(_np.sqrt)
abs = _w(_np.abs)
sin = _w(_np.sin)
cos = _w(_np.cos)
tan = _w(_np.tan)
exp = _w(_np.exp)
log = _w(_np.log)
arctan2 = _w(_np.arctan2)


def _pow_minus_third(x):
    """Correctly rounded pow(x, -1.0/3.0).

    The libm result is refined by one Newton step on y^-3 = x evaluated with
    error-free transformations (Veltkamp splitting), including the offset of
    the double exponent from -1/3, and rounded once.  glibc's pow misrounds
    about 0.07 % of these values; a correctly rounded result does not depend on
    the libm of the machine that generates the goldens.
    """
    import math
    from fractions import Fraction
    offset = float(Fraction(-1.0 / 3.0) + Fraction(1, 3))
    flat = x.reshape(-1)
    out = _np.empty_like(flat)

    def split(v):
        c = 134217729.0 * v
        hi = c - (c - v)
        return hi, v - hi

    def prod(a, b):
        p = a * b
        ah, al = split(a)
        bh, bl = split(b)
        return p, ((ah * bh - p) + ah * bl + al * bh) + al * bl

    third = Fraction(-1.0 / 3.0)
    off_f = Fraction(offset)
    for i, v in enumerate(flat.tolist()):
        if not (v > 0.0) or math.isinf(v):
            out[i] = math.pow(v, -1.0 / 3.0)
            continue
        if abs(v - 1.0) < 2.0 ** -20:
            # Exact rational midpoint tests: y* > m <=> x m^3 < x^(3 offset),
            # with x^(3 offset) = 1 + 3 offset ln x to far below any margin.
            xf = Fraction(v)
            xi = xf - 1
            rhs = 1 + 3 * off_f * (xi - xi * xi / 2 + xi ** 3 / 3)
            y = math.pow(v, -1.0 / 3.0)
            for _ in range(8):
                up = math.nextafter(y, 2.0)
                if xf * ((Fraction(y) + Fraction(up)) / 2) ** 3 < rhs:
                    y = up
                    continue
                dn = math.nextafter(y, 0.0)
                if not xf * ((Fraction(y) + Fraction(dn)) / 2) ** 3 < rhs:
                    y = dn
                    continue
                break
            out[i] = y
            continue
        y = math.pow(v, -1.0 / 3.0)
        y2, y2e = prod(y, y)
        y3, y3e = prod(y2, y)
        y3e += y2e * y
        xy, xye = prod(v, y3)
        xye += v * y3e
        s = 1.0 - xy
        bb = s - 1.0
        err = (1.0 - (s - bb)) + (-xy - bb)
        r = s + (err - xye)
        out[i] = y + y * (r / 3.0 + offset * math.log(v))
    return out.reshape(x.shape)


def power(x, y):
    """Elementwise power through the platform libm (correctly rounded pow).

    NumPy may route float64 ``power`` through SIMD approximations that differ
    from libm in the last bit on some CPUs; the goldens must not depend on the
    machine that generated them.  Squares are exact products.
    """
    import math
    x = _np.asarray(x)
    if _np.ndim(y) == 0 and float(y) == 2.0:
        return _wrap(x * x)
    if _np.ndim(y) == 0 and float(y) == -1.0 / 3.0:
        return _wrap(_pow_minus_third(x.astype(_np.float64)))
    y = _np.asarray(y, dtype=_np.float64)
    xb, yb = _np.broadcast_arrays(x.astype(_np.float64), y)
    out = _np.asarray(_np.frompyfunc(math.pow, 2, 1)(xb, yb), dtype=_np.float64)
    return _wrap(out)

floor = _w(_np.floor)
ceil = _w(_np.ceil)
round = _w(_np.round)
rint = _w(_np.rint)
maximum = _w(_np.maximum)
minimum = _w(_np.minimum)
clip = _w(_np.clip)
flip = _w(_np.flip)
expand_dims = _w(_np.expand_dims)
reshape = _w(_np.reshape)
squeeze = _w(_np.squeeze)
isfinite = _w(_np.isfinite)
isnan = _w(_np.isnan)
isclose = _w(_np.isclose)
allclose = _np.allclose
sign = _w(_np.sign)


def sum(a, axis=None, dtype=None, keepdims=False, **kwargs):
    """Reductions along one short axis accumulate left to right, the order of
    XLA's reduce loop; NumPy's pairwise scheme rounds differently."""
    a = _np.asarray(a)
    if isinstance(axis, int) and a.ndim and a.shape[axis] <= 16 and dtype is None and not kwargs:
        moved = _np.moveaxis(a, axis, 0)
        acc = moved[0].copy() if moved.shape[0] else _np.zeros(moved.shape[1:], a.dtype)
        for k in range(1, moved.shape[0]):
            acc = acc + moved[k]
        if keepdims:
            acc = _np.expand_dims(acc, axis)
        return _wrap(acc)
    return _wrap(_np.sum(a, axis=axis, dtype=dtype, keepdims=keepdims, **kwargs))

mean = _w(_np.mean)
max = _w(_np.max)
min = _w(_np.min)
amax = _w(_np.amax)
amin = _w(_np.amin)
all = _w(_np.all)
any = _w(_np.any)
prod = _w(_np.prod)
cumsum = _w(_np.cumsum)
argmax = _w(_np.argmax)
argmin = _w(_np.argmin)
dot = _w(_np.dot)
outer = _w(_np.outer)
pad = _w(_np.pad)
tile = _w(_np.tile)
repeat = _w(_np.repeat)
diag = _w(_np.diag)
trace = _w(_np.trace)
copy = _w(_np.copy)
logical_and = _w(_np.logical_and)
logical_or = _w(_np.logical_or)
logical_not = _w(_np.logical_not)
sort = _w(_np.sort)
unique = _w(_np.unique)
nonzero = _np.nonzero
shape = _np.shape
ndim = _np.ndim
size = _np.size
float_ = _np.float64
vdot = _w(_np.vdot)
matmul = _w(_np.matmul)
cross = _w(_np.cross)
real = _w(_np.real)
imag = _w(_np.imag)
conj = _w(_np.conj)
log2 = _w(_np.log2)
log10 = _w(_np.log10)
hypot = _w(_np.hypot)
arctan = _w(_np.arctan)
arccos = _w(_np.arccos)
arcsin = _w(_np.arcsin)
sinh = _w(_np.sinh)
cosh = _w(_np.cosh)
tanh = _w(_np.tanh)
square = _w(_np.square)
exp2 = _w(_np.exp2)
median = _w(_np.median)
std = _w(_np.std)
var = _w(_np.var)
diff = _w(_np.diff)
gradient = _np.gradient
trapezoid = _w(_np.trapezoid)
interp = _w(_np.interp)
searchsorted = _w(_np.searchsorted)
histogram = _np.histogram
array_equal = _np.array_equal
iscomplexobj = _np.iscomplexobj
finfo = _np.finfo
iinfo = _np.iinfo
resize = _w(_np.resize)
