"""NumPy-backed ``jax.numpy`` subset with JAX's dtype and immutability semantics.

Only what vivsim's library modules call is provided.  Every result is a
:class:`JArray` (an ``ndarray`` subclass) so that ``x.at[idx].set/add`` and
rebinding augmented assignment behave as in JAX.
"""

import builtins
import numbers

import numpy as _np

from .. import _state

float32 = _np.float32
float64 = _np.float64
int32 = _np.int32
int64 = _np.int64
bool_ = _np.bool_
pi = _np.pi
inf = _np.inf
nan = _np.nan
newaxis = None
ndarray = _np.ndarray


# ----------------------------------------------------------------- dtypes

def _canon_dtype(dt):
    dt = _np.dtype(dt)
    if _state.X64:
        return dt
    if dt == _np.float64:
        return _np.dtype(_np.float32)
    if dt == _np.int64:
        return _np.dtype(_np.int32)
    if dt == _np.uint64:
        return _np.dtype(_np.uint32)
    if dt == _np.complex128:
        return _np.dtype(_np.complex64)
    return dt


def _default_float():
    return _np.dtype(_np.float64 if _state.X64 else _np.float32)


def _is_weak(x):
    return isinstance(x, (bool, int, float, complex)) and not isinstance(x, _np.generic)


def _canon(x):
    """Array-like -> canonical plain ndarray; Python scalars stay weakly typed."""
    if _is_weak(x):
        return x
    a = _np.asarray(x)
    dt = _canon_dtype(a.dtype)
    if a.dtype != dt:
        a = a.astype(dt)
    return a


def _wrap(x):
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, list):
        return [_wrap(v) for v in x]
    if isinstance(x, (_np.ndarray, _np.generic)):
        a = _np.asarray(x)
        dt = _canon_dtype(a.dtype)
        if a.dtype != dt:
            a = a.astype(dt)
        return a.view(JArray)
    return x


def _jax_result_dtype(arrays):
    """JAX promotion for strongly typed inputs: ints sit below every float."""
    floats = [a.dtype for a in arrays if _np.issubdtype(a.dtype, _np.floating)]
    if floats:
        return builtins.max(floats, key=lambda d: d.itemsize)
    ints = [a.dtype for a in arrays if _np.issubdtype(a.dtype, _np.integer)]
    if ints:
        return _np.result_type(*ints)
    return None


def _promote(*xs):
    """Canonicalise inputs and cast strongly typed ones to JAX's common dtype."""
    cx = [_canon(x) for x in xs]
    strong = [a for a in cx if isinstance(a, _np.ndarray)]
    rdt = _jax_result_dtype([a for a in strong if a.dtype != _np.bool_])
    if rdt is None:
        return cx
    out = []
    for a in cx:
        if isinstance(a, _np.ndarray) and a.dtype != _np.bool_ and a.dtype != rdt:
            a = a.astype(rdt)
        out.append(a)
    return out


def _unwrap_tree(x):
    if isinstance(x, (list, tuple)):
        return type(x)(_unwrap_tree(v) for v in x)
    if isinstance(x, JArray):
        return x.view(_np.ndarray)
    return x


# ------------------------------------------------------------------ array

class _AtIndex:
    def __init__(self, arr, idx):
        self._arr = arr
        self._idx = _unwrap_tree(idx) if isinstance(idx, tuple) else _unwrap_tree(idx)

    def set(self, values):
        out = self._arr.view(_np.ndarray).copy()
        out[self._idx] = _canon(values)
        return _wrap(out)

    def add(self, values):
        out = self._arr.view(_np.ndarray).copy()
        _np.add.at(out, self._idx, _canon(values))
        return _wrap(out)

    def get(self):
        return self._arr[self._idx]


class _At:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtIndex(self._arr, idx)


class JArray(_np.ndarray):
    """Immutable-style ndarray: ``.at`` updates copy, ``x -= y`` rebinds."""

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        if "out" in kwargs:
            raise TypeError("in-place ufuncs are not JAX semantics")
        ins = _promote(*inputs) if len(inputs) > 1 else [_canon(i) for i in inputs]
        ins = [i.view(_np.ndarray) if isinstance(i, JArray) else i for i in ins]
        return _wrap(getattr(ufunc, method)(*ins, **kwargs))

    @property
    def at(self):
        return _At(self)

    def astype(self, dtype, *args, **kwargs):
        return _wrap(self.view(_np.ndarray).astype(_canon_dtype(dtype)))

    def __iadd__(self, other):
        return self.__add__(other)

    def __isub__(self, other):
        return self.__sub__(other)

    def __imul__(self, other):
        return self.__mul__(other)

    def __itruediv__(self, other):
        return self.__truediv__(other)


# ------------------------------------------------------------ constructors

def asarray(x, dtype=None):
    if dtype is not None:
        return _wrap(_np.asarray(_unwrap_tree(x), dtype=_canon_dtype(dtype)))
    if _is_weak(x):
        if isinstance(x, bool):
            return _wrap(_np.asarray(x))
        if isinstance(x, numbers.Integral):
            return _wrap(_np.asarray(x, dtype=_np.int64))
        return _wrap(_np.asarray(x, dtype=_default_float()))
    return _wrap(_np.asarray(_unwrap_tree(x)))


def array(x, dtype=None):
    if dtype is not None:
        return _wrap(_np.array(_unwrap_tree(x), dtype=_canon_dtype(dtype)))
    a = _np.array(_unwrap_tree(x))
    if a.dtype == _np.float64 and not _state.X64:
        a = a.astype(_np.float32)
    return _wrap(a)


def zeros(shape, dtype=None):
    return _wrap(_np.zeros(shape, dtype=_canon_dtype(dtype or _default_float())))


def ones(shape, dtype=None):
    return _wrap(_np.ones(shape, dtype=_canon_dtype(dtype or _default_float())))


def zeros_like(x, dtype=None):
    return _wrap(_np.zeros_like(_canon(x), dtype=dtype))


def ones_like(x, dtype=None):
    return _wrap(_np.ones_like(_canon(x), dtype=dtype))


def full(shape, fill_value, dtype=None):
    fv = _canon(fill_value)
    if dtype is None and _is_weak(fill_value):
        dtype = _np.int64 if isinstance(fill_value, numbers.Integral) else _default_float()
    return _wrap(_np.full(shape, _unwrap_tree(fv), dtype=None if dtype is None else _canon_dtype(dtype)))


def full_like(x, fill_value, dtype=None):
    return _wrap(_np.full_like(_canon(x), fill_value, dtype=dtype))


def arange(*args, dtype=None):
    a = _np.arange(*args)
    return _wrap(a if dtype is None else a.astype(_canon_dtype(dtype)))


def linspace(start, stop, num=50, endpoint=True, dtype=None):
    a = _np.linspace(start, stop, num, endpoint=endpoint)
    if dtype is None:
        a = a.astype(_default_float())
    return _wrap(a if dtype is None else a.astype(_canon_dtype(dtype)))


def eye(n, m=None, dtype=None):
    return _wrap(_np.eye(n, m, dtype=_canon_dtype(dtype or _default_float())))


def diag(x, k=0):
    return _wrap(_np.diag(_canon(x), k))


def meshgrid(*xs, indexing="xy"):
    return tuple(_wrap(a) for a in _np.meshgrid(*[_canon(x) for x in xs], indexing=indexing))


# -------------------------------------------------------------- elementwise

def _ufunc(name):
    f = getattr(_np, name)

    def g(*args, **kwargs):
        return _wrap(f(*_promote(*args), **kwargs))

    g.__name__ = name
    return g


abs = _ufunc("abs")  # noqa: A001
sqrt = _ufunc("sqrt")
cos = _ufunc("cos")
sin = _ufunc("sin")
exp = _ufunc("exp")
floor = _ufunc("floor")
maximum = _ufunc("maximum")
minimum = _ufunc("minimum")
sign = _ufunc("sign")


def where(cond, x, y):
    c = _canon(cond)
    xx, yy = _promote(x, y)
    return _wrap(_np.where(c, xx, yy))


# --------------------------------------------------------------- reductions

def sum(x, axis=None, keepdims=False):  # noqa: A001
    a = _canon(x)
    return _wrap(_np.sum(a, axis=axis, keepdims=keepdims, dtype=a.dtype))


def mean(x, axis=None, keepdims=False):
    a = _canon(x)
    return _wrap(_np.mean(a, axis=axis, keepdims=keepdims, dtype=a.dtype))


def max(x, axis=None):  # noqa: A001
    return _wrap(_np.max(_canon(x), axis=axis))


def min(x, axis=None):  # noqa: A001
    return _wrap(_np.min(_canon(x), axis=axis))


# ------------------------------------------------------------------- shapes

def stack(xs, axis=0):
    return _wrap(_np.stack(_promote(*xs), axis=axis))


def concatenate(xs, axis=0):
    return _wrap(_np.concatenate(_promote(*xs), axis=axis))


def repeat(x, repeats, axis=None):
    return _wrap(_np.repeat(_canon(x), repeats, axis=axis))


def roll(x, shift, axis=None):
    return _wrap(_np.roll(_canon(x), shift, axis=axis))


def pad(x, pad_width, mode="constant"):
    return _wrap(_np.pad(_canon(x), pad_width, mode=mode))


def swapaxes(x, axis1, axis2):
    return _wrap(_np.swapaxes(_canon(x), axis1, axis2))


def moveaxis(x, source, destination):
    return _wrap(_np.moveaxis(_canon(x), source, destination))


def take(x, indices, axis=None):
    return _wrap(_np.take(_canon(x), _canon(indices), axis=axis))


def broadcast_to(x, shape):
    return _wrap(_np.broadcast_to(_canon(x), shape))


def reshape(x, shape):
    return _wrap(_np.reshape(_canon(x), shape))


def ndim(x):
    return _np.ndim(x)


def shape(x):
    return _np.shape(x)


def isscalar(x):
    if _np.isscalar(x):
        return True
    return isinstance(x, _np.ndarray) and x.ndim == 0


# ------------------------------------------------------------ contractions

def einsum(subscripts, *operands, precision=None, optimize=None):
    ops = _promote(*operands)
    return _wrap(_np.einsum(subscripts, *ops))


def tensordot(a, b, axes=2, precision=None):
    aa, bb = _promote(a, b)
    return _wrap(_np.tensordot(aa, bb, axes=axes))


def dot(a, b, precision=None):
    aa, bb = _promote(a, b)
    return _wrap(_np.dot(aa, bb))


def matmul(a, b, precision=None):
    aa, bb = _promote(a, b)
    return _wrap(_np.matmul(aa, bb))


def cross(a, b, axis=-1):
    aa, bb = _promote(a, b)
    return _wrap(_np.cross(aa, bb, axis=axis))


def gradient(x, *varargs, axis=None):
    a = _canon(x)
    return _wrap(_np.gradient(a, *varargs, axis=axis))


from . import linalg  # noqa: E402,F401
