"""``jax.numpy.linalg`` subset for the NumPy-backed JAX stand-in."""

import numpy as _np

from . import _promote, _wrap, _canon


def norm(x, ord=None, axis=None):  # noqa: A002
    return _wrap(_np.linalg.norm(_canon(x), ord=ord, axis=axis))


def solve(a, b):
    aa, bb = _promote(a, b)
    return _wrap(_np.linalg.solve(aa, bb))


def inv(a):
    return _wrap(_np.linalg.inv(_canon(a)))
