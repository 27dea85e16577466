"""``jax.lax`` control flow and slicing for the NumPy-backed JAX stand-in."""

import numpy as _np

from .numpy import _wrap, _canon, stack


def fori_loop(lower, upper, body_fun, init_val):
    val = init_val
    for i in range(int(lower), int(upper)):
        val = body_fun(i, val)
    return val


def scan(f, init, xs=None, length=None):
    n = length if xs is None else len(xs)
    carry = init
    ys = []
    for i in range(n):
        carry, y = f(carry, None if xs is None else xs[i])
        ys.append(y)
    if ys and ys[0] is not None:
        if isinstance(ys[0], tuple):
            ys = tuple(stack([y[k] for y in ys]) for k in range(len(ys[0])))
        else:
            ys = stack(ys)
    else:
        ys = None
    return carry, ys


def _clamped_starts(shape, starts, sizes):
    out = []
    for dim, s, n in zip(shape, starts, sizes):
        s = int(_np.asarray(s))
        out.append(min(max(s, 0), dim - n))
    return out


def dynamic_slice(operand, start_indices, slice_sizes):
    a = _canon(operand)
    st = _clamped_starts(a.shape, start_indices, slice_sizes)
    sl = tuple(slice(s, s + n) for s, n in zip(st, slice_sizes))
    return _wrap(a[sl].copy())


def dynamic_update_slice(operand, update, start_indices):
    a = _canon(operand).copy()
    u = _canon(update)
    st = _clamped_starts(a.shape, start_indices, u.shape)
    sl = tuple(slice(s, s + n) for s, n in zip(st, u.shape))
    a[sl] = u
    return _wrap(a)
