"""NumPy-backed stand-in for the small part of the JAX API that vivsim uses.

JAX is not installed where the golden fixtures are generated, so this package lets
the reference's own Python source (``vivsim.lbm``, ``vivsim.lbm3d``, ``vivsim.ib``,
``vivsim.ib3d``, ``vivsim.dyn``) run unchanged on NumPy arrays.  It reproduces the
JAX semantics that matter for those functions:

* immutable-array updates (``x.at[idx].set/add``) and rebinding augmented
  assignment (``x -= y`` makes a new array, it never writes into a caller's array);
* JAX's dtype canonicalisation: with ``jax_enable_x64`` off every float64 value
  becomes float32 and every int64 becomes int32 before and after each operation,
  while Python scalars stay weakly typed;
* out-of-line control flow (``lax.fori_loop``, ``lax.scan``) as plain loops and
  ``lax.dynamic_slice`` / ``dynamic_update_slice`` with JAX's start-index clamping.

It is test infrastructure: only ``tests/golden/make_golden.py`` imports it.
"""

from types import SimpleNamespace

from . import _state
from . import numpy  # noqa: F401  (exposes jax.numpy)
from . import lax  # noqa: F401
from .numpy import JArray as Array


class _Config:
    def update(self, name, value):
        if name == "jax_enable_x64":
            _state.X64 = bool(value)
        else:
            raise KeyError(name)


config = _Config()


def jit(fn=None, **kwargs):
    if fn is None:
        return lambda f: f
    return fn


def block_until_ready(x):
    return x


def devices():
    return [SimpleNamespace(platform="cpu")]
