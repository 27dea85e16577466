"""The per-operator kernels as JAX custom calls (XLA FFI), for a ``jax.jit`` update step.

Needs jaxlib: its FFI headers (``jax.ffi.include_dir()``) compile ``xla/vs_xla_ffi.cc``
against libvivsim_gb300 on first use.  Without JAX, importing this module works and the
functions raise ImportError.  This build environment has no JAX, so the adapter is not
compiled or tested here.

    from vivsim_gb300 import jax_ffi as vj
    f = vj.collision_kbc(f, feq, omega)     # drop-in for vivsim.lbm.collision_kbc
"""

import ctypes
import os
import subprocess

from . import _build

HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(HERE, "xla", "vs_xla_ffi.cc")
_OUT = os.path.join(_build.OUT, "libvivsim_gb300_xla.so")
_TARGETS = {"vivsim_streaming": "VsStreaming", "vivsim_macroscopic": "VsMacroscopic",
            "vivsim_equilibrium": "VsEquilibrium", "vivsim_collision": "VsCollision"}
_REGISTERED = False


def _jax():
    try:
        import jax
        import jax.numpy as jnp
    except ImportError as e:  # no JAX: the adapter cannot be used
        raise ImportError("vivsim_gb300.jax_ffi needs jax and jaxlib") from e
    return jax, jnp


def build():
    """Compile the FFI handlers (g++, C++17) and link them against libvivsim_gb300."""
    jax, _ = _jax()
    lib = _build.build()
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if not os.path.exists(_OUT) or os.path.getmtime(_OUT) < max(os.path.getmtime(_SRC), os.path.getmtime(lib)):
        cmd = ["g++", "-std=c++17", "-O2", "-shared", "-fPIC", _SRC, "-o", _OUT, "-I", jax.ffi.include_dir(),
               "-I", os.path.join(_build.ROOT, "include"), "-I", os.path.join(cuda, "include"),
               "-L", os.path.dirname(lib), "-lvivsim_gb300", "-Wl,-rpath," + os.path.dirname(lib)]
        subprocess.run(cmd, check=True)
    return _OUT


def register():
    """Register the custom-call targets with XLA for the CUDA platform (once)."""
    global _REGISTERED
    if _REGISTERED:
        return
    jax, _ = _jax()
    so = ctypes.CDLL(build())
    for name, symbol in _TARGETS.items():
        jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(getattr(so, symbol)), platform="CUDA")
    _REGISTERED = True


def streaming(f):
    """lbm/basic.py:60-85, lbm3d/basic.py:52-87"""
    jax, _ = _jax()
    register()
    return jax.ffi.ffi_call("vivsim_streaming", jax.ShapeDtypeStruct(f.shape, f.dtype))(f)


def get_macroscopic(f):
    """lbm/basic.py:88-111, lbm3d/basic.py:90-106"""
    jax, _ = _jax()
    register()
    grid = f.shape[1:]
    out = (jax.ShapeDtypeStruct(grid, f.dtype), jax.ShapeDtypeStruct((len(grid),) + grid, f.dtype))
    return jax.ffi.ffi_call("vivsim_macroscopic", out)(f)


def get_equilibrium(rho, u):
    """lbm/basic.py:114-135, lbm3d/basic.py:109-130"""
    jax, _ = _jax()
    register()
    q = 9 if u.shape[0] == 2 else 19
    return jax.ffi.ffi_call("vivsim_equilibrium", jax.ShapeDtypeStruct((q,) + rho.shape, rho.dtype))(rho, u)


def _collision(kind):
    def fn(f, feq, omega):
        jax, _ = _jax()
        register()
        import numpy as np
        call = jax.ffi.ffi_call("vivsim_collision", jax.ShapeDtypeStruct(f.shape, f.dtype))
        return call(f, feq, kind=np.int32(kind), omega=np.float64(omega))
    return fn


collision_bgk = _collision(0)   # lbm/basic.py:138-156
collision_kbc = _collision(1)   # lbm/collision/kbc.py:10-60
collision_reg = _collision(3)   # lbm/collision/reg.py:4-49

__all__ = ["build", "register", "streaming", "get_macroscopic", "get_equilibrium", "collision_bgk",
           "collision_kbc", "collision_reg"]
