"""The library's kernels as JAX custom calls (XLA FFI), for a ``jax.jit`` update step.

Needs jaxlib: its FFI headers (``jax.ffi.include_dir()``) compile ``xla/vs_xla_ffi.cc``
against libvivsim_gb300 on first use.  Without JAX, importing this module works and every
function raises ImportError.

The names and argument meanings are the reference's (vivsim/lbm/__init__.py:1-42,
vivsim/lbm3d/__init__.py, vivsim/ib/__init__.py:3-6, vivsim/dyn.py:5-154):

    from vivsim_gb300 import jax_ffi as vj
    lbm = vj.lbm                               # D2Q9; vj.lbm3d for D3Q19
    rho, u = lbm.get_macroscopic(f)
    f = lbm.collision_kbc(f, lbm.get_equilibrium(rho, u), omega)
    g, h = vj.ib.multi_direct_forcing(u, W, I, u_target, ds, n_iter=3)

``streaming``, ``get_macroscopic``, ``get_equilibrium``, the BGK / KBC / regularised
collisions, ``forcing_edm``, ``interpolate``, ``spread`` and the scalar ``newmark`` carry a
``jax.custom_vjp`` whose backward runs the library's VJP kernels (interpolate and spread
are each other's transpose), so ``jax.grad`` of a composed step works.  Relaxation rates,
wall values and Newmark coefficients are static (attributes of the call) and get no
cotangent here.  ``run`` advances a library plan (solver.LatticeStep / RigidBody) by
n_steps fused steps with the population array donated (``input_output_aliases``).
"""

import ctypes
import functools
import os
import subprocess

import numpy as np

from . import _build
from . import _lib as V

HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(HERE, "xla", "vs_xla_ffi.cc")
_OUT = os.path.join(_build.OUT, "libvivsim_gb300_xla.so")

# custom-call target name -> exported handler symbol of vs_xla_ffi.cc
TARGETS = {
    "vivsim_streaming": "VsStreaming", "vivsim_macroscopic": "VsMacroscopic", "vivsim_equilibrium": "VsEquilibrium",
    "vivsim_collision": "VsCollision", "vivsim_collision_mrt": "VsCollisionMrt",
    "vivsim_guo_forcing_term": "VsGuoForcingTerm", "vivsim_forcing": "VsForcing",
    "vivsim_forcing_guo_mrt": "VsForcingGuoMrt", "vivsim_velocity_correction": "VsVelocityCorrection",
    "vivsim_boundary": "VsBoundary", "vivsim_boundary_arrays": "VsBoundaryArrays",
    "vivsim_obstacle_bounce_back": "VsObstacleBounceBack", "vivsim_characteristic": "VsCharacteristic",
    "vivsim_ib_kernel": "VsIbKernel", "vivsim_ib_stencil_2d": "VsIbStencil2d", "vivsim_ib_stencil_3d": "VsIbStencil3d",
    "vivsim_interpolate": "VsInterpolate", "vivsim_spread": "VsSpread", "vivsim_mdf": "VsMdf",
    "vivsim_newmark": "VsNewmark", "vivsim_newmark_matrix": "VsNewmarkMatrix", "vivsim_force_to_obj": "VsForceToObj",
    "vivsim_run": "VsRun", "vivsim_streaming_vjp": "VsStreamingVjp", "vivsim_macroscopic_vjp": "VsMacroscopicVjp",
    "vivsim_equilibrium_vjp": "VsEquilibriumVjp", "vivsim_collision_vjp": "VsCollisionVjp",
    "vivsim_collision_mrt_vjp": "VsCollisionMrtVjp", "vivsim_forcing_vjp": "VsForcingVjp",
    "vivsim_boundary_vjp": "VsBoundaryVjp", "vivsim_ib_pair_dot": "VsIbPairDot",
    "vivsim_ib_stencil_vjp_2d": "VsIbStencilVjp2d", "vivsim_ib_stencil_vjp_3d": "VsIbStencilVjp3d",
    "vivsim_newmark_vjp": "VsNewmarkVjp",
}
_REGISTERED = False
_KERNELS = {"peskin3": V.VS_KERNEL_PESKIN3, "peskin4": V.VS_KERNEL_PESKIN4, "cosine4": V.VS_KERNEL_COSINE4,
            "kernel_peskin_3pt": V.VS_KERNEL_PESKIN3, "kernel_peskin_4pt": V.VS_KERNEL_PESKIN4,
            "kernel_cosine_4pt": V.VS_KERNEL_COSINE4}


def _kernel_code(kernel):
    """A delta kernel given as the reference's function (vivsim/ib/kernels.py) or its name."""
    name = kernel if isinstance(kernel, str) else getattr(kernel, "__name__", "")
    if name not in _KERNELS:
        raise ValueError("kernel must be kernel_peskin_3pt, kernel_peskin_4pt or kernel_cosine_4pt")
    return _KERNELS[name]


def _jax():
    try:
        import jax
        import jax.numpy as jnp
    except ImportError as e:  # no JAX: the adapter cannot be used
        raise ImportError("vivsim_gb300.jax_ffi needs jax and jaxlib") from e
    return jax, jnp


def compile_command(include_dir, lib_dir, out=_OUT):
    """The g++ command line that builds the handler library (C++17, shared)."""
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    return ["g++", "-std=c++17", "-O2", "-shared", "-fPIC", _SRC, "-o", out, "-I", include_dir,
            "-I", os.path.join(_build.ROOT, "include"), "-I", os.path.join(cuda, "include"),
            "-L", lib_dir, "-lvivsim_gb300", "-Wl,-rpath," + lib_dir, "-L", os.path.join(cuda, "lib64"), "-lcudart"]


def build():
    """Compile the FFI handlers and link them against libvivsim_gb300."""
    jax, _ = _jax()
    lib = _build.build()
    if not os.path.exists(_OUT) or os.path.getmtime(_OUT) < max(os.path.getmtime(_SRC), os.path.getmtime(lib)):
        subprocess.run(compile_command(jax.ffi.include_dir(), os.path.dirname(lib)), check=True)
    return _OUT


def register():
    """Register every custom-call target with XLA for the CUDA platform (once)."""
    global _REGISTERED
    if _REGISTERED:
        return
    jax, _ = _jax()
    so = ctypes.CDLL(build())
    for name, symbol in TARGETS.items():
        jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(getattr(so, symbol)), platform="CUDA")
    _REGISTERED = True


def _call(target, out, *args, **attrs):
    jax, _ = _jax()
    register()
    return jax.ffi.ffi_call(target, out)(*args, **attrs)


def _sds(shape, dtype):
    jax, _ = _jax()
    return jax.ShapeDtypeStruct(tuple(shape), dtype)


def _f64(x):
    return np.float64(x)


def _i32(x):
    return np.int32(x)


# ------------------------------------------------------------------ the raw calls
def _streaming(f):
    return _call("vivsim_streaming", _sds(f.shape, f.dtype), f)


def _streaming_vjp(g):
    return _call("vivsim_streaming_vjp", _sds(g.shape, g.dtype), g)


def _macroscopic(f):
    grid = f.shape[1:]
    return _call("vivsim_macroscopic", (_sds(grid, f.dtype), _sds((len(grid),) + grid, f.dtype)), f)


def _equilibrium(rho, u):
    q = 9 if u.shape[0] == 2 else 19
    return _call("vivsim_equilibrium", _sds((q,) + rho.shape, rho.dtype), rho, u)


def _collision(kind, f, feq, omega):
    return _call("vivsim_collision", _sds(f.shape, f.dtype), f, feq, kind=_i32(kind), omega=_f64(omega))


def _forcing(kind, f, g, u, omega):
    return _call("vivsim_forcing", _sds(f.shape, f.dtype), f, g, u, kind=_i32(kind), omega=_f64(omega))


def _interpolate(grid, W, I):
    return _call("vivsim_interpolate", _sds((W.shape[0], grid.shape[0]), grid.dtype), grid, W, I)


def _spread(values, grid, W, I):
    return _call("vivsim_spread", _sds(grid.shape, grid.dtype), values, grid, W, I)


def _pair_dot(A, grid, I):
    return _call("vivsim_ib_pair_dot", _sds(I.shape, grid.dtype), A, grid, I)


# ---------------------------------------------------------------- differentiable
def _make_differentiable():
    """custom_vjp wrappers, built on first use (they need jax)."""
    jax, jnp = _jax()

    @jax.custom_vjp
    def streaming(f):
        return _streaming(f)

    streaming.defvjp(lambda f: (_streaming(f), None), lambda _, g: (_streaming_vjp(g),))

    @jax.custom_vjp
    def get_macroscopic(f):
        return _macroscopic(f)

    def mac_bwd(f, g):
        g_rho, g_u = g
        return (_call("vivsim_macroscopic_vjp", _sds(f.shape, f.dtype), f, g_rho, g_u),)

    get_macroscopic.defvjp(lambda f: (_macroscopic(f), f), mac_bwd)

    @jax.custom_vjp
    def get_equilibrium(rho, u):
        return _equilibrium(rho, u)

    def eq_bwd(res, g):
        rho, u = res
        return _call("vivsim_equilibrium_vjp", (_sds(rho.shape, rho.dtype), _sds(u.shape, u.dtype)), rho, u, g)

    get_equilibrium.defvjp(lambda rho, u: (_equilibrium(rho, u), (rho, u)), eq_bwd)

    def collision(kind):
        @functools.partial(jax.custom_vjp, nondiff_argnums=(2,))
        def fn(f, feq, omega):
            return _collision(kind, f, feq, omega)

        def bwd(omega, res, g):
            f, feq = res
            n = int(np.prod(f.shape[1:]))
            g_f, g_feq, _ = _call("vivsim_collision_vjp", (_sds(f.shape, f.dtype), _sds(f.shape, f.dtype),
                                                          _sds((n,), f.dtype)), f, feq, g, kind=_i32(kind),
                                  omega=_f64(omega))
            return g_f, g_feq

        fn.defvjp(lambda f, feq, omega: (_collision(kind, f, feq, omega), (f, feq)), bwd)
        return fn

    @jax.custom_vjp
    def forcing_edm(f, g, u):
        return _forcing(V.VS_FORCE_EDM, f, g, u, 0.0)

    def edm_bwd(res, gout):
        f_shape, f_dtype, g, u = res
        n = int(np.prod(u.shape[1:]))
        g_g, g_u, _ = _call("vivsim_forcing_vjp", (_sds(g.shape, g.dtype), _sds(u.shape, u.dtype),
                                                  _sds((n,), u.dtype)), g, u, gout, kind=_i32(V.VS_FORCE_EDM),
                            omega=_f64(0.0))
        return gout, g_g, g_u

    forcing_edm.defvjp(lambda f, g, u: (_forcing(V.VS_FORCE_EDM, f, g, u, 0.0), (f.shape, f.dtype, g, u)), edm_bwd)

    # interpolate^T = spread and spread^T = interpolate; the weights' cotangent is a pair dot
    @jax.custom_vjp
    def interpolate(grid, W, I):
        return _interpolate(grid, W, I)

    def interp_bwd(res, g):
        grid, W, I = res
        g_grid = _spread(g, jnp.zeros_like(grid), W, I)
        return g_grid, _pair_dot(g, grid, I), None

    interpolate.defvjp(lambda grid, W, I: (_interpolate(grid, W, I), (grid, W, I)), interp_bwd)

    @jax.custom_vjp
    def spread(values, grid, W, I):
        return _spread(values, grid, W, I)

    def spread_bwd(res, g):
        values, W, I = res
        return _interpolate(g, W, I), g, _pair_dot(values, g, I), None

    spread.defvjp(lambda values, grid, W, I: (_spread(values, grid, W, I), (values, W, I)), spread_bwd)

    @functools.partial(jax.custom_vjp, nondiff_argnums=(4, 5, 6, 7, 8, 9))
    def newmark(a, v, d, h, m, k, c, dt, gamma, beta):
        return _newmark(a, v, d, h, m, k, c, dt, gamma, beta)

    def nm_fwd(a, v, d, h, m, k, c, dt, gamma, beta):
        return _newmark(a, v, d, h, m, k, c, dt, gamma, beta), (a, v, d, h)

    def nm_bwd(m, k, c, dt, gamma, beta, res, g):
        a, v, d, h = res
        ga, gv, gd = g
        s = _sds(a.shape, a.dtype)
        out = _call("vivsim_newmark_vjp", (s, s, s, s, _sds((3,), a.dtype)), a, v, d, h, ga, gv, gd, m=_f64(m),
                    k=_f64(k), c=_f64(c), dt=_f64(dt), gamma=_f64(gamma), beta=_f64(beta))
        return out[0], out[1], out[2], out[3]

    newmark.defvjp(nm_fwd, nm_bwd)
    return dict(streaming=streaming, get_macroscopic=get_macroscopic, get_equilibrium=get_equilibrium,
                collision_bgk=collision(V.VS_COLLIDE_BGK), collision_kbc=collision(V.VS_COLLIDE_KBC),
                collision_reg=collision(V.VS_COLLIDE_REG), forcing_edm=forcing_edm, interpolate=interpolate,
                spread=spread, newmark=newmark)


@functools.lru_cache(maxsize=1)
def _diff():
    return _make_differentiable()


def _newmark(a, v, d, h, m, k, c, dt, gamma, beta):
    s = _sds(a.shape, a.dtype)
    return _call("vivsim_newmark", (s, s, s), a, v, d, h, m=_f64(m), k=_f64(k), c=_f64(c), dt=_f64(dt),
                 gamma=_f64(gamma), beta=_f64(beta))


# ------------------------------------------------------------------- lattice ops
class JaxLattice:
    """The per-operator functions of one velocity set (vivsim.lbm or vivsim.lbm3d)."""

    def __init__(self, q):
        self.q = q
        self.d = 2 if q == 9 else 3
        self.locs = ("left", "right", "top", "bottom") if q == 9 else \
            ("left", "right", "bottom", "top", "back", "front")

    def streaming(self, f):
        return _diff()["streaming"](f)

    def get_macroscopic(self, f):
        return _diff()["get_macroscopic"](f)

    def get_equilibrium(self, rho, u):
        return _diff()["get_equilibrium"](rho, u)

    def collision_bgk(self, f, feq, omega):
        return _diff()["collision_bgk"](f, feq, float(omega))

    def collision_kbc(self, f, feq, omega):
        return _diff()["collision_kbc"](f, feq, float(omega))

    def collision_reg(self, f, feq, omega):
        return _diff()["collision_reg"](f, feq, float(omega))

    def collision_mrt(self, f, feq, mrt_collision_operator):
        op = np.ascontiguousarray(np.asarray(mrt_collision_operator, np.float64).reshape(-1))
        return _call("vivsim_collision_mrt", _sds(f.shape, f.dtype), f, feq, op=op)

    @staticmethod
    def get_omega(nu):
        return 1 / (3 * nu + 0.5)

    def get_velocity_correction(self, g, rho=1):
        _, jnp = _jax()
        rho = rho if hasattr(rho, "shape") else jnp.full(g.shape[1:], rho, g.dtype)
        return _call("vivsim_velocity_correction", _sds(g.shape, g.dtype), g, rho)

    def get_guo_forcing_term(self, g, u):
        return _call("vivsim_guo_forcing_term", _sds((self.q,) + g.shape[1:], g.dtype), g, u)

    def forcing_edm(self, f, g, u):
        return _diff()["forcing_edm"](f, g, u)

    def forcing_guo_bgk(self, f, g, u, omega):
        return _forcing(V.VS_FORCE_GUO_BGK, f, g, u, omega)

    def forcing_guo_mrt(self, f, g, u, mrt_forcing_operator):
        op = np.ascontiguousarray(np.asarray(mrt_forcing_operator, np.float64).reshape(-1))
        return _call("vivsim_forcing_guo_mrt", _sds(f.shape, f.dtype), f, g, u, op=op)

    def _loc(self, loc):
        if loc not in self.locs:
            raise ValueError(f"loc must be one of: {', '.join(repr(x) for x in self.locs)}")
        return V.LOCS[loc]

    def boundary(self, kind, mode, f, loc, f_before_stream=None, rho=1.0, ux=0.0, uy=0.0, uz=0.0, gx=0.0, gy=0.0,
                 gz=0.0):
        """One face boundary with scalar wall values (kind VS_BC_*, mode VS_WALL_*)."""
        pre = f if f_before_stream is None else f_before_stream
        return _call("vivsim_boundary", _sds(f.shape, f.dtype), f, pre, kind=_i32(kind), mode=_i32(mode),
                     loc=_i32(self._loc(loc)), rho=_f64(rho), ux=_f64(ux), uy=_f64(uy), uz=_f64(uz), gx=_f64(gx),
                     gy=_f64(gy), gz=_f64(gz))

    def boundary_nee(self, f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0):
        return self.boundary(V.VS_BC_NEE, V.VS_WALL_GIVEN, f, loc, rho=rho_wall, ux=ux_wall, uy=uy_wall, uz=uz_wall)

    def boundary_velocity_nee(self, f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
        return self.boundary(V.VS_BC_NEE, V.VS_WALL_VELOCITY, f, loc, ux=ux_wall, uy=uy_wall, uz=uz_wall)

    def boundary_pressure_nee(self, f, loc, rho_wall=1):
        return self.boundary(V.VS_BC_NEE, V.VS_WALL_PRESSURE, f, loc, rho=rho_wall)

    def boundary_nebb(self, f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0):
        return self.boundary(V.VS_BC_NEBB, V.VS_WALL_GIVEN, f, loc, rho=rho_wall, ux=ux_wall, uy=uy_wall, uz=uz_wall)

    def boundary_velocity_nebb(self, f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
        return self.boundary(V.VS_BC_NEBB, V.VS_WALL_VELOCITY, f, loc, ux=ux_wall, uy=uy_wall, uz=uz_wall)

    def boundary_pressure_nebb(self, f, loc, rho_wall=1):
        return self.boundary(V.VS_BC_NEBB, V.VS_WALL_PRESSURE, f, loc, rho=rho_wall)

    def boundary_equilibrium(self, f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0):
        return self.boundary(V.VS_BC_EQ, V.VS_WALL_GIVEN, f, loc, rho=rho_wall, ux=ux_wall, uy=uy_wall, uz=uz_wall)

    def boundary_velocity_equilibrium(self, f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
        return self.boundary(V.VS_BC_EQ, V.VS_WALL_VELOCITY, f, loc, ux=ux_wall, uy=uy_wall, uz=uz_wall)

    def boundary_pressure_equilibrium(self, f, loc, rho_wall=1):
        return self.boundary(V.VS_BC_EQ, V.VS_WALL_PRESSURE, f, loc, rho=rho_wall)

    def boundary_bounce_back(self, f_before_stream, f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
        return self.boundary(V.VS_BC_BB, V.VS_WALL_GIVEN, f, loc, f_before_stream, ux=ux_wall, uy=uy_wall, uz=uz_wall)

    def boundary_specular_reflection(self, f_before_stream, f, loc):
        return self.boundary(V.VS_BC_SPECULAR, V.VS_WALL_GIVEN, f, loc, f_before_stream)

    def obstacle_bounce_back(self, f, mask):
        return _call("vivsim_obstacle_bounce_back", _sds(f.shape, f.dtype), f, mask.astype(np.uint8))

    def boundary_characteristic(self, rho, u, loc="right"):
        code = self._loc(loc)
        axis = {0: 0, 1: 0, 2: 1, 3: 1, 4: 2, 5: 2}[code]
        face = tuple(n for a, n in enumerate(rho.shape) if a != axis)
        return _call("vivsim_characteristic", (_sds(face, rho.dtype), _sds((self.d,) + face, rho.dtype)), rho, u,
                     loc=_i32(code))


lbm = JaxLattice(9)
lbm3d = JaxLattice(19)


# ------------------------------------------------------------------------ IB ops
class _IB:
    """vivsim.ib / vivsim.ib3d on the device."""

    @staticmethod
    def kernel(r, kernel="kernel_peskin_4pt"):
        return _call("vivsim_ib_kernel", _sds(r.shape, r.dtype), r, kernel=_i32(_kernel_code(kernel)))

    @staticmethod
    def get_ib_stencil(marker_x, marker_y, ny, kernel="kernel_peskin_4pt", stencil_radius=2):
        """ib/stencil.py:7-51: W (M, (2r)^2), I int32"""
        m, s = marker_x.shape[0], (2 * stencil_radius) ** 2
        return _call("vivsim_ib_stencil_2d", (_sds((m, s), marker_x.dtype), _sds((m, s), np.int32)), marker_x,
                     marker_y, kernel=_i32(_kernel_code(kernel)), radius=_i32(stencil_radius), ny=_i32(ny))

    @staticmethod
    def get_ib_stencil_3d(coords, shape, kernel="kernel_peskin_4pt", stencil_radius=2):
        """ib3d/stencil.py:7-59: W (M, (2r)^3), I int32"""
        m, s = coords.shape[0], (2 * stencil_radius) ** 3
        return _call("vivsim_ib_stencil_3d", (_sds((m, s), coords.dtype), _sds((m, s), np.int32)), coords,
                     kernel=_i32(_kernel_code(kernel)), radius=_i32(stencil_radius), nx=_i32(shape[0]),
                     ny=_i32(shape[1]), nz=_i32(shape[2]))

    @staticmethod
    def interpolate(grid, W, I):
        return _diff()["interpolate"](grid, W, I)

    @staticmethod
    def spread(values, grid, W, I):
        return _diff()["spread"](values, grid, W, I)

    @staticmethod
    def multi_direct_forcing(u, W, I, u_target, ds, n_iter=3):
        """ib/mdf.py:10-64: (grid force, marker force); ds per marker (M,) or a scalar"""
        _, jnp = _jax()
        per_marker = hasattr(ds, "shape") and len(ds.shape) == 1
        ds_arr = ds if per_marker else jnp.zeros((1,), u.dtype)
        return _call("vivsim_mdf", (_sds(u.shape, u.dtype), _sds((W.shape[0], u.shape[0]), u.dtype)), u, W, I,
                     u_target, ds_arr, n_iter=_i32(n_iter), per_marker_ds=_i32(per_marker),
                     ds=_f64(0.0 if per_marker else ds))


ib = _IB()


# ---------------------------------------------------------------------- dynamics
class _Dyn:
    """vivsim.dyn on the device."""

    @staticmethod
    def newmark(a, v, d, h, m, k, c, dt=1, gamma=0.5, beta=0.25):
        """dyn.py:5-51; m, k, c scalars (differentiable in a, v, d, h) or ndof x ndof matrices"""
        if np.ndim(m) == 2:
            s = _sds(a.shape, a.dtype)
            return _call("vivsim_newmark_matrix", (s, s, s), a, v, d, h, m, k, c, dt=_f64(dt), gamma=_f64(gamma),
                         beta=_f64(beta))
        return _diff()["newmark"](a, v, d, h, float(m), float(k), float(c), float(dt), float(gamma), float(beta))

    @staticmethod
    def get_force_to_obj(h):
        return _call("vivsim_force_to_obj", _sds((h.shape[1],), h.dtype), h)


dyn = _Dyn()


# ---------------------------------------------------------------------- fused run
def run(f, lattice, body=None, n_steps=1):
    """n_steps fused steps (vs_run) of a solver.LatticeStep and optional solver.RigidBody;
    returns (f, force history (n_steps, 3)).  f is donated to the result."""
    jax, _ = _jax()
    register()
    hist = (n_steps, 3) if body is not None else (0, 3)
    call = jax.ffi.ffi_call("vivsim_run", (_sds(f.shape, f.dtype), _sds(hist, f.dtype)),
                            input_output_aliases={0: 0})
    return call(f, lattice=np.int64(lattice.handle.value), body=np.int64(body.handle.value if body else 0),
                n_steps=np.int32(n_steps))


__all__ = ["build", "register", "compile_command", "TARGETS", "JaxLattice", "lbm", "lbm3d", "ib", "dyn", "run"]
