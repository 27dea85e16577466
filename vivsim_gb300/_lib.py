"""ctypes binding of ``libvivsim_gb300.so`` (the C ABI declared in include/vivsim_gb300.h).

The library is loaded from the in-tree build directory.  There is no fallback: if the
library or a CUDA device is missing, every operator raises.
"""

import ctypes as C
import os

import torch

from . import _build

VS_OK = 0
VS_ERR_INVALID_ARG = 1
VS_ERR_TIMEOUT = 5
VS_ERR_NONFINITE = 6
VS_ERR_TIMEOUT_INFLIGHT = 7
VS_F32, VS_F64 = 0, 1
VS_COLLIDE_BGK, VS_COLLIDE_KBC, VS_COLLIDE_MRT, VS_COLLIDE_REG = 0, 1, 2, 3
VS_FORCE_NONE, VS_FORCE_EDM, VS_FORCE_GUO_BGK, VS_FORCE_GUO_MRT = 0, 1, 2, 3
VS_LEFT, VS_RIGHT, VS_BOTTOM, VS_TOP, VS_BACK, VS_FRONT = range(6)
VS_BC_NEE, VS_BC_NEBB, VS_BC_EQ, VS_BC_BB, VS_BC_SPECULAR = range(5)
VS_WALL_GIVEN, VS_WALL_VELOCITY, VS_WALL_PRESSURE, VS_WALL_FORCE_CORRECTED, VS_WALL_CHARACTERISTIC = range(5)
VS_KERNEL_PESKIN3, VS_KERNEL_PESKIN4, VS_KERNEL_COSINE4 = range(3)
VS_MAX_BC = 8
VS_GRID_AUTO, VS_GRID_PLAIN, VS_GRID_TMA = 0, 1, 2
VS_RUN_STEPS, VS_RUN_PERSISTENT = 0, 1

REFINE_DIRS = {"left": 0, "right": 1, "up": 2, "down": 3}
LOCS = {"left": VS_LEFT, "right": VS_RIGHT, "bottom": VS_BOTTOM, "top": VS_TOP, "back": VS_BACK,
        "front": VS_FRONT}


class VivsimError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, fn, status, msg):
        super().__init__(f"{fn}: {msg} (status {status})")
        self.status = status


class vs_wall(C.Structure):
    _fields_ = [("rho", C.c_double), ("ux", C.c_double), ("uy", C.c_double), ("uz", C.c_double),
                ("gx", C.c_double), ("gy", C.c_double), ("gz", C.c_double),
                ("rho_arr", C.c_void_p), ("ux_arr", C.c_void_p), ("uy_arr", C.c_void_p), ("uz_arr", C.c_void_p)]


class vs_bc(C.Structure):
    _fields_ = [("kind", C.c_int), ("mode", C.c_int), ("loc", C.c_int),
                ("rho", C.c_double), ("ux", C.c_double), ("uy", C.c_double), ("uz", C.c_double),
                ("gx", C.c_double), ("gy", C.c_double), ("gz", C.c_double)]


class vs_lattice_cfg(C.Structure):
    _fields_ = [("q", C.c_int), ("dtype", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("collision", C.c_int), ("omega", C.c_double), ("mrt_op", C.c_double * 361),
                ("forcing", C.c_int), ("g_uniform", C.c_double * 3), ("mrt_fop", C.c_double * 361),
                ("n_bc", C.c_int), ("bc", vs_bc * VS_MAX_BC), ("variant", C.c_int),
                ("obstacle_mask", C.c_void_p), ("watchdog_every", C.c_int)]


class vs_body_cfg(C.Structure):
    _fields_ = [("dim", C.c_int), ("dtype", C.c_int), ("n_markers", C.c_int),
                ("x0_host", C.POINTER(C.c_double)), ("y0_host", C.POINTER(C.c_double)),
                ("z0_host", C.POINTER(C.c_double)), ("ds_host", C.POINTER(C.c_double)),
                ("ds_scalar", C.c_double), ("kernel", C.c_int), ("radius", C.c_int), ("n_iter", C.c_int),
                ("moving", C.c_int), ("free_dof", C.c_int * 3),
                ("mass", C.c_double), ("stiffness", C.c_double), ("damping", C.c_double),
                ("added_mass_area", C.c_double),
                ("d0", C.c_double * 3), ("v0", C.c_double * 3), ("a0", C.c_double * 3),
                ("window_margin", C.c_int),
                ("center_x", C.c_double), ("center_y", C.c_double),
                ("inertia", C.c_double), ("rot_stiffness", C.c_double), ("rot_damping", C.c_double),
                ("added_inertia", C.c_double), ("fsi_iter", C.c_int)]


class vs_adjoint_cfg(C.Structure):
    _fields_ = [("dtype", C.c_int), ("nx", C.c_int), ("ny", C.c_int),
                ("U0", C.c_double), ("D", C.c_double), ("Re", C.c_double), ("rho_out", C.c_double),
                ("n_markers", C.c_int), ("cx", C.c_double), ("cy", C.c_double),
                ("offsets_host", C.POINTER(C.c_double)),
                ("kernel", C.c_int), ("radius", C.c_int), ("n_iter", C.c_int),
                ("mass", C.c_double), ("stiffness", C.c_double), ("damping", C.c_double),
                ("added_mass_area", C.c_double),
                ("n_steps", C.c_int), ("checkpoint_every", C.c_int), ("obj_start", C.c_int),
                ("collision", C.c_int), ("mrt_op", C.c_double * 81), ("mrt_dop", C.c_double * 81)]


_i, _d, _p, _l, _z = C.c_int, C.c_double, C.c_void_p, C.c_int64, C.c_size_t
_SIGS = {
    "vs_last_error": (C.c_char_p, []),
    "vs_status_string": (C.c_char_p, [_i]),
    "vs_version": (_i, []),
    "vs_streaming": (_i, [_i, _i, _p, _p, _i, _i, _i, _p]),
    "vs_get_macroscopic": (_i, [_i, _i, _p, _p, _p, _l, _p]),
    "vs_get_equilibrium": (_i, [_i, _i, _p, _p, _p, _l, _p]),
    "vs_collision": (_i, [_i, _i, _i, _p, _p, _d, _p, _l, _p]),
    "vs_collision_mrt": (_i, [_i, _i, _p, _p, C.POINTER(_d), _p, _l, _p]),
    "vs_guo_forcing_term": (_i, [_i, _i, _p, _p, _p, _l, _p]),
    "vs_forcing": (_i, [_i, _i, _i, _p, _p, _p, _d, _p, _l, _p]),
    "vs_forcing_guo_mrt": (_i, [_i, _i, _p, _p, _p, C.POINTER(_d), _p, _l, _p]),
    "vs_velocity_correction": (_i, [_i, _i, _p, _p, _p, _l, _p]),
    "vs_boundary": (_i, [_i, _i, _i, _i, _i, _p, _p, _p, _i, _i, _i, C.POINTER(vs_wall), _p]),
    "vs_obstacle_bounce_back": (_i, [_i, _i, _p, _p, _p, _l, _p]),
    "vs_boundary_characteristic": (_i, [_i, _i, _i, _p, _p, _i, _i, _i, _p, _p, _p]),
    "vs_ib_kernel": (_i, [_i, _i, _p, _p, _l, _p]),
    "vs_ib_stencil_2d": (_i, [_i, _i, _i, _p, _p, _i, _i, _p, _p, _p]),
    "vs_ib_stencil_3d": (_i, [_i, _i, _i, _p, _i, _i, _i, _i, _p, _p, _p]),
    "vs_ib_interpolate": (_i, [_i, _p, _i, _l, _p, _p, _i, _i, _p, _p]),
    "vs_ib_workspace_bytes": (_z, [_i, _i]),
    "vs_ib_spread": (_i, [_i, _p, _p, _p, _i, _l, _p, _p, _i, _i, _p, _z, _p]),
    "vs_ib_mdf": (_i, [_i, _p, _i, _l, _p, _p, _i, _i, _p, _p, _d, _i, _p, _p, _p, _z, _p]),
    "vs_ib_spread_noalloc": (_i, [_i, _p, _p, _p, _i, _l, _p, _p, _i, _i, _p]),
    "vs_ib_status": (_i, [C.POINTER(C.c_uint), _i]),
    "vs_newmark": (_i, [_i, _i, _p, _p, _p, _p, _d, _d, _d, _p, _p, _p, _d, _d, _d, _p, _p, _p, _p]),
    "vs_markers_coords_2dof": (_i, [_i, _p, _p, _i, _p, _p, _p, _p]),
    "vs_markers_coords_3dof": (_i, [_i, _p, _p, _i, _d, _d, _p, _p, _p, _p]),
    "vs_markers_velocity_3dof": (_i, [_i, _p, _p, _i, _d, _d, _p, _p, _p, _p]),
    "vs_force_to_obj": (_i, [_i, _p, _i, _i, _p, _p]),
    "vs_torque_to_obj": (_i, [_i, _p, _p, _i, _d, _d, _p, _p, _p, _p]),
    "vs_lattice_plan_create": (_i, [C.POINTER(vs_lattice_cfg), C.POINTER(_p)]),
    "vs_lattice_plan_destroy": (_i, [_p]),
    "vs_body_plan_create": (_i, [C.POINTER(vs_body_cfg), _p, C.POINTER(_p)]),
    "vs_body_plan_destroy": (_i, [_p]),
    "vs_body_get_state": (_i, [_p, C.POINTER(_d), _p]),
    "vs_body_set_state": (_i, [_p, C.POINTER(_d), _p]),
    "vs_step": (_i, [_p, _p, _p, _p, _p, _p]),
    "vs_run": (_i, [_p, _p, _p, _p, _i, _p, _p]),
    "vs_run_graph": (_i, [_p, _p, _p, _p, _i, _p, _p]),
    "vs_run_persistent": (_i, [_p, _p, _i]),
    "vs_lattice_set_run_form": (_i, [_p, _i]),
    "vs_step_grid_only": (_i, [_p, _p, _p, _p, _p]),
    "vs_body_state_device": (_i, [_p, C.POINTER(C.c_void_p)]),
    "vs_body_set_state_device": (_i, [_p, _p, _p]),
    "vs_batch_plan_create": (_i, [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), _i, C.POINTER(C.c_void_p)]),
    "vs_batch_plan_destroy": (_i, [_p]),
    "vs_batch_set_launch": (_i, [_p, _i, _i]),
    "vs_batch_set_nodes_per_thread": (_i, [_p, _i]),
    "vs_batch_run": (_i, [_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), _i, _p]),
    "vs_post": (_i, [_i, _i, _i, _p, _p, _i, _i, _i, _p, _p, _p]),
    "vs_post_pressure": (_i, [_i, _p, _l, _d, _p, _p]),
    "vs_post_components": (_i, [_i, _i]),
    "vs_adjoint_plan_create": (_i, [C.POINTER(vs_adjoint_cfg), C.POINTER(C.c_void_p)]),
    "vs_adjoint_plan_destroy": (_i, [_p]),
    "vs_adjoint_forward": (_i, [_p, _i, C.POINTER(_d), _p]),
    "vs_adjoint_backward": (_i, [_p, _d, C.POINTER(_d), C.POINTER(_d), C.POINTER(_d), _p]),
    "vs_streaming_vjp": (_i, [_i, _i, _p, _p, _i, _i, _i, _p]),
    "vs_macroscopic_vjp": (_i, [_i, _i, _p, _p, _p, _p, _l, _p]),
    "vs_equilibrium_vjp": (_i, [_i, _i, _p, _p, _p, _p, _p, _l, _p]),
    "vs_collision_vjp": (_i, [_i, _i, _i, _p, _p, _d, _p, _p, _p, _p, _l, _p]),
    "vs_collision_mrt_vjp": (_i, [_i, _i, _p, _p, C.POINTER(_d), _p, _p, _p, _p, _l, _p]),
    "vs_forcing_vjp": (_i, [_i, _i, _i, _p, _p, _d, _p, _p, _p, _p, _p, _l, _p]),
    "vs_forcing_guo_mrt_vjp": (_i, [_i, _i, _p, _p, C.POINTER(_d), _p, _p, _p, _p, _p, _p, _l, _p]),
    "vs_boundary_vjp": (_i, [_i, _i, _i, _i, _i, _p, _p, _p, _p, _p, _p, _i, _i, _i, _d, _d, _d, _d, _p]),
    "vs_ib_pair_dot": (_i, [_i, _p, _p, _i, _l, _p, _i, _i, _p, _p]),
    "vs_ib_stencil_vjp": (_i, [_i, _i, _i, _i, _p, _p, _p, _p, _p, _p, _p, _i, _p]),
    "vs_newmark_vjp": (_i, [_i, _i, _p, _p, _p, _p, _d, _d, _d, _p, _p, _p, _d, _d, _d, _p, _p, _p, _p, _p, _p, _p,
                           _p, _p, _p]),
    "vs_sum_ordered": (_i, [_i, _p, _l, _l, _p, _p, _p]),
    "vs_lattice_status": (_i, [_p, _i, _p]),
    "vs_check_finite": (_i, [_i, _p, _l, _p, _p]),
    "vs_selftest_bounded_wait": (_i, [_i, _p, _p]),
    "vs_fine_to_coarse": (_i, [_i, _p, _i, _i, _p, _i, _i, _i, _p]),
    "vs_coarse_to_fine": (_i, [_i, _p, _i, _i, _p, _i, _i, _i, _p]),
}

_LIB = None


def exported_symbols():
    """Names of the C entry points this binding declares (all must be exported)."""
    return sorted(_SIGS)


def load(path=None):
    """Load the library (no CUDA call is made)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    # VIVSIM_GB300_LIBRARY selects another build of the library, e.g. the bounds-checked one
    path = path or os.environ.get("VIVSIM_GB300_LIBRARY") or _build.lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"vivsim_gb300 CUDA library not found at {path}; build it with "
                           f"`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def lib():
    return load()


def check(status, fn):
    if status != VS_OK:
        L = lib()
        msg = L.vs_last_error().decode()
        raise VivsimError(fn, status, msg or L.vs_status_string(status).decode())


def call(name, *args):
    """Call a C entry point and raise VivsimError on a non-zero status."""
    check(getattr(lib(), name)(*args), name)


# ----------------------------------------------------------------- tensor helpers

def require_cuda(*tensors):
    for t in tensors:
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"expected a torch.Tensor, got {type(t).__name__}")
        if not t.is_cuda:
            raise ValueError("vivsim_gb300 operators run on CUDA tensors only (got a CPU tensor)")


def dtype_code(t):
    if t.dtype == torch.float32:
        return VS_F32
    if t.dtype == torch.float64:
        return VS_F64
    raise TypeError(f"unsupported dtype {t.dtype}: use float32 or float64")


def ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def cont(t):
    return t if t.is_contiguous() else t.contiguous()


def stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)
