"""Grid refinement with the reference's names (vivsim/multigrid.py), transfers on the GPU.

``fine_to_coarse`` and ``coarse_to_fine`` take CUDA population tensors (9, NX, NY) and run
one kernel each (vs_fine_to_coarse / vs_coarse_to_fine); like the reference they return
the updated destination and leave their arguments untouched.  ``init_grid``,
``get_omega`` and ``coord_to_indices`` are host arithmetic, as in the reference.
``vivsim_gb300.solver.Refined`` steps whole block layouts with these transfers.
"""

import torch

from . import _lib as V


def init_grid(width, height, level=0, buffer_x=0, buffer_y=0, device="cuda"):
    """multigrid.py:21-55: f = 0, rho = 1, u = 0 on a block of the given level (float32)."""
    nx = int(width * 2 ** level) + buffer_x
    ny = int(height * 2 ** level) + buffer_y
    return (torch.zeros((9, nx, ny), dtype=torch.float32, device=device),
            torch.ones((nx, ny), dtype=torch.float32, device=device),
            torch.zeros((2, nx, ny), dtype=torch.float32, device=device))


def _check(f, name):
    V.require_cuda(f)
    if f.dim() != 3 or f.shape[0] != 9:
        raise ValueError(f"{name} must have shape (9, NX, NY)")
    return V.cont(f)


def transfer_(kind, src, dst, dir):
    """In-place form: rewrite the interface line of dst (no copy); kind is 'fine_to_coarse'
    (src fine, dst coarse) or 'coarse_to_fine'."""
    code = V.REFINE_DIRS[dir]
    if dst.dtype != src.dtype:
        raise ValueError("both blocks must have the same dtype")
    fn = "vs_fine_to_coarse" if kind == "fine_to_coarse" else "vs_coarse_to_fine"
    V.call(fn, V.dtype_code(src), V.ptr(src), int(src.shape[1]), int(src.shape[2]), V.ptr(dst),
           int(dst.shape[1]), int(dst.shape[2]), code, V.stream())
    return dst


def _shape_errors(fn, *args):
    """Blocks whose interface extents do not match raise ValueError, as the reference's
    array assignment does."""
    try:
        return fn(*args)
    except V.VivsimError as e:
        if e.status == V.VS_ERR_INVALID_ARG:
            raise ValueError(str(e)) from e
        raise


def fine_to_coarse(f_fine, f_coarse, dir):
    """multigrid.py:58-95: the coarse buffer line gets the 2 x 2 average of the fine
    populations moving in ``dir``.  An unknown dir returns f_coarse unchanged."""
    f_fine, f_coarse = _check(f_fine, "f_fine"), _check(f_coarse, "f_coarse")
    if dir not in V.REFINE_DIRS:
        return f_coarse
    return _shape_errors(transfer_, "fine_to_coarse", f_fine, f_coarse.clone(), dir)


def coarse_to_fine(f_coarse, f_fine, dir):
    """multigrid.py:97-128: each coarse population of the interface onto the two fine nodes
    it covers.  An unknown dir returns f_fine unchanged."""
    f_coarse, f_fine = _check(f_coarse, "f_coarse"), _check(f_fine, "f_fine")
    if dir not in V.REFINE_DIRS:
        return f_fine
    return _shape_errors(transfer_, "coarse_to_fine", f_coarse, f_fine.clone(), dir)


def get_omega(nu, level=0):
    """multigrid.py:131-146"""
    omega_l0 = 1 / (3 * nu + 0.5)
    return 2 * omega_l0 / (2 ** (level + 1) + (1 - 2 ** level) * omega_l0)


def coord_to_indices(x, y, grid_start_x, grid_start_y, level=0):
    """multigrid.py:149-170"""
    return int((x - grid_start_x) * 2 ** level), int((y - grid_start_y) * 2 ** level)


__all__ = ["init_grid", "fine_to_coarse", "coarse_to_fine", "get_omega", "coord_to_indices"]
