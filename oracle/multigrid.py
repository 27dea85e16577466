"""Grid-refinement transfers — NumPy restatement of vivsim/multigrid.py (test infrastructure
only: imported by the tests and the CPU baseline, never by the product path).

Blocks of neighbouring refinement levels differ by a factor 2; the coarser block carries an
overlapping buffer layer.  After streaming, ``fine_to_coarse`` fills the coarse block's
buffer line with the 2 x 2 average of the fine populations that cross into it, and
``coarse_to_fine`` copies each coarse population onto the two fine nodes it covers.
NumPy's assignment broadcasting follows the same rules as ``.at[].set``.
"""

import numpy as np

from .lattice import Q9_DOWN, Q9_LEFT, Q9_RIGHT, Q9_UP

_L, _R, _U, _D = list(Q9_LEFT), list(Q9_RIGHT), list(Q9_UP), list(Q9_DOWN)


def init_grid(width, height, level=0, buffer_x=0, buffer_y=0):
    """multigrid.py:21-55: zero populations, unit density, zero velocity (always float32)."""
    nx = int(width * 2 ** level) + buffer_x
    ny = int(height * 2 ** level) + buffer_y
    return (np.zeros((9, nx, ny), np.float32), np.ones((nx, ny), np.float32),
            np.zeros((2, nx, ny), np.float32))


def fine_to_coarse(f_fine, f_coarse, dir):
    """multigrid.py:58-95.  The sum runs left to right, then the product with 0.25."""
    out = np.array(f_coarse, copy=True)
    q = np.float32(0.25) if f_fine.dtype == np.float32 else 0.25
    if dir == "left":
        out[_L, -1] = q * (f_fine[_L, 0, 0::2] + f_fine[_L, 0, 1::2] + f_fine[_L, 1, 0::2] + f_fine[_L, 1, 1::2])
    if dir == "right":
        out[_R, 0] = q * (f_fine[_R, -1, 0::2] + f_fine[_R, -1, 1::2] + f_fine[_R, -2, 0::2]
                          + f_fine[_R, -2, 1::2])
    if dir == "up":
        out[_U, :, 0] = q * (f_fine[_U, 0::2, -1] + f_fine[_U, 1::2, -1] + f_fine[_U, 0::2, -2]
                             + f_fine[_U, 1::2, -2])
    if dir == "down":
        out[_D, :, -1] = q * (f_fine[_D, 0::2, 0] + f_fine[_D, 1::2, 0] + f_fine[_D, 0::2, 1]
                              + f_fine[_D, 1::2, 1])
    return out


def coarse_to_fine(f_coarse, f_fine, dir):
    """multigrid.py:97-128: each coarse population onto the even and the odd fine node."""
    out = np.array(f_fine, copy=True)
    if dir == "left":
        out[_L, -1, 0::2] = f_coarse[_L, 0]
        out[_L, -1, 1::2] = f_coarse[_L, 0]
    if dir == "right":
        out[_R, 0, 0::2] = f_coarse[_R, -1]
        out[_R, 0, 1::2] = f_coarse[_R, -1]
    if dir == "up":
        out[_U, 0::2, 0] = f_coarse[_U, :, -1]
        out[_U, 1::2, 0] = f_coarse[_U, :, -1]
    if dir == "down":
        out[_D, 0::2, -1] = f_coarse[_D, :, 0]
        out[_D, 1::2, -1] = f_coarse[_D, :, 0]
    return out


def get_omega(nu, level=0):
    """multigrid.py:131-146: the relaxation rate that keeps the viscosity across levels."""
    omega_l0 = 1 / (3 * nu + 0.5)
    return 2 * omega_l0 / (2 ** (level + 1) + (1 - 2 ** level) * omega_l0)


def coord_to_indices(x, y, grid_start_x, grid_start_y, level=0):
    """multigrid.py:149-170"""
    return int((x - grid_start_x) * 2 ** level), int((y - grid_start_y) * 2 ** level)
