"""Immersed-boundary operators — NumPy restatement of vivsim/ib and vivsim/ib3d.

Test infrastructure only.  Stencils are tensor products of a 1-D discrete delta
kernel over offsets ``-r+1 .. r`` around ``floor(X)``; indices are flattened C-order
node numbers of the grid the stencil is built for.
"""

import numpy as np


def _seq(terms):
    out = terms[0]
    for t in terms[1:]:
        out = out + t
    return out


def kernel_peskin_3pt(r):
    """(vivsim/ib/kernels.py:4-22)."""
    a = np.abs(r)
    with np.errstate(invalid="ignore"):
        inner = (1 + np.sqrt(1 - 3 * (a * a))) / 3
        outer = ((5 - 3 * a) - np.sqrt((-2 + 6 * a) - 3 * (a * a))) / 6
    return np.where(a > 1.5, 0, np.where(a < 0.5, inner, outer)).astype(a.dtype)


def kernel_peskin_4pt(r):
    """(vivsim/ib/kernels.py:25-43)."""
    a = np.abs(r)
    with np.errstate(invalid="ignore"):
        inner = ((3 - 2 * a) + np.sqrt((1 + 4 * a) - 4 * (a * a))) * 0.125
        outer = ((5 - 2 * a) - np.sqrt((-7 + 12 * a) - 4 * (a * a))) * 0.125
    return np.where(a > 2, 0, np.where(a < 1, inner, outer)).astype(a.dtype)


def kernel_cosine_4pt(r):
    """(vivsim/ib/kernels.py:46-61)."""
    a = np.abs(r)
    return np.where(a > 2, 0, (1 + np.cos((np.pi * a) * 0.5)) * 0.25).astype(a.dtype)


KERNELS = {"peskin3": kernel_peskin_3pt, "peskin4": kernel_peskin_4pt, "cosine4": kernel_cosine_4pt}


def _offsets(radius):
    return np.arange(-radius + 1, radius + 1, dtype=np.int32)


def get_ib_stencil(marker_x, marker_y, ny, kernel=kernel_peskin_4pt, stencil_radius=2):
    """(M, (2r)^2) weights and flat indices x*ny + y (vivsim/ib/stencil.py:7-51)."""
    mx = np.asarray(marker_x)
    my = np.asarray(marker_y)
    off = _offsets(stencil_radius)
    ox, oy = np.meshgrid(off, off, indexing="ij")
    ox = ox.reshape(1, -1)
    oy = oy.reshape(1, -1)
    sx = np.floor(mx).astype(np.int32)[:, None] + ox
    sy = np.floor(my).astype(np.int32)[:, None] + oy
    dt = mx.dtype
    W = kernel(sx.astype(dt) - mx[:, None]) * kernel(sy.astype(dt) - my[:, None])
    return W, (sx * ny + sy).astype(np.int32)


def get_ib_stencil_3d(marker_coords, grid_shape, kernel=kernel_peskin_4pt, stencil_radius=2):
    """(M, (2r)^3) weights and flat indices x*ny*nz + y*nz + z (vivsim/ib3d/stencil.py:7-59)."""
    if len(grid_shape) != 3:
        raise ValueError(f"grid_shape must be a 3-tuple, got {grid_shape}.")
    X = np.asarray(marker_coords)
    if X.ndim != 2 or X.shape[1] != 3:
        raise ValueError(f"marker_coords must have shape (n_markers, 3), got {X.shape}.")
    nx, ny, nz = grid_shape
    off = _offsets(stencil_radius)
    ox, oy, oz = (a.reshape(1, -1) for a in np.meshgrid(off, off, off, indexing="ij"))
    ref = np.floor(X).astype(np.int32)
    sx = ref[:, 0:1] + ox
    sy = ref[:, 1:2] + oy
    sz = ref[:, 2:3] + oz
    dt = X.dtype
    W = (kernel(sx.astype(dt) - X[:, 0:1]) * kernel(sy.astype(dt) - X[:, 1:2])) * kernel(sz.astype(dt) - X[:, 2:3])
    return W, (sx * (ny * nz) + sy * nz + sz).astype(np.int32)


def interpolate(grid_values, stencil_weights, stencil_indices):
    """U_mc = sum_s W_ms grid_c[I_ms], s in order (vivsim/ib/stencil.py:54-78)."""
    flat = grid_values.reshape(grid_values.shape[0], -1)
    vals = flat[:, stencil_indices]  # (C, M, S)
    S = stencil_weights.shape[1]
    out = _seq([stencil_weights[None, :, s] * vals[:, :, s] for s in range(S)])  # (C, M)
    return out.T.copy()


def spread(marker_values, grid_values, stencil_weights, stencil_indices):
    """grid_c[I_ms] += F_mc W_ms in (m, s) order (vivsim/ib/stencil.py:81-110)."""
    shp = grid_values.shape
    flat = grid_values.reshape(shp[0], -1).copy()
    contrib = marker_values.T[:, :, None] * stencil_weights[None, :, :]  # (C, M, S)
    np.add.at(flat, (slice(None), stencil_indices), contrib)
    return flat.reshape(shp)


def multi_direct_forcing(grid_u, stencil_weights, stencil_indices, marker_u_target, marker_ds, n_iter=5):
    """Multi-direct forcing, returns (grid_force, marker_reaction_force) (vivsim/ib/mdf.py:10-64)."""
    ds = np.asarray(marker_ds, dtype=grid_u.dtype).reshape(-1, 1)
    zero = np.zeros_like(grid_u)
    total = np.zeros_like(marker_u_target)
    mu = interpolate(grid_u, stencil_weights, stencil_indices)
    for _ in range(n_iter):
        step = (marker_u_target - mu) * (ds * 2.0)
        total = total + step
        gstep = spread(step, zero, stencil_weights, stencil_indices)
        mu = mu + interpolate(gstep * 0.5, stencil_weights, stencil_indices)
    return spread(total, zero, stencil_weights, stencil_indices), -total


# ----------------------------------------------------------------- geometry

def get_ds(marker_coords, closed=True):
    """Marker segment lengths on a curve (vivsim/ib/geometry.py:25-43)."""
    X = np.asarray(marker_coords)
    if closed:
        seg = np.linalg.norm(X - np.roll(X, -1, axis=0), axis=1)
        return (seg + np.roll(seg, 1)) / 2.0
    seg = np.linalg.norm(X[1:] - X[:-1], axis=1)
    return np.pad(seg / 2, (1, 0)) + np.pad(seg / 2, (0, 1))
