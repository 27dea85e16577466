"""Immersed-boundary operators with the signatures of ``vivsim.ib`` / ``vivsim.ib3d``.

Marker arrays are CUDA tensors; stencil weights are (n_markers, n_stencil) in the grid's
float dtype and stencil indices int32 flattened C-order node numbers, exactly as
vivsim/ib/stencil.py:7-51 and vivsim/ib3d/stencil.py:7-59 return them.
"""

import numbers

import torch

from . import _lib as V


class _DeltaKernel:
    """1-D discrete delta kernel; callable on a CUDA tensor of distances."""

    def __init__(self, name, code, width, doc):
        self.__name__ = name
        self.code = code
        self.width = width
        self.__doc__ = doc

    def __call__(self, r):
        V.require_cuda(r)
        r = V.cont(r)
        out = torch.empty_like(r)
        V.call("vs_ib_kernel", self.code, V.dtype_code(r), V.ptr(r), V.ptr(out), int(r.numel()), V.stream())
        return out

    def __repr__(self):
        return f"<delta kernel {self.__name__}>"


kernel_peskin_3pt = _DeltaKernel("kernel_peskin_3pt", V.VS_KERNEL_PESKIN3, 3,
                                 "Peskin 3-point kernel (vivsim/ib/kernels.py:4-22).")
kernel_peskin_4pt = _DeltaKernel("kernel_peskin_4pt", V.VS_KERNEL_PESKIN4, 4,
                                 "Peskin 4-point kernel (vivsim/ib/kernels.py:25-43).")
kernel_cosine_4pt = _DeltaKernel("kernel_cosine_4pt", V.VS_KERNEL_COSINE4, 4,
                                 "Cosine 4-point kernel (vivsim/ib/kernels.py:46-61).")


def _kernel_code(kernel):
    if isinstance(kernel, _DeltaKernel):
        return kernel.code
    raise TypeError("kernel must be one of kernel_peskin_3pt, kernel_peskin_4pt, kernel_cosine_4pt")


def get_ib_stencil(marker_x, marker_y, ny, kernel=kernel_peskin_4pt, stencil_radius=2):
    """Stencil weights and flat indices x*ny + y per marker (vivsim/ib/stencil.py:7-51)."""
    V.require_cuda(marker_x, marker_y)
    mx = V.cont(marker_x)
    my = V.cont(marker_y.to(mx.dtype))
    m = int(mx.numel())
    s = (2 * stencil_radius) ** 2
    W = torch.empty((m, s), dtype=mx.dtype, device=mx.device)
    I = torch.empty((m, s), dtype=torch.int32, device=mx.device)
    V.call("vs_ib_stencil_2d", _kernel_code(kernel), int(stencil_radius), V.dtype_code(mx), V.ptr(mx), V.ptr(my), m,
           int(ny), V.ptr(W), V.ptr(I), V.stream())
    return W, I


def get_ib_stencil_3d(marker_coords, grid_shape, kernel=kernel_peskin_4pt, stencil_radius=2):
    """(vivsim/ib3d/stencil.py:7-59) weights and flat indices x*ny*nz + y*nz + z."""
    if len(grid_shape) != 3:
        raise ValueError(f"grid_shape must be a 3-tuple, got {grid_shape}.")
    V.require_cuda(marker_coords)
    X = V.cont(marker_coords)
    if X.ndim != 2 or X.shape[1] != 3:
        raise ValueError(f"marker_coords must have shape (n_markers, 3), got {tuple(X.shape)}.")
    m = int(X.shape[0])
    s = (2 * stencil_radius) ** 3
    W = torch.empty((m, s), dtype=X.dtype, device=X.device)
    I = torch.empty((m, s), dtype=torch.int32, device=X.device)
    nx, ny, nz = (int(v) for v in grid_shape)
    V.call("vs_ib_stencil_3d", _kernel_code(kernel), int(stencil_radius), V.dtype_code(X), V.ptr(X), m, nx, ny, nz,
           V.ptr(W), V.ptr(I), V.stream())
    return W, I


def _stencil_args(W, I):
    V.require_cuda(W, I)
    if I.dtype != torch.int32:
        I = I.to(torch.int32)
    return V.cont(W), V.cont(I)


def interpolate(grid_values, stencil_weights, stencil_indices):
    """Marker values (n_markers, n_components) (vivsim/ib/stencil.py:54-78)."""
    V.require_cuda(grid_values)
    g = V.cont(grid_values)
    W, I = _stencil_args(stencil_weights.to(g.dtype), stencil_indices)
    c = int(g.shape[0])
    n_grid = int(g[0].numel())
    m, s = (int(x) for x in W.shape)
    out = torch.empty((m, c), dtype=g.dtype, device=g.device)
    V.call("vs_ib_interpolate", V.dtype_code(g), V.ptr(g), c, n_grid, V.ptr(W), V.ptr(I), m, s, V.ptr(out),
           V.stream())
    return out


def _workspace(m, s, device):
    n = int(V.lib().vs_ib_workspace_bytes(m, s))
    return torch.empty(n, dtype=torch.uint8, device=device), n


def spread(marker_values, grid_values, stencil_weights, stencil_indices):
    """grid + scatter of marker values through the stencil (vivsim/ib/stencil.py:81-110)."""
    V.require_cuda(marker_values, grid_values)
    g = V.cont(grid_values)
    mv = V.cont(marker_values.to(g.dtype))
    W, I = _stencil_args(stencil_weights.to(g.dtype), stencil_indices)
    c = int(g.shape[0])
    n_grid = int(g[0].numel())
    m, s = (int(x) for x in W.shape)
    out = torch.empty_like(g)
    ws, nb = _workspace(m, s, g.device)
    V.call("vs_ib_spread", V.dtype_code(g), V.ptr(mv), V.ptr(g), V.ptr(out), c, n_grid, V.ptr(W), V.ptr(I), m, s,
           V.ptr(ws), nb, V.stream())
    return out


def multi_direct_forcing(grid_u, stencil_weights, stencil_indices, marker_u_target, marker_ds, n_iter=5):
    """(grid_force, marker_reaction_force) of multi-direct forcing (vivsim/ib/mdf.py:10-64)."""
    V.require_cuda(grid_u, marker_u_target)
    g = V.cont(grid_u)
    ut = V.cont(marker_u_target.to(g.dtype))
    W, I = _stencil_args(stencil_weights.to(g.dtype), stencil_indices)
    c = int(g.shape[0])
    n_grid = int(g[0].numel())
    m, s = (int(x) for x in W.shape)
    ds_t, ds_s = None, 0.0
    if isinstance(marker_ds, numbers.Number):
        ds_s = float(marker_ds)
    elif isinstance(marker_ds, torch.Tensor) and marker_ds.numel() == 1:
        ds_s = float(marker_ds.item())
    else:
        V.require_cuda(marker_ds)
        ds_t = V.cont(marker_ds.reshape(-1).to(g.dtype))
        if ds_t.numel() != m:
            raise ValueError("marker_ds must be a scalar or have one value per marker")
    gf = torch.empty_like(g)
    mf = torch.empty((m, c), dtype=g.dtype, device=g.device)
    ws, nb = _workspace(m, s, g.device)
    V.call("vs_ib_mdf", V.dtype_code(g), V.ptr(g), c, n_grid, V.ptr(W), V.ptr(I), m, s, V.ptr(ut), V.ptr(ds_t),
           ds_s, int(n_iter), V.ptr(gf), V.ptr(mf), V.ptr(ws), nb, V.stream())
    return gf, mf


# ---------------------------------------------------------------- geometry (setup time)

def get_area(marker_coords):
    """Polygon area (vivsim/ib/geometry.py:6-22)."""
    x, y = marker_coords[:, 0], marker_coords[:, 1]
    return 0.5 * torch.abs(torch.sum(x * torch.roll(y, 1) - y * torch.roll(x, 1)))


def get_ds(marker_coords, closed=True):
    """Segment length per marker of a curve (vivsim/ib/geometry.py:25-43)."""
    X = marker_coords
    if closed:
        seg = torch.linalg.norm(X - torch.roll(X, -1, dims=0), dim=1)
        return (seg + torch.roll(seg, 1)) / 2.0
    seg = torch.linalg.norm(X[1:] - X[:-1], dim=1)
    z = seg.new_zeros(1)
    return torch.cat([z, seg / 2]) + torch.cat([seg / 2, z])


def get_triangle_areas(vertex_coords, faces):
    """(vivsim/ib3d/geometry.py:6-19)."""
    t = vertex_coords[faces.long()]
    return 0.5 * torch.linalg.norm(torch.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0], dim=1), dim=1)


def get_surface_area(vertex_coords, faces):
    """(vivsim/ib3d/geometry.py:22-24)."""
    return torch.sum(get_triangle_areas(vertex_coords, faces))


def get_volume(vertex_coords, faces):
    """(vivsim/ib3d/geometry.py:27-47)."""
    t = vertex_coords[faces.long()]
    return torch.abs(torch.sum(torch.einsum("ij,ij->i", t[:, 0], torch.cross(t[:, 1], t[:, 2], dim=1)) / 6.0))


def get_vertex_ds(vertex_coords, faces):
    """Vertex area weights: each triangle's area split equally (vivsim/ib3d/geometry.py:50-67)."""
    areas = get_triangle_areas(vertex_coords, faces)
    out = torch.zeros(vertex_coords.shape[0], dtype=vertex_coords.dtype, device=vertex_coords.device)
    return out.index_add(0, faces.reshape(-1).long(), torch.repeat_interleave(areas / 3.0, 3))
