"""Rigid-body dynamics with the signatures of ``vivsim.dyn`` (vivsim/dyn.py:5-154).

Tensor arguments run on the device through the C ABI.  The reference's scalar Newmark
path on plain Python numbers is host arithmetic in the reference as well (no array is
involved), so plain numbers are evaluated the same way here.
"""

import numbers

import torch

from . import _lib as V


def _is_num(x):
    return isinstance(x, numbers.Number)


def newmark(a, v, d, h, m, k, c, dt=1, gamma=0.5, beta=0.25):
    """Newmark-beta step; scalar or matrix mass (vivsim/dyn.py:5-51)."""
    if all(_is_num(x) for x in (a, v, d, h, m, k, c)):
        c1, c2 = gamma * dt, beta * dt ** 2
        v1 = v + dt * (1 - gamma) * a
        v2 = d + dt * v + dt ** 2 * (0.5 - beta) * a
        a_next = (h - c * v1 - k * v2) / (m + c1 * c + c2 * k)
        return a_next, c1 * a_next + v1, c2 * a_next + v2
    ref = next(x for x in (a, v, d, h) if isinstance(x, torch.Tensor))
    V.require_cuda(ref)
    dt_ = ref.dtype

    def dev(x):
        if isinstance(x, torch.Tensor):
            return V.cont(x.to(device=ref.device, dtype=dt_).reshape(-1))
        return torch.full((ref.numel(),), float(x), dtype=dt_, device=ref.device)

    A, Vv, D, H = (dev(x) for x in (a, v, d, h))
    ndof = int(A.numel())
    an, vn, dn = torch.empty_like(A), torch.empty_like(A), torch.empty_like(A)
    matrix = isinstance(m, torch.Tensor) and m.ndim > 0
    if matrix:
        Mm, Km, Cm = (V.cont(x.to(device=ref.device, dtype=dt_)) for x in (m, k, c))
        V.call("vs_newmark", V.dtype_code(A), ndof, V.ptr(A), V.ptr(Vv), V.ptr(D), V.ptr(H), 0.0, 0.0, 0.0,
               V.ptr(Mm), V.ptr(Km), V.ptr(Cm), float(dt), float(gamma), float(beta), V.ptr(an), V.ptr(vn),
               V.ptr(dn), V.stream())
    else:
        V.call("vs_newmark", V.dtype_code(A), ndof, V.ptr(A), V.ptr(Vv), V.ptr(D), V.ptr(H), float(m), float(k),
               float(c), None, None, None, float(dt), float(gamma), float(beta), V.ptr(an), V.ptr(vn), V.ptr(dn),
               V.stream())
    shape = ref.shape
    return an.reshape(shape), vn.reshape(shape), dn.reshape(shape)


def newmark_2dof(a, v, d, h, m, k, c, dt=1, gamma=0.5, beta=0.25):
    """(vivsim/dyn.py:55-57)."""
    return newmark(a, v, d, h, m, k, c, dt, gamma, beta)


def newmark_3dof(a, v, d, h, m, k, c, dt=1, gamma=0.5, beta=0.25):
    """(vivsim/dyn.py:60-62)."""
    return newmark(a, v, d, h, m, k, c, dt, gamma, beta)


def get_markers_coords_2dof(x_markers_init, y_markers_init, d):
    """(vivsim/dyn.py:68-81)."""
    V.require_cuda(x_markers_init, y_markers_init, d)
    x0 = V.cont(x_markers_init)
    y0 = V.cont(y_markers_init.to(x0.dtype))
    dd = V.cont(d.to(x0.dtype))
    x, y = torch.empty_like(x0), torch.empty_like(x0)
    V.call("vs_markers_coords_2dof", V.dtype_code(x0), V.ptr(x0), V.ptr(y0), int(x0.numel()), V.ptr(dd), V.ptr(x),
           V.ptr(y), V.stream())
    return x, y


def get_markers_coords_3dof(x_markers_init, y_markers_init, x_center_init, y_center_init, d):
    """(vivsim/dyn.py:84-99)."""
    V.require_cuda(x_markers_init, y_markers_init, d)
    x0 = V.cont(x_markers_init)
    y0 = V.cont(y_markers_init.to(x0.dtype))
    dd = V.cont(d.to(x0.dtype))
    x, y = torch.empty_like(x0), torch.empty_like(x0)
    V.call("vs_markers_coords_3dof", V.dtype_code(x0), V.ptr(x0), V.ptr(y0), int(x0.numel()), float(x_center_init),
           float(y_center_init), V.ptr(dd), V.ptr(x), V.ptr(y), V.stream())
    return x, y


def get_markers_velocity_3dof(x_markers, y_markers, x_center_init, y_center_init, d, v):
    """(vivsim/dyn.py:102-120)."""
    V.require_cuda(x_markers, y_markers, d, v)
    x = V.cont(x_markers)
    y = V.cont(y_markers.to(x.dtype))
    dd, vv = V.cont(d.to(x.dtype)), V.cont(v.to(x.dtype))
    out = torch.empty((x.numel(), 2), dtype=x.dtype, device=x.device)
    V.call("vs_markers_velocity_3dof", V.dtype_code(x), V.ptr(x), V.ptr(y), int(x.numel()), float(x_center_init),
           float(y_center_init), V.ptr(dd), V.ptr(vv), V.ptr(out), V.stream())
    return out


def get_force_to_obj(h_markers):
    """Total force, summed in marker order (vivsim/dyn.py:126-136)."""
    V.require_cuda(h_markers)
    h = V.cont(h_markers)
    m, c = int(h.shape[0]), int(h.shape[1])
    out = torch.empty((c,), dtype=h.dtype, device=h.device)
    V.call("vs_force_to_obj", V.dtype_code(h), V.ptr(h), m, c, V.ptr(out), V.stream())
    return out


def get_torque_to_obj(x_markers, y_markers, x_center_init, y_center_init, d, h_markers):
    """(vivsim/dyn.py:139-154)."""
    V.require_cuda(x_markers, y_markers, d, h_markers)
    x = V.cont(x_markers)
    y = V.cont(y_markers.to(x.dtype))
    dd, h = V.cont(d.to(x.dtype)), V.cont(h_markers.to(x.dtype))
    out = torch.empty((), dtype=x.dtype, device=x.device)
    V.call("vs_torque_to_obj", V.dtype_code(x), V.ptr(x), V.ptr(y), int(x.numel()), float(x_center_init),
           float(y_center_init), V.ptr(dd), V.ptr(h), V.ptr(out), V.stream())
    return out
