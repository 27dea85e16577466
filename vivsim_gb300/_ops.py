"""Shared implementation of the per-operator LBM shims for D2Q9 (q=9) and D3Q19 (q=19).

``vivsim_gb300.lbm`` and ``vivsim_gb300.lbm3d`` expose these under the reference's
function names and signatures (vivsim/lbm/__init__.py:1-42, vivsim/lbm3d/__init__.py:1-44).
Every array function takes and returns CUDA tensors and runs one kernel of the C ABI.
"""

import ctypes as C
import numbers

import numpy as np
import torch

from . import _lib as V

# MRT moment bases.  These tables fix the moment numbering the relaxation rates refer to,
# so they are the reference's: vivsim/lbm/collision/mrt.py:9-23 (D2Q9, Gram-Schmidt) and
# vivsim/lbm3d/collision/mrt.py:7-29 (D3Q19).
_M9 = np.array([
    [1, 1, 1, 1, 1, 1, 1, 1, 1],
    [-4, -1, -1, -1, -1, 2, 2, 2, 2],
    [4, -2, -2, -2, -2, 1, 1, 1, 1],
    [0, 1, 0, -1, 0, 1, -1, -1, 1],
    [0, -2, 0, 2, 0, 1, -1, -1, 1],
    [0, 0, 1, 0, -1, 1, 1, -1, -1],
    [0, 0, -2, 0, 2, 1, 1, -1, -1],
    [0, 1, -1, 1, -1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 1, -1, 1, -1],
])
_M9_INV = np.linalg.inv(_M9)


def _m19():
    """D3Q19 moment basis as listed by the reference (lbm3d/collision/mrt.py:7-29)."""
    return np.array([
        [1] * 19,
        [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
        [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1],
        [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1],
        [0, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2],
        [0, 2, 2, -1, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2],
        [0, 0, 0, 1, 1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1],
        [0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1],
        [0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1],
    ], dtype=np.float32)


_M19 = _m19()
_M19_INV = np.linalg.inv(_M19)  # float32 inverse, as the reference computes it


def _np_dtype(dtype):
    if dtype in (torch.float64, np.float64, "float64"):
        return np.float64
    return np.float32


def mrt_relaxation(q, omega):
    """Diagonal of S: lbm/collision/mrt.py:29-44 (q=9), lbm3d/collision/mrt.py:34-77 (q=19)."""
    if q == 9:
        return [0, 1.4, 1.4, 0, 1.2, 0, 1.2, omega, omega]
    return [0.0, 0.0, 0.0, 0.0, 1.1] + [omega] * 5 + [1.2] * 6 + [1.4] * 3


def mrt_collision_operator(q, omega, dtype=torch.float32):
    """M^-1 S M, formed in ``dtype`` the way JAX forms it (host; returns a CPU tensor)."""
    dt = _np_dtype(dtype)
    M, Mi = (_M9, _M9_INV) if q == 9 else (_M19, _M19_INV)
    S = np.diag(np.array(mrt_relaxation(q, omega), dtype=dt))
    return torch.from_numpy((Mi.astype(dt) @ S) @ M.astype(dt))


def mrt_forcing_operator(q, omega, dtype=torch.float32):
    """M^-1 (I - S/2) M (lbm/forcing/guo.py:62-80, lbm3d/forcing/guo.py:58-68)."""
    dt = _np_dtype(dtype)
    M, Mi = (_M9, _M9_INV) if q == 9 else (_M19, _M19_INV)
    S = np.diag(np.array(mrt_relaxation(q, omega), dtype=dt))
    return torch.from_numpy((Mi.astype(dt) @ (np.eye(q, dtype=dt) - 0.5 * S)) @ M.astype(dt))


def _host_matrix(op, q):
    a = op.detach().cpu().double().numpy() if isinstance(op, torch.Tensor) else np.asarray(op, dtype=np.float64)
    if a.shape != (q, q):
        raise ValueError(f"operator must be {q}x{q}, got {a.shape}")
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def _check_f(f, q):
    V.require_cuda(f)
    if f.shape[0] != q:
        raise ValueError(f"expected populations of shape ({q}, ...), got {tuple(f.shape)}")
    return V.cont(f)


def _nodes(t):
    return int(t[0].numel())


class Lattice:
    """Per-operator entry points for one velocity set."""

    def __init__(self, q):
        self.q = q
        self.d = 2 if q == 9 else 3
        self.locs = ("left", "right", "top", "bottom") if q == 9 else \
            ("left", "right", "bottom", "top", "back", "front")

    # -------------------------------------------------------------- basic ops
    def streaming(self, f):
        f = _check_f(f, self.q)
        shp = f.shape[1:]
        if len(shp) != self.d:
            raise ValueError(f"streaming needs f of shape ({self.q}, {'NX, NY' if self.d == 2 else 'NX, NY, NZ'})")
        out = torch.empty_like(f)
        nz = 1 if self.d == 2 else shp[2]
        V.call("vs_streaming", self.q, V.dtype_code(f), V.ptr(f), V.ptr(out), shp[0], shp[1], nz, V.stream())
        return out

    def get_macroscopic(self, f):
        f = _check_f(f, self.q)
        rho = torch.empty(f.shape[1:], dtype=f.dtype, device=f.device)
        u = torch.empty((self.d,) + tuple(f.shape[1:]), dtype=f.dtype, device=f.device)
        V.call("vs_get_macroscopic", self.q, V.dtype_code(f), V.ptr(f), V.ptr(rho), V.ptr(u), _nodes(f), V.stream())
        return rho, u

    def get_equilibrium(self, rho, u):
        V.require_cuda(rho, u)
        rho, u = V.cont(rho), V.cont(u.to(rho.dtype))
        if u.shape != (self.d,) + tuple(rho.shape):
            raise ValueError(f"u must have shape ({self.d}, *rho.shape)")
        feq = torch.empty((self.q,) + tuple(rho.shape), dtype=rho.dtype, device=rho.device)
        V.call("vs_get_equilibrium", self.q, V.dtype_code(rho), V.ptr(rho), V.ptr(u), V.ptr(feq), int(rho.numel()),
               V.stream())
        return feq

    def _collide(self, kind, f, feq, omega):
        f = _check_f(f, self.q)
        feq = V.cont(feq.to(f.dtype))
        out = torch.empty_like(f)
        V.call("vs_collision", self.q, V.dtype_code(f), kind, V.ptr(f), V.ptr(feq), float(omega), V.ptr(out),
               _nodes(f), V.stream())
        return out

    def collision_bgk(self, f, feq, omega):
        return self._collide(V.VS_COLLIDE_BGK, f, feq, omega)

    def collision_kbc(self, f, feq, omega):
        return self._collide(V.VS_COLLIDE_KBC, f, feq, omega)

    def collision_reg(self, f, feq, omega):
        return self._collide(V.VS_COLLIDE_REG, f, feq, omega)

    def get_mrt_collision_operator(self, omega, dtype=torch.float32):
        return mrt_collision_operator(self.q, omega, dtype)

    def collision_mrt(self, f, feq, mrt_collision_matrix):
        f = _check_f(f, self.q)
        feq = V.cont(feq.to(f.dtype))
        keep, mp = _host_matrix(mrt_collision_matrix, self.q)
        out = torch.empty_like(f)
        V.call("vs_collision_mrt", self.q, V.dtype_code(f), V.ptr(f), V.ptr(feq), mp, V.ptr(out), _nodes(f),
               V.stream())
        del keep
        return out

    @staticmethod
    def get_omega(nu):
        return 1 / (3 * nu + 0.5)

    def get_velocity_correction(self, g, rho=1):
        V.require_cuda(g)
        g = V.cont(g)
        if not isinstance(rho, torch.Tensor):
            rho = torch.full(g.shape[1:], float(rho), dtype=g.dtype, device=g.device)
        rho = V.cont(rho.to(g.dtype))
        out = torch.empty_like(g)
        V.call("vs_velocity_correction", self.q, V.dtype_code(g), V.ptr(g), V.ptr(rho), V.ptr(out), int(rho.numel()),
               V.stream())
        return out

    # ---------------------------------------------------------------- forcing
    def get_guo_forcing_term(self, g, u):
        V.require_cuda(g, u)
        g, u = V.cont(g), V.cont(u.to(g.dtype))
        out = torch.empty((self.q,) + tuple(g.shape[1:]), dtype=g.dtype, device=g.device)
        V.call("vs_guo_forcing_term", self.q, V.dtype_code(g), V.ptr(g), V.ptr(u), V.ptr(out), _nodes(g),
               V.stream())
        return out

    def _force(self, kind, f, g, u, omega):
        f = _check_f(f, self.q)
        g, u = V.cont(g.to(f.dtype)), V.cont(u.to(f.dtype))
        out = torch.empty_like(f)
        V.call("vs_forcing", self.q, V.dtype_code(f), kind, V.ptr(f), V.ptr(g), V.ptr(u), float(omega), V.ptr(out),
               _nodes(f), V.stream())
        return out

    def forcing_edm(self, f, g, u):
        return self._force(V.VS_FORCE_EDM, f, g, u, 0.0)

    def forcing_guo_bgk(self, f, g, u, omega):
        return self._force(V.VS_FORCE_GUO_BGK, f, g, u, omega)

    def get_mrt_forcing_operator(self, omega, dtype=torch.float32):
        return mrt_forcing_operator(self.q, omega, dtype)

    def forcing_guo_mrt(self, f, g, u, mrt_forcing_operator):
        f = _check_f(f, self.q)
        g, u = V.cont(g.to(f.dtype)), V.cont(u.to(f.dtype))
        keep, mp = _host_matrix(mrt_forcing_operator, self.q)
        out = torch.empty_like(f)
        V.call("vs_forcing_guo_mrt", self.q, V.dtype_code(f), V.ptr(f), V.ptr(g), V.ptr(u), mp, V.ptr(out),
               _nodes(f), V.stream())
        del keep
        return out

    # ------------------------------------------------------------- boundaries
    def _loc(self, loc):
        if loc not in self.locs:
            raise ValueError(f"loc must be one of: {', '.join(repr(x) for x in self.locs)}")
        return V.LOCS[loc]

    def _dims(self, f):
        s = tuple(f.shape[1:])
        if len(s) != self.d:
            raise ValueError("boundary functions need f over the whole grid")
        return (s[0], s[1], 1) if self.d == 2 else s

    def _wall(self, f, values):
        """vs_wall from scalars / tensors; returns (struct, tensors kept alive)."""
        w = V.vs_wall()
        keep = []
        for name, val in values.items():
            if isinstance(val, torch.Tensor) and val.numel() > 1:
                t = V.cont(val.to(device=f.device, dtype=f.dtype))
                keep.append(t)
                setattr(w, name + "_arr", t.data_ptr())
            else:
                v = float(val.item()) if isinstance(val, torch.Tensor) else float(val)
                setattr(w, name, v)
        return w, keep

    def _boundary(self, kind, mode, f, loc, values, f_pre=None):
        f = _check_f(f, self.q)
        code = self._loc(loc)
        nx, ny, nz = self._dims(f)
        w, keep = self._wall(f, values)
        out = torch.empty_like(f)
        pre = V.cont(f_pre.to(f.dtype)) if f_pre is not None else None
        V.call("vs_boundary", self.q, V.dtype_code(f), kind, mode, code, V.ptr(f), V.ptr(out), V.ptr(pre), nx, ny,
               nz, C.byref(w), V.stream())
        del keep
        return out

    def make_boundary(self, kind, mode):
        d = self.d

        if mode == V.VS_WALL_GIVEN:
            if d == 2:
                def fn(f, loc, rho_wall=1, ux_wall=0, uy_wall=0):
                    return self._boundary(kind, mode, f, loc, dict(rho=rho_wall, ux=ux_wall, uy=uy_wall))
            else:
                def fn(f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0):
                    return self._boundary(kind, mode, f, loc, dict(rho=rho_wall, ux=ux_wall, uy=uy_wall,
                                                                   uz=uz_wall))
        elif mode == V.VS_WALL_VELOCITY:
            if d == 2:
                def fn(f, loc, ux_wall=0, uy_wall=0):
                    return self._boundary(kind, mode, f, loc, dict(rho=1.0, ux=ux_wall, uy=uy_wall))
            else:
                def fn(f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
                    return self._boundary(kind, mode, f, loc, dict(rho=1.0, ux=ux_wall, uy=uy_wall, uz=uz_wall))
        elif mode == V.VS_WALL_PRESSURE:
            def fn(f, loc, rho_wall=1):
                return self._boundary(kind, mode, f, loc, dict(rho=rho_wall))
        else:
            if d == 2:
                def fn(f, loc, rho_wall=1, ux_wall=0, uy_wall=0, gx_wall=0, gy_wall=0):
                    _scalars_only(rho_wall, ux_wall, uy_wall, gx_wall, gy_wall)
                    return self._boundary(kind, mode, f, loc, dict(rho=rho_wall, ux=ux_wall, uy=uy_wall,
                                                                   gx=gx_wall, gy=gy_wall))
            else:
                def fn(f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0, gx_wall=0, gy_wall=0, gz_wall=0):
                    _scalars_only(rho_wall, ux_wall, uy_wall, uz_wall, gx_wall, gy_wall, gz_wall)
                    return self._boundary(kind, mode, f, loc, dict(rho=rho_wall, ux=ux_wall, uy=uy_wall, uz=uz_wall,
                                                                   gx=gx_wall, gy=gy_wall, gz=gz_wall))
        return fn

    def make_bounce_back(self, kind):
        if self.d == 2:
            def fn(f_before_stream, f, loc, ux_wall=0, uy_wall=0):
                return self._boundary(kind, V.VS_WALL_GIVEN, f, loc, dict(ux=ux_wall, uy=uy_wall), f_before_stream)
        else:
            def fn(f_before_stream, f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
                return self._boundary(kind, V.VS_WALL_GIVEN, f, loc, dict(ux=ux_wall, uy=uy_wall, uz=uz_wall),
                                      f_before_stream)
        return fn

    def obstacle_bounce_back(self, f, mask):
        f = _check_f(f, self.q)
        V.require_cuda(mask)
        m = V.cont(mask.to(torch.uint8))
        if tuple(m.shape) != tuple(f.shape[1:]):
            raise ValueError("mask must have the grid's shape")
        out = torch.empty_like(f)
        V.call("vs_obstacle_bounce_back", self.q, V.dtype_code(f), V.ptr(f), V.ptr(out), V.ptr(m), _nodes(f),
               V.stream())
        return out

    def boundary_characteristic(self, rho, u, loc="right"):
        V.require_cuda(rho, u)
        code = self._loc(loc)
        rho, u = V.cont(rho), V.cont(u.to(rho.dtype))
        s = tuple(rho.shape)
        nx, ny, nz = (s[0], s[1], 1) if self.d == 2 else s
        axis = {0: 0, 1: 0, 2: 1, 3: 1, 4: 2, 5: 2}[code]
        face = tuple(n for a, n in enumerate(s) if a != axis)
        rho_next = torch.empty(face, dtype=rho.dtype, device=rho.device)
        u_next = torch.empty((self.d,) + face, dtype=rho.dtype, device=rho.device)
        V.call("vs_boundary_characteristic", self.q, V.dtype_code(rho), code, V.ptr(rho), V.ptr(u), nx, ny, nz,
               V.ptr(rho_next), V.ptr(u_next), V.stream())
        return rho_next, u_next


def _scalars_only(*vals):
    for v in vals:
        if isinstance(v, torch.Tensor) and v.numel() > 1:
            raise NotImplementedError("force-corrected boundaries take scalar wall data in this build")
        if not isinstance(v, (numbers.Number, torch.Tensor)):
            raise TypeError("wall data must be numbers or tensors")


def export(module_globals, lat):
    """Bind the reference's public names of one lattice module to ``lat``."""
    g = module_globals
    for name in ("streaming", "get_macroscopic", "get_equilibrium", "collision_bgk", "collision_kbc",
                 "collision_reg", "collision_mrt", "get_mrt_collision_operator", "get_omega",
                 "get_velocity_correction", "get_guo_forcing_term", "forcing_edm", "forcing_guo_bgk",
                 "get_mrt_forcing_operator", "forcing_guo_mrt", "obstacle_bounce_back", "boundary_characteristic"):
        g[name] = getattr(lat, name)
    for scheme, kind in (("nee", V.VS_BC_NEE), ("nebb", V.VS_BC_NEBB), ("equilibrium", V.VS_BC_EQ)):
        g[f"boundary_{scheme}"] = lat.make_boundary(kind, V.VS_WALL_GIVEN)
        g[f"boundary_velocity_{scheme}"] = lat.make_boundary(kind, V.VS_WALL_VELOCITY)
        g[f"boundary_pressure_{scheme}"] = lat.make_boundary(kind, V.VS_WALL_PRESSURE)
        g[f"boundary_force_corrected_{scheme}"] = lat.make_boundary(kind, V.VS_WALL_FORCE_CORRECTED)
    g["boundary_bounce_back"] = lat.make_bounce_back(V.VS_BC_BB)
    g["boundary_specular_reflection"] = lat.make_bounce_back(V.VS_BC_SPECULAR)
