"""Differentiable versions of the per-operator functions (reverse mode, PyTorch autograd).

The reference differentiates a user-composed ``update_step`` with ``jax.grad``.  The
functions here keep the reference's names and arguments and run the same CUDA kernels
as ``vivsim_gb300.lbm`` / ``lbm3d`` / ``ib`` / ``ib3d`` / ``dyn`` forward; their backward
passes call the hand-written vector-Jacobian-product kernels of ``csrc/vs_grad.cu``
(``vs_*_vjp``), so an update step composed from them differentiates end to end with
``torch.autograd``::

    from vivsim_gb300 import autodiff as ad
    rho, u = ad.get_macroscopic(f)
    f = ad.collision_kbc(f, ad.get_equilibrium(rho, u), omega)   # omega: float or 0-d tensor
    ...
    loss.backward()

Scalar parameters (omega, wall values, spring constants, marker spacing) may be Python
numbers or 0-d tensors; gradients flow to the tensors.  Every reduction over nodes runs
in a fixed order, so gradients are the same bits from run to run.
"""

import ctypes as C

import numpy as np
import torch

from . import _ib
from . import _lib as V
from . import lbm as _lbm
from . import lbm3d as _lbm3d
from ._ops import _M9, _m19, mrt_relaxation

# ----------------------------------------------------------------- helpers


def _lat(f):
    return _lbm._LAT if f.shape[0] == 9 else _lbm3d._LAT


def _as_tensor(x, like):
    """A 0-d tensor on like's device and dtype (keeps the autograd history of tensors)."""
    if isinstance(x, torch.Tensor):
        return x.to(device=like.device, dtype=like.dtype).reshape(())
    return torch.tensor(float(x), device=like.device, dtype=like.dtype)


def _needs(x):
    return isinstance(x, torch.Tensor) and x.requires_grad


def _grid_dims(f):
    s = tuple(f.shape[1:])
    return (s[0], s[1], 1) if len(s) == 2 else s


def _ordered_sum(x, stride=1, n=None):
    """Deterministic sum of x[0], x[stride], ... (vs_sum_ordered) as a 0-d tensor."""
    x = V.cont(x)
    if n is None:
        n = x.numel() // stride
    scratch = torch.empty(256, dtype=torch.float64, device=x.device)
    out = torch.empty((), dtype=torch.float64, device=x.device)
    V.call("vs_sum_ordered", V.dtype_code(x), V.ptr(x), int(n), int(stride), V.ptr(scratch), V.ptr(out), V.stream())
    return out.to(x.dtype)


def _zeros_like_or(g, like):
    return V.cont(g) if g is not None else torch.zeros_like(like)


# ----------------------------------------------------------------- streaming


class _Streaming(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f):
        return _lat(f).streaming(f)

    @staticmethod
    def backward(ctx, g):
        g = V.cont(g)
        out = torch.empty_like(g)
        nx, ny, nz = _grid_dims(g)
        V.call("vs_streaming_vjp", g.shape[0], V.dtype_code(g), V.ptr(g), V.ptr(out), nx, ny, nz, V.stream())
        return out


def streaming(f):
    """Periodic streaming (vivsim/lbm/basic.py:60-85, vivsim/lbm3d/basic.py:52-87)."""
    return _Streaming.apply(f)


# ----------------------------------------------------------------- moments, equilibrium


class _Macroscopic(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f):
        rho, u = _lat(f).get_macroscopic(f)
        ctx.save_for_backward(f)
        return rho, u

    @staticmethod
    def backward(ctx, g_rho, g_u):
        (f,) = ctx.saved_tensors
        if g_rho is None and g_u is None:
            return torch.zeros_like(f)
        f = V.cont(f)
        gf = torch.empty_like(f)
        g_rho = V.cont(g_rho) if g_rho is not None else None
        g_u = V.cont(g_u) if g_u is not None else None
        V.call("vs_macroscopic_vjp", f.shape[0], V.dtype_code(f), V.ptr(f), V.ptr(g_rho), V.ptr(g_u), V.ptr(gf),
               int(f[0].numel()), V.stream())
        return gf


def get_macroscopic(f):
    """rho, u (vivsim/lbm/basic.py:88-111, vivsim/lbm3d/basic.py:90-106)."""
    return _Macroscopic.apply(f)


class _Equilibrium(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho, u):
        lat = _lbm._LAT if u.shape[0] == 2 else _lbm3d._LAT
        ctx.save_for_backward(rho, u)
        return lat.get_equilibrium(rho, u)

    @staticmethod
    def backward(ctx, g):
        rho, u = ctx.saved_tensors
        g = V.cont(g)
        g_rho, g_u = torch.empty_like(rho), torch.empty_like(u)
        V.call("vs_equilibrium_vjp", g.shape[0], V.dtype_code(g), V.ptr(V.cont(rho)), V.ptr(V.cont(u)), V.ptr(g),
               V.ptr(g_rho), V.ptr(g_u), int(rho.numel()), V.stream())
        return g_rho, g_u


def get_equilibrium(rho, u):
    """feq (vivsim/lbm/basic.py:114-135, vivsim/lbm3d/basic.py:109-130)."""
    return _Equilibrium.apply(rho, u.to(rho.dtype))


def get_omega(nu):
    """1 / (3 nu + 0.5) (vivsim/lbm/basic.py:159-172); differentiable for a tensor nu."""
    return 1 / (3 * nu + 0.5)


# ----------------------------------------------------------------- collisions


class _Collide(torch.autograd.Function):
    @staticmethod
    def forward(ctx, kind, f, feq, omega):
        om = float(omega)
        out = _lat(f)._collide(kind, f, feq, om)
        ctx.kind, ctx.om = kind, om
        ctx.save_for_backward(f, feq)
        return out

    @staticmethod
    def backward(ctx, g):
        f, feq = ctx.saved_tensors
        g = V.cont(g)
        gf, gfeq = torch.empty_like(f), torch.empty_like(f)
        want_om = ctx.needs_input_grad[3]
        gnode = torch.empty(f.shape[1:], dtype=f.dtype, device=f.device) if want_om else None
        V.call("vs_collision_vjp", f.shape[0], V.dtype_code(f), ctx.kind, V.ptr(V.cont(f)), V.ptr(V.cont(feq)),
               ctx.om, V.ptr(g), V.ptr(gf), V.ptr(gfeq), V.ptr(gnode), int(f[0].numel()), V.stream())
        return None, gf, gfeq, (_ordered_sum(gnode) if want_om else None)


def _collide(kind, f, feq, omega):
    return _Collide.apply(kind, f, feq.to(f.dtype), _as_tensor(omega, f) if _needs(omega) else float(omega))


def collision_bgk(f, feq, omega):
    """(1 - omega) f + omega feq (vivsim/lbm/basic.py:138-156, lbm3d/basic.py:133-146)."""
    return _collide(V.VS_COLLIDE_BGK, f, feq, omega)


def collision_kbc(f, feq, omega):
    """Entropic KBC (vivsim/lbm/collision/kbc.py:10-60, lbm3d/collision/kbc.py:8-42)."""
    return _collide(V.VS_COLLIDE_KBC, f, feq, omega)


def collision_reg(f, feq, omega):
    """Regularised BGK (vivsim/lbm/collision/reg.py:4-49, lbm3d/collision/reg.py:44-62)."""
    return _collide(V.VS_COLLIDE_REG, f, feq, omega)


def get_mrt_collision_operator(omega, q=9, dtype=torch.float64, device="cuda"):
    """M^-1 S M (vivsim/lbm/collision/mrt.py:47-63, lbm3d/collision/mrt.py:75-80) as torch
    arithmetic on the reference's moment basis, differentiable in a tensor omega."""
    Mn = (_M9 if q == 9 else _m19()).astype(np.float64)
    M = torch.as_tensor(Mn, dtype=dtype, device=device)
    Mi = torch.as_tensor(np.linalg.inv(Mn), dtype=dtype, device=device)
    om = _as_tensor(omega, M) if isinstance(omega, torch.Tensor) else torch.tensor(float(omega), dtype=dtype,
                                                                                   device=device)
    marker = 1234.5  # the slots of S that hold omega
    rates = mrt_relaxation(q, marker)
    s = torch.stack([om if r == marker else torch.tensor(float(r), dtype=dtype, device=device) for r in rates])
    return Mi @ torch.diag(s) @ M


class _CollideMRT(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, feq, op):
        out = _lat(f).collision_mrt(f, feq, op)
        ctx.save_for_backward(f, feq, op)
        return out

    @staticmethod
    def backward(ctx, g):
        f, feq, op = ctx.saved_tensors
        q = f.shape[0]
        g = V.cont(g)
        gf, gfeq = torch.empty_like(f), torch.empty_like(f)
        a = np.ascontiguousarray(op.detach().cpu().double().numpy().reshape(-1))
        want_op = ctx.needs_input_grad[2]
        gop = torch.empty(q * q, dtype=torch.float64, device=f.device) if want_op else None
        # (the operator travels by value in the launch parameters: the host array is read
        # during the call)
        V.call("vs_collision_mrt_vjp", q, V.dtype_code(f), V.ptr(V.cont(f)), V.ptr(V.cont(feq)),
               a.ctypes.data_as(C.POINTER(C.c_double)), V.ptr(g), V.ptr(gf), V.ptr(gfeq), V.ptr(gop),
               int(f[0].numel()), V.stream())
        return gf, gfeq, (gop.reshape(q, q).to(op.dtype) if want_op else None)


def collision_mrt(f, feq, mrt_collision_matrix):
    """f + (M^-1 S M)(feq - f) (vivsim/lbm/collision/mrt.py:66-88)."""
    op = mrt_collision_matrix
    if not isinstance(op, torch.Tensor):
        op = torch.as_tensor(np.asarray(op, dtype=np.float64), device=f.device)
    return _CollideMRT.apply(f, feq.to(f.dtype), op)


# ----------------------------------------------------------------- forcing


class _Force(torch.autograd.Function):
    @staticmethod
    def forward(ctx, kind, f, g, u, omega):
        om = float(omega)
        out = _lat(f)._force(kind, f, g, u, om)
        ctx.kind, ctx.om = kind, om
        ctx.save_for_backward(g, u)
        return out

    @staticmethod
    def backward(ctx, go):
        g, u = ctx.saved_tensors
        go = V.cont(go)
        q = go.shape[0]
        gg, gu = torch.empty_like(g), torch.empty_like(u)
        want_om = ctx.kind == V.VS_FORCE_GUO_BGK and ctx.needs_input_grad[4]
        gs = torch.empty(go.shape[1:], dtype=go.dtype, device=go.device) if want_om else None
        V.call("vs_forcing_vjp", q, V.dtype_code(go), ctx.kind, V.ptr(V.cont(g)), V.ptr(V.cont(u)), ctx.om, V.ptr(go),
               None, V.ptr(gg), V.ptr(gu), V.ptr(gs), int(go[0].numel()), V.stream())
        g_om = -0.5 * _ordered_sum(gs) if want_om else None
        return None, go, gg, gu, g_om


def forcing_edm(f, g, u):
    """Exact-difference forcing (vivsim/lbm/forcing/edm.py:4-31, lbm3d/forcing/edm.py:6-26)."""
    return _Force.apply(V.VS_FORCE_EDM, f, g.to(f.dtype), u.to(f.dtype), 0.0)


def forcing_guo_bgk(f, g, u, omega):
    """Guo forcing for BGK (vivsim/lbm/forcing/guo.py:38-59)."""
    om = _as_tensor(omega, f) if _needs(omega) else float(omega)
    return _Force.apply(V.VS_FORCE_GUO_BGK, f, g.to(f.dtype), u.to(f.dtype), om)


def get_velocity_correction(g, rho=1):
    """g * 0.5 / rho (vivsim/lbm/basic.py:175-194), torch arithmetic."""
    return g * 0.5 / rho


# ----------------------------------------------------------------- boundaries

_KINDS = {"nee": V.VS_BC_NEE, "nebb": V.VS_BC_NEBB, "equilibrium": V.VS_BC_EQ}
_AXIS = {0: 0, 1: 0, 2: 1, 3: 1, 4: 2, 5: 2}


class _Boundary(torch.autograd.Function):
    @staticmethod
    def forward(ctx, kind, mode, loc, f, f_pre, rho, ux, uy, uz, gx, gy, gz):
        lat = _lat(f)
        vals = dict(rho=float(rho), ux=float(ux), uy=float(uy))
        if lat.d == 3:
            vals["uz"] = float(uz)
        if mode == V.VS_WALL_FORCE_CORRECTED:
            vals.update(gx=float(gx), gy=float(gy))
            if lat.d == 3:
                vals["gz"] = float(gz)
        out = lat._boundary(kind, mode, f, loc, vals, f_pre)
        ctx.kind, ctx.mode, ctx.loc = kind, mode, lat._loc(loc)
        ctx.vals = [float(x) for x in (rho, ux, uy, uz, gx, gy, gz)]
        ctx.save_for_backward(f, f_pre if f_pre is not None else f)
        ctx.has_pre = f_pre is not None
        return out

    @staticmethod
    def backward(ctx, go):
        f, f_pre = ctx.saved_tensors
        go = V.cont(go)
        nx, ny, nz = _grid_dims(f)
        rho, ux, uy, uz, gx, gy, gz = ctx.vals
        mode = ctx.mode
        u_eff = [ux, uy, uz]
        if mode == V.VS_WALL_FORCE_CORRECTED:  # the given wall at u - 0.5 g / rho (_helpers.py:156-177)
            u_eff = [ux - 0.5 * gx / rho, uy - 0.5 * gy / rho, uz - 0.5 * gz / rho]
            mode = V.VS_WALL_GIVEN
        gin = torch.empty_like(f)
        gpre = torch.empty_like(f) if ctx.has_pre else None
        want_wall = any(ctx.needs_input_grad[5:12])
        face = [nn for a, nn in enumerate((nx, ny, nz)) if a != _AXIS[ctx.loc]]
        nf = face[0] * face[1]
        gw = torch.empty(4 * nf, dtype=f.dtype, device=f.device) if want_wall else None
        V.call("vs_boundary_vjp", f.shape[0], V.dtype_code(f), ctx.kind, mode, ctx.loc, V.ptr(V.cont(f)),
               V.ptr(V.cont(f_pre)) if ctx.has_pre else None, V.ptr(go), V.ptr(gin), V.ptr(gpre), V.ptr(gw), nx, ny,
               nz, rho, u_eff[0], u_eff[1], u_eff[2], V.stream())
        grads = [None] * 7
        if want_wall:
            s = [_ordered_sum(gw[k:], stride=4, n=nf) for k in range(4)]  # rho, ux, uy, uz (effective)
            g_rho, g_u = s[0], s[1:]
            if ctx.mode == V.VS_WALL_FORCE_CORRECTED:
                gvec = (gx, gy, gz)
                g_rho = g_rho + sum(g_u[d] * (0.5 * gvec[d] / (rho * rho)) for d in range(3))
                grads[4:7] = [g_u[d] * (-0.5 / rho) for d in range(3)]
            grads[0:4] = [g_rho] + list(g_u)
            if ctx.mode == V.VS_WALL_VELOCITY:
                grads[0] = None
            if ctx.mode == V.VS_WALL_PRESSURE:
                grads[1:4] = [None, None, None]
            grads = [g if ctx.needs_input_grad[5 + i] else None for i, g in enumerate(grads)]
        return (None, None, None, gin, gpre) + tuple(grads)


def _boundary(kind, mode, f, loc, f_pre=None, rho=1.0, ux=0.0, uy=0.0, uz=0.0, gx=0.0, gy=0.0, gz=0.0):
    _lat(f)._loc(loc)  # an unknown face raises ValueError here
    vals = []
    for x in (rho, ux, uy, uz, gx, gy, gz):
        if isinstance(x, torch.Tensor) and x.numel() > 1:
            raise NotImplementedError("differentiable boundaries take scalar wall values")
        vals.append(_as_tensor(x, f) if _needs(x) else float(x))
    return _Boundary.apply(kind, mode, loc, f, f_pre, *vals)


def _make_boundary(kind, mode):
    if mode == V.VS_WALL_PRESSURE:
        def fn(f, loc, rho_wall=1):
            return _boundary(kind, mode, f, loc, rho=rho_wall)
    elif mode == V.VS_WALL_VELOCITY:
        def fn(f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
            return _boundary(kind, mode, f, loc, ux=ux_wall, uy=uy_wall, uz=uz_wall)
    elif mode == V.VS_WALL_FORCE_CORRECTED:
        def fn(f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0, gx_wall=0, gy_wall=0, gz_wall=0):
            return _boundary(kind, mode, f, loc, rho=rho_wall, ux=ux_wall, uy=uy_wall, uz=uz_wall, gx=gx_wall,
                             gy=gy_wall, gz=gz_wall)
    else:
        def fn(f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0):
            return _boundary(kind, mode, f, loc, rho=rho_wall, ux=ux_wall, uy=uy_wall, uz=uz_wall)
    return fn


for _scheme, _kind in _KINDS.items():
    globals()[f"boundary_{_scheme}"] = _make_boundary(_kind, V.VS_WALL_GIVEN)
    globals()[f"boundary_velocity_{_scheme}"] = _make_boundary(_kind, V.VS_WALL_VELOCITY)
    globals()[f"boundary_pressure_{_scheme}"] = _make_boundary(_kind, V.VS_WALL_PRESSURE)
    globals()[f"boundary_force_corrected_{_scheme}"] = _make_boundary(_kind, V.VS_WALL_FORCE_CORRECTED)


def boundary_bounce_back(f_before_stream, f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
    """Bounce-back wall (vivsim/lbm/boundary/bb.py:15-53, lbm3d/boundary/bb.py:20-34)."""
    return _boundary(V.VS_BC_BB, V.VS_WALL_GIVEN, f, loc, f_pre=f_before_stream, ux=ux_wall, uy=uy_wall, uz=uz_wall)


def boundary_specular_reflection(f_before_stream, f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
    """Specular reflection (vivsim/lbm/boundary/bb.py:56-95, lbm3d/boundary/bb.py:37-53)."""
    return _boundary(V.VS_BC_SPECULAR, V.VS_WALL_GIVEN, f, loc, f_pre=f_before_stream, ux=ux_wall, uy=uy_wall,
                     uz=uz_wall)


# ----------------------------------------------------------------- immersed boundary


def _pair_dot(A, grid, I, s):
    """out[m, s] = sum_c A[m, c] grid[c, I[m, s]] (vs_ib_pair_dot)."""
    A, grid = V.cont(A), V.cont(grid)
    m, c = int(A.shape[0]), int(A.shape[1])
    out = torch.empty((m, s), dtype=A.dtype, device=A.device)
    V.call("vs_ib_pair_dot", V.dtype_code(A), V.ptr(A), V.ptr(grid), c, int(grid[0].numel()), V.ptr(V.cont(I)), m, s,
           V.ptr(out), V.stream())
    return out


def _spread0(values, W, I, shape):
    """spread onto a zero grid of the given (c, ...) shape."""
    zero = torch.zeros(shape, dtype=values.dtype, device=values.device)
    return _ib.spread(values, zero, W, I)


class _Stencil2D(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, ny, kernel, radius):
        W, I = _ib.get_ib_stencil(x, y, ny, kernel, radius)
        ctx.save_for_backward(x, y)
        ctx.kernel, ctx.radius = _ib._kernel_code(kernel), radius
        ctx.mark_non_differentiable(I)
        return W, I

    @staticmethod
    def backward(ctx, gW, gI):
        x, y = ctx.saved_tensors
        x, y = V.cont(x), V.cont(y)
        gx, gy = torch.empty_like(x), torch.empty_like(y)
        gW = _zeros_like_or(gW, torch.empty((x.numel(), (2 * ctx.radius) ** 2), dtype=x.dtype, device=x.device))
        V.call("vs_ib_stencil_vjp", ctx.kernel, ctx.radius, V.dtype_code(x), 2, V.ptr(x), V.ptr(y), None, V.ptr(gW),
               V.ptr(gx), V.ptr(gy), None, int(x.numel()), V.stream())
        return gx, gy, None, None, None


def get_ib_stencil(marker_x, marker_y, ny, kernel=_ib.kernel_peskin_4pt, stencil_radius=2):
    """(W, I) (vivsim/ib/stencil.py:7-51); W is differentiable in the marker coordinates."""
    return _Stencil2D.apply(marker_x, marker_y.to(marker_x.dtype), int(ny), kernel, int(stencil_radius))


class _Stencil3D(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X, shape, kernel, radius):
        W, I = _ib.get_ib_stencil_3d(X, shape, kernel, radius)
        ctx.save_for_backward(X)
        ctx.kernel, ctx.radius = _ib._kernel_code(kernel), radius
        ctx.mark_non_differentiable(I)
        return W, I

    @staticmethod
    def backward(ctx, gW, gI):
        (X,) = ctx.saved_tensors
        cols = [V.cont(X[:, d]) for d in range(3)]
        g = [torch.empty_like(c) for c in cols]
        gW = _zeros_like_or(gW, torch.empty((X.shape[0], (2 * ctx.radius) ** 3), dtype=X.dtype, device=X.device))
        V.call("vs_ib_stencil_vjp", ctx.kernel, ctx.radius, V.dtype_code(X), 3, V.ptr(cols[0]), V.ptr(cols[1]),
               V.ptr(cols[2]), V.ptr(gW), V.ptr(g[0]), V.ptr(g[1]), V.ptr(g[2]), int(X.shape[0]), V.stream())
        return torch.stack(g, dim=1), None, None, None


def get_ib_stencil_3d(marker_coords, grid_shape, kernel=_ib.kernel_peskin_4pt, stencil_radius=2):
    """(W, I) (vivsim/ib3d/stencil.py:7-59); W is differentiable in the marker coordinates."""
    return _Stencil3D.apply(marker_coords, tuple(int(v) for v in grid_shape), kernel, int(stencil_radius))


class _Interpolate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid, W, I):
        out = _ib.interpolate(grid, W, I)
        ctx.save_for_backward(grid, W, I)
        return out

    @staticmethod
    def backward(ctx, gU):
        grid, W, I = ctx.saved_tensors
        gU = V.cont(gU)
        g_grid = _spread0(gU, W, I, grid.shape) if ctx.needs_input_grad[0] else None  # interp^T = spread
        g_W = _pair_dot(gU, grid, I, W.shape[1]) if ctx.needs_input_grad[1] else None
        return g_grid, g_W, None


def interpolate(grid_values, stencil_weights, stencil_indices):
    """(n_markers, n_components) (vivsim/ib/stencil.py:54-78)."""
    return _Interpolate.apply(grid_values, stencil_weights.to(grid_values.dtype), stencil_indices.to(torch.int32))


class _Spread(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, grid, W, I):
        out = _ib.spread(values, grid, W, I)
        ctx.save_for_backward(values, W, I)
        return out

    @staticmethod
    def backward(ctx, go):
        values, W, I = ctx.saved_tensors
        go = V.cont(go)
        g_vals = _ib.interpolate(go, W, I) if ctx.needs_input_grad[0] else None  # spread^T = interp
        g_W = _pair_dot(values, go, I, W.shape[1]) if ctx.needs_input_grad[2] else None
        return g_vals, go, g_W, None


def spread(marker_values, grid_values, stencil_weights, stencil_indices):
    """grid + scatter of marker values (vivsim/ib/stencil.py:81-110)."""
    return _Spread.apply(marker_values.to(grid_values.dtype), grid_values, stencil_weights.to(grid_values.dtype),
                         stencil_indices.to(torch.int32))


def mdf_vjp(grid_u, W, I, ut, ds, n_iter, gg, gh, want_ds=False):
    """Reverse of multi_direct_forcing (vivsim/ib/mdf.py:10-64): the MDF iterations run
    backwards over recomputed forward iterates, built from interpolate^T = spread, spread^T =
    interpolate and the weights' cotangents (vs_ib_pair_dot).  Returns the cotangents of
    grid_u, W, the target velocity and (want_ds) the marker spacing."""
    s = W.shape[1]
    cfac = (2.0 * ds).reshape(-1, 1)  # marker_ds * 2 (mdf.py:44)
    U = _ib.interpolate(grid_u, W, I)
    Us, Fs_list, V_list = [], [], []
    Ft = torch.zeros_like(ut)
    for _ in range(n_iter):
        Us.append(U)
        Fs = (ut - U) * cfac
        Ft = Ft + Fs
        Vk = _spread0(Fs, W, I, grid_u.shape) * 0.5
        U = U + _ib.interpolate(Vk, W, I)
        Fs_list.append(Fs)
        V_list.append(Vk)
    gg = _zeros_like_or(gg, grid_u)
    gh = _zeros_like_or(gh, ut)
    gFt = _ib.interpolate(gg, W, I) - gh
    gW = _pair_dot(Ft, gg, I, s)
    gU = torch.zeros_like(ut)
    gUt = torch.zeros_like(ut)
    gc = torch.zeros_like(cfac)
    for k in range(n_iter - 1, -1, -1):
        gV = _spread0(gU, W, I, grid_u.shape)
        gW = gW + _pair_dot(gU, V_list[k], I, s)
        gFs = _ib.interpolate(gV, W, I) * 0.5 + gFt
        gW = gW + 0.5 * _pair_dot(Fs_list[k], gV, I, s)
        gUt = gUt + gFs * cfac
        gc = gc + (gFs * (ut - Us[k])).sum(dim=1, keepdim=True)
        gU = gU - gFs * cfac
    g_grid = _spread0(gU, W, I, grid_u.shape)
    gW = gW + _pair_dot(gU, grid_u, I, s)
    g_ds = None
    if want_ds:
        g_ds = 2.0 * gc.reshape(-1)
        g_ds = _ordered_sum(g_ds).reshape(ds.shape) if ds.numel() == 1 else g_ds.reshape(ds.shape)
    return g_grid, gW, gUt, g_ds


class _MDF(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid_u, W, I, u_target, ds, n_iter):
        ds_arg = ds if ds.numel() > 1 else float(ds)
        g, mh = _ib.multi_direct_forcing(grid_u, W, I, u_target, ds_arg, n_iter)
        ctx.n_iter = n_iter
        ctx.save_for_backward(grid_u, W, I, u_target, ds)
        return g, mh

    @staticmethod
    def backward(ctx, gg, gh):
        grid_u, W, I, ut, ds = ctx.saved_tensors
        g_grid, gW, gUt, g_ds = mdf_vjp(grid_u, W, I, ut, ds, ctx.n_iter, gg, gh, ctx.needs_input_grad[4])
        return g_grid, gW, None, gUt, g_ds, None


def multi_direct_forcing(grid_u, stencil_weights, stencil_indices, marker_u_target, marker_ds, n_iter=5):
    """(grid_force, marker_reaction_force) (vivsim/ib/mdf.py:10-64)."""
    dt = grid_u.dtype
    ds = marker_ds if isinstance(marker_ds, torch.Tensor) else torch.tensor(float(marker_ds), dtype=dt,
                                                                            device=grid_u.device)
    return _MDF.apply(grid_u, stencil_weights.to(dt), stencil_indices.to(torch.int32), marker_u_target.to(dt),
                      ds.to(dt), int(n_iter))


# ----------------------------------------------------------------- rigid-body dynamics


class _Newmark(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, v, d, h, m, k, c, dt, gamma, beta):
        x = [V.cont(t.reshape(-1)) for t in (a, v, d, h)]
        nd = int(x[0].numel())
        outs = [torch.empty_like(x[0]) for _ in range(3)]
        V.call("vs_newmark", V.dtype_code(x[0]), nd, *[V.ptr(t) for t in x], float(m), float(k), float(c), None, None,
               None, float(dt), float(gamma), float(beta), *[V.ptr(t) for t in outs], V.stream())
        ctx.save_for_backward(*x)
        ctx.consts = (float(m), float(k), float(c), float(dt), float(gamma), float(beta))
        ctx.shape = a.shape
        return tuple(t.reshape(a.shape) for t in outs)

    @staticmethod
    def backward(ctx, ga, gv, gd):
        a, v, d, h = ctx.saved_tensors
        m, k, c, dt, gamma, beta = ctx.consts
        nd = int(a.numel())
        g_in = [V.cont(g.reshape(-1)) if g is not None else None for g in (ga, gv, gd)]
        outs = [torch.empty_like(a) for _ in range(4)]
        gmkc = torch.empty(3, dtype=a.dtype, device=a.device)
        V.call("vs_newmark_vjp", V.dtype_code(a), nd, V.ptr(a), V.ptr(v), V.ptr(d), V.ptr(h), m, k, c, None, None, None,
               dt, gamma, beta, *[V.ptr(t) for t in g_in], *[V.ptr(t) for t in outs], V.ptr(gmkc), None, V.stream())
        res = [t.reshape(ctx.shape) for t in outs]
        scal = [gmkc[i] if ctx.needs_input_grad[4 + i] else None for i in range(3)]
        return (*res, *scal, None, None, None)


def newmark(a, v, d, h, m, k, c, dt=1, gamma=0.5, beta=0.25):
    """Newmark-beta, scalar branch (vivsim/dyn.py:5-51, :42-45); a, v, d, h tensors (any
    shape, one DOF per element), m, k, c numbers or 0-d tensors."""
    def sc(x):
        return _as_tensor(x, a) if _needs(x) else float(x)

    return _Newmark.apply(a, v.to(a.dtype), d.to(a.dtype), h.to(a.dtype), sc(m), sc(k), sc(c), float(dt),
                          float(gamma), float(beta))


newmark_2dof = newmark
newmark_3dof = newmark


def get_markers_coords_2dof(x_markers_init, y_markers_init, d):
    """(vivsim/dyn.py:68-81)."""
    return x_markers_init + d[0], y_markers_init + d[1]


def get_markers_coords_3dof(x_markers_init, y_markers_init, x_center_init, y_center_init, d):
    """(vivsim/dyn.py:84-99)."""
    xr, yr = x_markers_init - x_center_init, y_markers_init - y_center_init
    cs, sn = torch.cos(d[2]), torch.sin(d[2])
    return x_center_init + d[0] + xr * cs - yr * sn, y_center_init + d[1] + xr * sn + yr * cs


def get_force_to_obj(h_markers):
    """Total force on the body, summed over the markers (vivsim/dyn.py:126-136)."""
    return torch.sum(h_markers, dim=0)


def get_torque_to_obj(x_markers, y_markers, x_center_init, y_center_init, d, h_markers):
    """(vivsim/dyn.py:139-154)."""
    xr = x_markers - (x_center_init + d[0])
    yr = y_markers - (y_center_init + d[1])
    return torch.sum(xr * h_markers[:, 1] - yr * h_markers[:, 0])


kernel_peskin_3pt = _ib.kernel_peskin_3pt
kernel_peskin_4pt = _ib.kernel_peskin_4pt
kernel_cosine_4pt = _ib.kernel_cosine_4pt
