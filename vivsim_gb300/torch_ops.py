"""The per-operator kernels as PyTorch operators (``torch.ops.vivsim.*``).

Registered with ``torch.library.custom_op`` so that they compose with other PyTorch code
(fake implementations give shapes to tracing).  Each forwards to the C-ABI shim of the
same name in ``vivsim_gb300.lbm`` / ``lbm3d`` / ``ib``, i.e. to one CUDA kernel.

    import vivsim_gb300.torch_ops  # registers the operators
    f = torch.ops.vivsim.collision_kbc(f, feq, 1.8)
"""

import torch

from . import ib as _ib
from . import lbm as _lbm
from . import lbm3d as _lbm3d
from . import multigrid as _mg


def _lat(f):
    return _lbm if f.shape[0] == 9 else _lbm3d


@torch.library.custom_op("vivsim::streaming", mutates_args=())
def streaming(f: torch.Tensor) -> torch.Tensor:
    return _lat(f).streaming(f)


@streaming.register_fake
def _(f):
    return torch.empty_like(f)


@torch.library.custom_op("vivsim::get_macroscopic", mutates_args=())
def get_macroscopic(f: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    return _lat(f).get_macroscopic(f)


@get_macroscopic.register_fake
def _(f):
    d = f.dim() - 1
    return f.new_empty(f.shape[1:]), f.new_empty((d,) + tuple(f.shape[1:]))


@torch.library.custom_op("vivsim::get_equilibrium", mutates_args=())
def get_equilibrium(rho: torch.Tensor, u: torch.Tensor) -> torch.Tensor:
    return (_lbm if u.shape[0] == 2 else _lbm3d).get_equilibrium(rho, u)


@get_equilibrium.register_fake
def _(rho, u):
    q = 9 if u.shape[0] == 2 else 19
    return rho.new_empty((q,) + tuple(rho.shape))


def _collision(name):
    @torch.library.custom_op(f"vivsim::{name}", mutates_args=())
    def op(f: torch.Tensor, feq: torch.Tensor, omega: float) -> torch.Tensor:
        return getattr(_lat(f), name)(f, feq, omega)

    @op.register_fake
    def _(f, feq, omega):
        return torch.empty_like(f)

    return op


collision_bgk = _collision("collision_bgk")
collision_kbc = _collision("collision_kbc")
collision_reg = _collision("collision_reg")


@torch.library.custom_op("vivsim::forcing_edm", mutates_args=())
def forcing_edm(f: torch.Tensor, g: torch.Tensor, u: torch.Tensor) -> torch.Tensor:
    return _lat(f).forcing_edm(f, g, u)


@forcing_edm.register_fake
def _(f, g, u):
    return torch.empty_like(f)


@torch.library.custom_op("vivsim::interpolate", mutates_args=())
def interpolate(grid_values: torch.Tensor, stencil_weights: torch.Tensor, stencil_indices: torch.Tensor) -> torch.Tensor:
    return _ib.interpolate(grid_values, stencil_weights, stencil_indices)


@interpolate.register_fake
def _(grid_values, stencil_weights, stencil_indices):
    return grid_values.new_empty((stencil_weights.shape[0], grid_values.shape[0]))


@torch.library.custom_op("vivsim::spread", mutates_args=())
def spread(marker_values: torch.Tensor, grid_values: torch.Tensor, stencil_weights: torch.Tensor,
           stencil_indices: torch.Tensor) -> torch.Tensor:
    return _ib.spread(marker_values, grid_values, stencil_weights, stencil_indices)


@spread.register_fake
def _(marker_values, grid_values, stencil_weights, stencil_indices):
    return torch.empty_like(grid_values)


@torch.library.custom_op("vivsim::multi_direct_forcing", mutates_args=())
def multi_direct_forcing(grid_u: torch.Tensor, stencil_weights: torch.Tensor, stencil_indices: torch.Tensor,
                         marker_u_target: torch.Tensor, marker_ds: float,
                         n_iter: int) -> tuple[torch.Tensor, torch.Tensor]:
    return _ib.multi_direct_forcing(grid_u, stencil_weights, stencil_indices, marker_u_target, marker_ds, n_iter)


@multi_direct_forcing.register_fake
def _(grid_u, stencil_weights, stencil_indices, marker_u_target, marker_ds, n_iter):
    return torch.empty_like(grid_u), marker_u_target.new_empty(marker_u_target.shape)


@torch.library.custom_op("vivsim::fine_to_coarse", mutates_args=())
def fine_to_coarse(f_fine: torch.Tensor, f_coarse: torch.Tensor, dir: str) -> torch.Tensor:
    out = _mg.fine_to_coarse(f_fine, f_coarse, dir)
    return out.clone() if out.data_ptr() == f_coarse.data_ptr() else out  # an operator returns no alias


@fine_to_coarse.register_fake
def _(f_fine, f_coarse, dir):
    return torch.empty_like(f_coarse)


@torch.library.custom_op("vivsim::coarse_to_fine", mutates_args=())
def coarse_to_fine(f_coarse: torch.Tensor, f_fine: torch.Tensor, dir: str) -> torch.Tensor:
    out = _mg.coarse_to_fine(f_coarse, f_fine, dir)
    return out.clone() if out.data_ptr() == f_fine.data_ptr() else out


@coarse_to_fine.register_fake
def _(f_coarse, f_fine, dir):
    return torch.empty_like(f_fine)


# ------------------------------------------------------------------ backward passes
# Reverse-mode rules for the operators above, from the hand-written vector-Jacobian
# kernels (csrc/vs_grad.cu, through vivsim_gb300.autodiff).  Scalar float arguments
# (omega, marker_ds given as a float) are constants here; vivsim_gb300.autodiff takes them
# as tensors when their gradient is wanted.

from . import _lib as _V  # noqa: E402
from . import autodiff as _ad  # noqa: E402


def _save_inputs(ctx, inputs, output):
    ctx.save_for_backward(*[x for x in inputs if isinstance(x, torch.Tensor)])
    ctx.scalars = [x for x in inputs if not isinstance(x, torch.Tensor)]


streaming.register_autograd(lambda ctx, g: _ad._Streaming.backward(ctx, g), setup_context=_save_inputs)
get_macroscopic.register_autograd(lambda ctx, g_rho, g_u: _ad._Macroscopic.backward(ctx, g_rho, g_u),
                                  setup_context=_save_inputs)
get_equilibrium.register_autograd(lambda ctx, g: _ad._Equilibrium.backward(ctx, g), setup_context=_save_inputs)


def _collision_backward(kind):
    def bwd(ctx, g):
        f, feq = ctx.saved_tensors
        g = _V.cont(g)
        gf, gfeq = torch.empty_like(f), torch.empty_like(f)
        _V.call("vs_collision_vjp", f.shape[0], _V.dtype_code(f), kind, _V.ptr(_V.cont(f)), _V.ptr(_V.cont(feq)),
                float(ctx.scalars[0]), _V.ptr(g), _V.ptr(gf), _V.ptr(gfeq), None, int(f[0].numel()), _V.stream())
        return gf, gfeq, None
    return bwd


collision_bgk.register_autograd(_collision_backward(_V.VS_COLLIDE_BGK), setup_context=_save_inputs)
collision_kbc.register_autograd(_collision_backward(_V.VS_COLLIDE_KBC), setup_context=_save_inputs)
collision_reg.register_autograd(_collision_backward(_V.VS_COLLIDE_REG), setup_context=_save_inputs)


def _forcing_edm_backward(ctx, go):
    f, g, u = ctx.saved_tensors
    go = _V.cont(go)
    gg, gu = torch.empty_like(g), torch.empty_like(u)
    _V.call("vs_forcing_vjp", go.shape[0], _V.dtype_code(go), _V.VS_FORCE_EDM, _V.ptr(_V.cont(g)), _V.ptr(_V.cont(u)),
            0.0, _V.ptr(go), None, _V.ptr(gg), _V.ptr(gu), None, int(go[0].numel()), _V.stream())
    return go, gg, gu


forcing_edm.register_autograd(_forcing_edm_backward, setup_context=_save_inputs)


def _interpolate_backward(ctx, gU):
    grid, W, I = ctx.saved_tensors
    gU = _V.cont(gU)
    return _ad._spread0(gU, W, I, grid.shape), _ad._pair_dot(gU, grid, I, W.shape[1]), None


interpolate.register_autograd(_interpolate_backward, setup_context=_save_inputs)


def _spread_backward(ctx, go):
    values, grid, W, I = ctx.saved_tensors
    go = _V.cont(go)
    return _ib.interpolate(go, W, I), go, _ad._pair_dot(values, go, I, W.shape[1]), None


spread.register_autograd(_spread_backward, setup_context=_save_inputs)


def _mdf_backward(ctx, gg, gh):
    grid_u, W, I, ut = ctx.saved_tensors
    ds, n_iter = ctx.scalars
    ds_t = torch.tensor(float(ds), dtype=grid_u.dtype, device=grid_u.device)
    g_grid, gW, gUt, _ = _ad.mdf_vjp(grid_u, W, I, ut, ds_t, int(n_iter), gg, gh)
    return g_grid, gW, None, gUt, None, None


multi_direct_forcing.register_autograd(_mdf_backward, setup_context=_save_inputs)
