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
