"""D3Q19 operators with the signatures of ``vivsim.lbm3d`` (vivsim/lbm3d/__init__.py:1-44).

Arrays are CUDA tensors of shape (19, NX, NY, NZ) / (3, NX, NY, NZ) / (NX, NY, NZ); each call runs
one kernel of libvivsim_gb300 on the current CUDA stream.
"""

from .._ops import Lattice, export

_LAT = Lattice(19)
export(globals(), _LAT)

__all__ = [
    "streaming", "collision_bgk", "get_equilibrium", "get_macroscopic", "get_velocity_correction", "get_omega",
    "collision_kbc", "get_mrt_collision_operator", "collision_mrt", "collision_reg", "forcing_edm",
    "get_guo_forcing_term", "forcing_guo_bgk", "get_mrt_forcing_operator", "forcing_guo_mrt",
    "boundary_bounce_back", "boundary_specular_reflection", "obstacle_bounce_back", "boundary_characteristic",
    "boundary_equilibrium", "boundary_force_corrected_equilibrium", "boundary_pressure_equilibrium",
    "boundary_velocity_equilibrium", "boundary_force_corrected_nebb", "boundary_nebb", "boundary_pressure_nebb",
    "boundary_velocity_nebb", "boundary_nee", "boundary_force_corrected_nee", "boundary_pressure_nee",
    "boundary_velocity_nee",
]
