"""Immersed-boundary operators (3-D) with the signatures of ``vivsim.ib3d`` (vivsim/ib3d/__init__.py:3-12)."""

from .._ib import get_ib_stencil_3d as get_ib_stencil
from .._ib import (get_surface_area, get_triangle_areas, get_volume, interpolate, kernel_cosine_4pt,
                   kernel_peskin_3pt, kernel_peskin_4pt, multi_direct_forcing, spread)
from .._ib import get_vertex_ds as get_ds

__all__ = ["get_ds", "get_surface_area", "get_triangle_areas", "get_volume", "get_ib_stencil",
           "kernel_cosine_4pt", "kernel_peskin_3pt", "kernel_peskin_4pt", "multi_direct_forcing", "interpolate",
           "spread"]
