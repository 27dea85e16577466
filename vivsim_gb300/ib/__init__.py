"""Immersed-boundary operators (2-D) with the signatures of ``vivsim.ib`` (vivsim/ib/__init__.py:3-6)."""

from .._ib import (get_area, get_ds, get_ib_stencil, interpolate, kernel_cosine_4pt, kernel_peskin_3pt,
                   kernel_peskin_4pt, multi_direct_forcing, spread)

__all__ = ["get_area", "get_ds", "kernel_cosine_4pt", "kernel_peskin_3pt", "kernel_peskin_4pt",
           "multi_direct_forcing", "get_ib_stencil", "interpolate", "spread"]
