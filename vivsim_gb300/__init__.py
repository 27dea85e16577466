"""vivsim_gb300 — GB300-native (sm_103a) IB-LBM time step with the API of haimingz/vivsim.

Subpackages mirror the reference's modules: ``lbm`` (D2Q9), ``lbm3d`` (D3Q19), ``ib``,
``ib3d`` and ``dyn`` keep its pure-function signatures on CUDA tensors; ``solver`` runs the
fused multi-step loop.  All compute goes through ``libvivsim_gb300.so`` (C ABI in
include/vivsim_gb300.h); nothing falls back to the CPU.
"""

from . import _lib  # noqa: F401

__version__ = "1.0.0"


def build(verbose=False, force=False):
    """Compile the CUDA library in-tree (nvcc, sm_103a) and return its path."""
    from . import _build
    return _build.build(verbose=verbose, force=force)
