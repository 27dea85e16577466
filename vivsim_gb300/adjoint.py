"""Gradients of the 2-D cylinder VIV drag by the hand-written discrete adjoint.

The reference differentiates its jitted update loop with ``jax.grad``
(examples/2d/vortex_induced_vibration.py:96-157 is the loop).  Here the forward run is the
fused CUDA step and the gradient comes from adjoint kernels (reverse streaming fused with
the transposed collision/forcing Jacobian, the transposed immersed-boundary operators and
Newmark), with the populations checkpointed every ``checkpoint_every`` steps.

    drag = CylinderDrag(nx=512, ny=256, ...)
    J = drag.forward()                      # objective
    gU0, gK, goff = drag.backward()         # its gradient

``cylinder_drag(U0, K, offsets, **case)`` is the same as a ``torch.autograd.Function``.
"""

import ctypes as C
import math

import numpy as np
import torch

from . import _lib as V
from ._ops import _M9, mrt_collision_operator
from .solver import COLLISIONS, KERNELS


class CylinderDrag:
    """Mean x force on a spring-mounted cylinder over steps [obj_start, n_steps)."""

    def __init__(self, nx=512, ny=256, U0=0.05, D=20.0, Re=100.0, n_markers=64, offsets=None, center=None,
                 mass_ratio=10.0, U_r=5.0, stiffness=None, damping=0.0, n_steps=4000, checkpoint_every=100,
                 obj_start=None, kernel="peskin4", radius=2, n_iter=3, rho_out=1.0, dtype=torch.float32,
                 collision="bgk"):
        self.M = int(n_markers)
        off = np.zeros(self.M) if offsets is None else np.asarray(offsets, dtype=np.float64).reshape(-1)
        if off.shape[0] != self.M:
            raise ValueError("offsets must have n_markers entries")
        self._off = np.ascontiguousarray(off)
        area = math.pi * (D / 2) ** 2
        mass = area * mass_ratio
        if stiffness is None:  # spring from the reduced velocity (examples/2d/vortex_induced_vibration.py:56-59)
            fn = U0 / (U_r * D)
            stiffness = (2 * math.pi * fn) ** 2 * mass * (1 + 1 / mass_ratio)
        cx, cy = (nx / 4.0, ny / 2.0) if center is None else center
        cfg = V.vs_adjoint_cfg()
        cfg.dtype = V.VS_F64 if dtype in (torch.float64, "float64", np.float64) else V.VS_F32
        cfg.nx, cfg.ny = int(nx), int(ny)
        cfg.U0, cfg.D, cfg.Re, cfg.rho_out = float(U0), float(D), float(Re), float(rho_out)
        cfg.n_markers = self.M
        cfg.cx, cfg.cy = float(cx), float(cy)
        cfg.offsets_host = self._off.ctypes.data_as(C.POINTER(C.c_double))
        cfg.kernel, cfg.radius, cfg.n_iter = KERNELS[kernel], int(radius), int(n_iter)
        cfg.mass, cfg.stiffness, cfg.damping, cfg.added_mass_area = mass, float(stiffness), float(damping), area
        cfg.n_steps = int(n_steps)
        cfg.checkpoint_every = int(checkpoint_every)
        cfg.obj_start = int(n_steps // 2 if obj_start is None else obj_start)
        cfg.collision = COLLISIONS[collision]
        if collision == "mrt":
            # operator at omega = 1 / (3 U0 D / Re + 0.5) and its derivative in omega
            # (only the two shear rates of lbm/collision/mrt.py:44 depend on omega)
            omega = 1.0 / (3.0 * U0 * D / Re + 0.5)
            op = mrt_collision_operator(9, omega, torch.float64).numpy().reshape(-1)
            Mi = np.linalg.inv(_M9.astype(np.float64))
            dS = np.diag([0, 0, 0, 0, 0, 0, 0, 1.0, 1.0])
            dop = (Mi @ dS @ _M9.astype(np.float64)).reshape(-1)
            for i in range(81):
                cfg.mrt_op[i] = float(op[i])
                cfg.mrt_dop[i] = float(dop[i])
        self.cfg = cfg
        self.stiffness = float(stiffness)
        h = C.c_void_p()
        V.call("vs_adjoint_plan_create", C.byref(cfg), C.byref(h))
        self.handle = h

    def forward(self, keep_checkpoints=True):
        J = C.c_double()
        V.call("vs_adjoint_forward", self.handle, 1 if keep_checkpoints else 0, C.byref(J), V.stream())
        return J.value

    def backward(self, seed=1.0):
        gU0, gK = C.c_double(), C.c_double()
        goff = (C.c_double * self.M)()
        V.call("vs_adjoint_backward", self.handle, float(seed), C.byref(gU0), C.byref(gK), goff, V.stream())
        return gU0.value, gK.value, np.frombuffer(goff, dtype=np.float64).copy()

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            V.lib().vs_adjoint_plan_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _DragFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U0, K, offsets, case):
        plan = CylinderDrag(U0=float(U0), stiffness=float(K), offsets=offsets.detach().cpu().numpy(), **case)
        J = plan.forward(keep_checkpoints=True)
        ctx.plan = plan
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        gU0, gK, goff = ctx.plan.backward(float(gJ))
        ctx.plan.close()
        return (torch.tensor(gU0, dtype=torch.float64), torch.tensor(gK, dtype=torch.float64),
                torch.from_numpy(goff), None)


def cylinder_drag(U0, K, offsets, **case):
    """Differentiable objective J(U0, K, offsets) (tensors in, 0-d float64 tensor out)."""
    return _DragFn.apply(U0, K, offsets, case)
