"""Discrete adjoint of the cylinder VIV drag against central finite differences (FP64).

128 x 64 grid, 200 steps, objective = mean x force over the last 100 steps; gradients with
respect to the inflow velocity U0, the spring stiffness and marker radial offsets.  Bar:
1e-3 relative to the finite difference (the FP64 finite differences are accurate to
about 1e-8 here, so agreement is limited by the adjoint itself).
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

CASE = dict(nx=128, ny=64, D=10.0, Re=50.0, n_markers=32, n_steps=200, checkpoint_every=50, obj_start=100,
            dtype=torch.float64)


@pytest.fixture(scope="module")
def A():
    import vivsim_gb300
    vivsim_gb300.build()
    from vivsim_gb300 import adjoint
    return adjoint


def _J(A, U0, K, off, collision="bgk"):
    p = A.CylinderDrag(U0=U0, stiffness=K, offsets=off, collision=collision, **CASE)
    J = p.forward(keep_checkpoints=False)
    p.close()
    return J


@pytest.mark.parametrize("collision", ["bgk", "kbc", "mrt", "reg"])
def test_adjoint_matches_finite_differences(A, collision):
    """BGK has a hand-derived node transpose; KBC, MRT and regularised go through the
    dual-number node Jacobian."""
    off = np.random.default_rng(2).normal(0.0, 0.1, CASE["n_markers"])
    base = A.CylinderDrag(U0=0.05, offsets=off, collision=collision, **CASE)
    K = base.stiffness
    J = base.forward()
    gU0, gK, goff = base.backward()
    assert np.isfinite(J) and J != 0.0
    h = 1e-4
    fd_U0 = (_J(A, 0.05 * (1 + h), K, off, collision) - _J(A, 0.05 * (1 - h), K, off, collision)) / (2 * 0.05 * h)
    fd_K = (_J(A, 0.05, K * (1 + h), off, collision) - _J(A, 0.05, K * (1 - h), off, collision)) / (2 * K * h)
    assert abs(gU0 - fd_U0) <= 1e-3 * abs(fd_U0), (gU0, fd_U0)
    assert abs(gK - fd_K) <= 1e-3 * abs(fd_K), (gK, fd_K)
    scale = np.max(np.abs(goff))
    for m in (0, 7, 19):
        op, om = off.copy(), off.copy()
        op[m] += 1e-4
        om[m] -= 1e-4
        fd = (_J(A, 0.05, K, op, collision) - _J(A, 0.05, K, om, collision)) / 2e-4
        assert abs(goff[m] - fd) <= 1e-3 * max(abs(fd), 1e-2 * scale), (m, goff[m], fd)


def test_autograd_function_matches_plan(A):
    off = np.random.default_rng(2).normal(0.0, 0.1, CASE["n_markers"])
    ref = A.CylinderDrag(U0=0.05, offsets=off, **CASE)
    J0 = ref.forward()
    g0 = ref.backward()
    U0 = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    K = torch.tensor(ref.stiffness, dtype=torch.float64, requires_grad=True)
    o = torch.tensor(off, dtype=torch.float64, requires_grad=True)
    J = A.cylinder_drag(U0, K, o, **CASE)
    J.backward()
    # every gradient sum runs in a fixed order: the two computations agree bit for bit
    assert float(J.detach()) == J0
    assert float(U0.grad) == g0[0]
    assert float(K.grad) == g0[1]
    assert np.array_equal(o.grad.numpy(), g0[2])


def test_adjoint_float32_runs_close_to_float64(A):
    off = np.random.default_rng(2).normal(0.0, 0.1, CASE["n_markers"])
    case32 = dict(CASE, dtype=torch.float32)
    p32 = A.CylinderDrag(U0=0.05, offsets=off, **case32)
    p64 = A.CylinderDrag(U0=0.05, offsets=off, **CASE)
    p32.forward()
    p64.forward()
    g32, g64 = p32.backward(), p64.backward()
    assert abs(g32[0] - g64[0]) <= 1e-2 * abs(g64[0])
    assert abs(g32[1] - g64[1]) <= 1e-2 * abs(g64[1])
    assert np.max(np.abs(g32[2] - g64[2])) <= 1e-2 * np.max(np.abs(g64[2]))


def test_adjoint_config4_size_matches_finite_differences(A):
    """The differentiable-cylinder configuration itself (512 x 256, D = 20, Re 100, 64
    markers with N(0, 0.1) radial offsets, 4000 steps, checkpoints every 100, objective the
    mean drag over the second half), in FP64: the adjoint gradients against central finite
    differences with h = 1e-3 relative (1e-4 absolute for an offset)."""
    full = dict(nx=512, ny=256, D=20.0, Re=100.0, n_markers=64, n_steps=4000, checkpoint_every=100, obj_start=2000,
                dtype=torch.float64)
    off = np.random.default_rng(2).normal(0.0, 0.1, 64)

    def J(U0, K, o):
        p = A.CylinderDrag(U0=U0, stiffness=K, offsets=o, **full)
        v = p.forward(keep_checkpoints=False)
        p.close()
        return v

    base = A.CylinderDrag(U0=0.05, offsets=off, **full)
    K = base.stiffness
    J0 = base.forward()
    gU0, gK, goff = base.backward()
    base.close()
    h = 1e-3
    fd_U0 = (J(0.05 * (1 + h), K, off) - J(0.05 * (1 - h), K, off)) / (2 * 0.05 * h)
    fd_K = (J(0.05, K * (1 + h), off) - J(0.05, K * (1 - h), off)) / (2 * K * h)
    print(f"\nconfig 4: J {J0:.12e}; dJ/dU0 adjoint {gU0:.10e} fd {fd_U0:.10e}; dJ/dK adjoint {gK:.6e} fd {fd_K:.6e}")
    assert abs(gU0 - fd_U0) <= 1e-3 * abs(fd_U0), (gU0, fd_U0)
    scale = np.max(np.abs(goff))
    assert abs(gK - fd_K) <= 1e-3 * max(abs(fd_K), 1e-6 * abs(fd_U0)), (gK, fd_K)
    for m in (3, 40):
        op, om = off.copy(), off.copy()
        op[m] += 1e-4
        om[m] -= 1e-4
        fd = (J(0.05, K, op) - J(0.05, K, om)) / 2e-4
        print(f"dJ/d offset[{m}] adjoint {goff[m]:.8e} fd {fd:.8e}")
        assert abs(goff[m] - fd) <= 1e-3 * max(abs(fd), 1e-2 * scale), (m, goff[m], fd)
