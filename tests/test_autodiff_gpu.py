"""Reverse-mode gradients of the per-operator functions (vivsim_gb300.autodiff and the
torch.ops.vivsim backward rules) in float64.

* Each function's hand-written vector-Jacobian product against torch.autograd.gradcheck
  (central finite differences of the forward CUDA kernel).
* Gradients are deterministic: two backward passes give the same bits.
* An update step composed from the differentiable functions, as the reference's VIV
  example composes it (examples/2d/vortex_induced_vibration.py:96-148), differentiates end
  to end and matches the fused discrete adjoint (adjoint.CylinderDrag) to 1e-10.
"""

import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DT = torch.float64


@pytest.fixture(scope="module")
def ad():
    import vivsim_gb300
    vivsim_gb300.build()
    from vivsim_gb300 import autodiff
    return autodiff


def rnd(*shape, seed=0, scale=1.0, shift=0.0):
    g = torch.Generator().manual_seed(seed)
    return (shift + scale * torch.rand(*shape, generator=g, dtype=DT)).cuda()


def populations(q, shape, seed=0, spread=0.02):
    """Positive populations near an equilibrium with u ~ 0.05 (smooth inputs for the
    collision models); ``spread`` is the relative size of their non-equilibrium part."""
    from vivsim_gb300 import lbm, lbm3d
    L = lbm if q == 9 else lbm3d
    rho = rnd(*shape, seed=seed, scale=0.05, shift=0.98)
    u = rnd(len(shape), *shape, seed=seed + 1, scale=0.04, shift=-0.02)
    u[0] += 0.05
    f = L.get_equilibrium(rho, u)
    return (f * rnd(q, *shape, seed=seed + 2, scale=spread, shift=1.0 - 0.5 * spread)).contiguous()


def check(fn, *inputs, atol=1e-7, rtol=1e-5):
    ins = tuple(x.detach().clone().requires_grad_(True) if isinstance(x, torch.Tensor) and x.is_floating_point()
                else x for x in inputs)
    assert torch.autograd.gradcheck(fn, ins, eps=1e-6, atol=atol, rtol=rtol, nondet_tol=0.0, fast_mode=False)


SHAPES = {9: (7, 6), 19: (5, 4, 4)}


@pytest.mark.parametrize("q", [9, 19])
def test_lbm_basic_vjps(ad, q):
    f = populations(q, SHAPES[q])
    check(ad.streaming, f)
    check(lambda x: ad.get_macroscopic(x), f)
    rho, u = (t.detach() for t in ad.get_macroscopic(f))
    check(ad.get_equilibrium, rho, u)


@pytest.mark.parametrize("q", [9, 19])
@pytest.mark.parametrize("name", ["collision_bgk", "collision_kbc", "collision_reg"])
def test_collision_vjps(ad, q, name):
    """KBC divides by <h, h>_feq, which is small where the higher-order non-equilibrium
    part h is small: its inputs keep a 20 % non-equilibrium part so that the central
    differences (step 1e-6) resolve the curvature, and its bar is 1e-4 relative."""
    kbc = name == "collision_kbc"
    f = populations(q, SHAPES[q], spread=0.2 if kbc else 0.02)
    rho, u = ad.get_macroscopic(f)
    feq = ad.get_equilibrium(rho, u).detach()
    omega = torch.tensor(1.7, dtype=DT, device="cuda")
    tol = dict(atol=1e-6, rtol=1e-4) if kbc else {}
    check(lambda a, b, w: getattr(ad, name)(a, b, w), f, feq, omega, **tol)


def test_collision_mrt_vjp(ad):
    f = populations(9, SHAPES[9])
    feq = ad.get_equilibrium(*ad.get_macroscopic(f)).detach()
    omega = torch.tensor(1.7, dtype=DT, device="cuda")
    check(lambda a, b, w: ad.collision_mrt(a, b, ad.get_mrt_collision_operator(w, 9)), f, feq, omega)


@pytest.mark.parametrize("q", [9, 19])
def test_forcing_vjps(ad, q):
    f = populations(q, SHAPES[q])
    d = 2 if q == 9 else 3
    g = rnd(d, *SHAPES[q], seed=5, scale=2e-3, shift=-1e-3)
    u = rnd(d, *SHAPES[q], seed=6, scale=0.04, shift=-0.02)
    check(ad.forcing_edm, f, g, u)
    omega = torch.tensor(1.6, dtype=DT, device="cuda")
    check(ad.forcing_guo_bgk, f, g, u, omega)


BOUNDARIES = [
    ("boundary_nee", dict(rho_wall=1.01, ux_wall=0.04, uy_wall=0.01)),
    ("boundary_nebb", dict(rho_wall=1.0, ux_wall=0.05, uy_wall=-0.01)),
    ("boundary_equilibrium", dict(rho_wall=1.0, ux_wall=0.05)),
    ("boundary_velocity_nee", dict(ux_wall=0.05, uy_wall=0.01)),
    ("boundary_velocity_nebb", dict(ux_wall=0.05)),
    ("boundary_pressure_nee", dict(rho_wall=1.0)),
    ("boundary_pressure_nebb", dict(rho_wall=1.02)),
    ("boundary_pressure_equilibrium", dict(rho_wall=0.99)),
    ("boundary_force_corrected_nebb", dict(rho_wall=1.0, ux_wall=0.05, gx_wall=1e-3, gy_wall=-2e-3)),
]


@pytest.mark.parametrize("q", [9, 19])
@pytest.mark.parametrize("name,kw", BOUNDARIES)
@pytest.mark.parametrize("loc", ["left", "right", "top"])
def test_boundary_vjps(ad, q, name, kw, loc):
    f = populations(q, SHAPES[q])
    keys = sorted(kw)
    vals = [torch.tensor(float(kw[k]), dtype=DT, device="cuda") for k in keys]
    fn = getattr(ad, name)
    check(lambda x, *w: fn(x, loc, **dict(zip(keys, w))), f, *vals)


@pytest.mark.parametrize("q", [9, 19])
@pytest.mark.parametrize("name", ["boundary_bounce_back", "boundary_specular_reflection"])
def test_bounce_back_vjps(ad, q, name):
    f = populations(q, SHAPES[q])
    pre = populations(q, SHAPES[q], seed=9)
    ux = torch.tensor(0.03, dtype=DT, device="cuda")
    check(lambda p, x, w: getattr(ad, name)(p, x, "bottom", ux_wall=w), pre, f, ux)


def _markers(m, nx, ny, seed):
    th = 2 * math.pi * np.arange(m) / m
    r = 0.25 * min(nx, ny) + 0.2 * np.sin(3 * th + seed)
    x = 0.5 * nx + 0.37 + r * np.cos(th)
    y = 0.5 * ny + 0.29 + r * np.sin(th)
    return torch.tensor(x, dtype=DT, device="cuda"), torch.tensor(y, dtype=DT, device="cuda")


def test_ib_vjps(ad):
    nx, ny, m = 24, 20, 12
    x, y = _markers(m, nx, ny, 1)
    check(lambda a, b: ad.get_ib_stencil(a, b, ny)[0], x, y)
    W, I = ad.get_ib_stencil(x, y, ny)
    W = W.detach()
    grid = rnd(2, nx, ny, seed=3, scale=0.1)
    vals = rnd(m, 2, seed=4, scale=0.1)
    check(lambda gd, w: ad.interpolate(gd, w, I), grid, W)
    check(lambda v, gd, w: ad.spread(v, gd, w, I), vals, grid, W)
    ut = rnd(m, 2, seed=5, scale=0.02)
    ds = torch.tensor(1.1, dtype=DT, device="cuda")
    check(lambda gu, w, t, s: ad.multi_direct_forcing(gu, w, I, t, s, 3), grid, W, ut, ds)
    dsm = rnd(m, seed=6, scale=0.2, shift=0.9)
    check(lambda gu, t, s: ad.multi_direct_forcing(gu, W, I, t, s, 2), grid, ut, dsm)


def test_ib_stencil_3d_vjp(ad):
    g = torch.Generator().manual_seed(7)
    X = (torch.rand(9, 3, generator=g, dtype=DT) * 4 + 5.2).cuda()
    check(lambda c: ad.get_ib_stencil_3d(c, (14, 13, 12))[0], X)


def test_newmark_vjp(ad):
    a, v, d, h = (rnd(2, seed=s, scale=1e-3) for s in range(4))
    k = torch.tensor(3e-3, dtype=DT, device="cuda")
    m = torch.tensor(800.0, dtype=DT, device="cuda")
    check(lambda a_, v_, d_, h_, m_, k_: ad.newmark(a_, v_, d_, h_, m_, k_, 0.2), a, v, d, h, m, k)


def test_torch_ops_backward(ad):
    """torch.ops.vivsim.* carry the same backward rules (tensor arguments)."""
    import vivsim_gb300.torch_ops  # noqa: F401
    f = populations(9, SHAPES[9], spread=0.2)
    feq = ad.get_equilibrium(*ad.get_macroscopic(f)).detach()
    check(lambda a: torch.ops.vivsim.streaming(a), f)
    check(lambda a, b: torch.ops.vivsim.collision_kbc(a, b, 1.7), f, feq, atol=1e-6, rtol=1e-4)
    nx, ny = SHAPES[9]
    x, y = _markers(6, nx, ny, 2)
    W, I = ad.get_ib_stencil(x, y, ny)
    grid = rnd(2, nx, ny, seed=3, scale=0.1)
    check(lambda gd, w: torch.ops.vivsim.interpolate(gd, w, I), grid, W.detach())


def test_gradients_are_deterministic(ad):
    f = populations(9, (64, 48))
    omega = torch.tensor(1.7, dtype=DT, device="cuda", requires_grad=True)
    grads = []
    for _ in range(2):
        x = f.clone().requires_grad_(True)
        rho, u = ad.get_macroscopic(x)
        out = ad.collision_kbc(x, ad.get_equilibrium(rho, u), omega)
        out = ad.boundary_pressure_nee(ad.streaming(out), "right", rho_wall=1.0)
        loss = (out * out).sum()
        gx, gw = torch.autograd.grad(loss, (x, omega))
        grads.append((gx, gw))
    assert torch.equal(grads[0][0], grads[1][0]) and torch.equal(grads[0][1], grads[1][1])


CASE = dict(nx=128, ny=64, D=10.0, Re=50.0, n_markers=32, n_steps=200, checkpoint_every=50, obj_start=100)


def composed_drag(ad, U0, K, off, case):
    """The cylinder-VIV step composed from the differentiable per-operator functions as
    examples/2d/vortex_induced_vibration.py:96-148 composes it (BGK, full-grid stencil,
    MDF 3, transverse spring, equilibrium inflow, pressure-NEE outflow), objective = mean
    x force over steps [obj_start, n_steps)."""
    nx, ny, D, Re, M = case["nx"], case["ny"], case["D"], case["Re"], case["n_markers"]
    dev = U0.device
    omega = ad.get_omega(U0 * D / Re)
    area = math.pi * (D / 2) ** 2
    mass = area * 10.0
    ds = math.pi * D / M
    th = torch.tensor(2 * np.pi * np.arange(M) / M, dtype=DT, device=dev)
    r = 0.5 * D + off
    X0 = nx / 4.0 + r * torch.cos(th)
    Y0 = ny / 2.0 + r * torch.sin(th)
    u0 = torch.stack([U0 * torch.ones(nx, ny, dtype=DT, device=dev), torch.zeros(nx, ny, dtype=DT, device=dev)])
    f = ad.get_equilibrium(torch.ones(nx, ny, dtype=DT, device=dev), u0)
    z = torch.zeros(1, dtype=DT, device=dev)
    a = v = d = torch.zeros(2, dtype=DT, device=dev)
    J = 0.0
    for step in range(case["n_steps"]):
        rho, u = ad.get_macroscopic(f)
        f = ad.collision_bgk(f, ad.get_equilibrium(rho, u), omega)
        mx, my = ad.get_markers_coords_2dof(X0, Y0, d)
        W, I = ad.get_ib_stencil(mx, my, ny)
        g, mh = ad.multi_direct_forcing(u, W, I, v[None, :].expand(M, 2), ds, 3)
        h = ad.get_force_to_obj(mh) + a * area
        ay, vy, dy = ad.newmark(a[1:], v[1:], d[1:], h[1:], mass, K, 0.0)
        a, v, d = torch.cat([z, ay]), torch.cat([z, vy]), torch.cat([z, dy])
        f = ad.forcing_edm(f, g, u)
        f = ad.streaming(f)
        f = ad.boundary_equilibrium(f, "left", ux_wall=U0)
        f = ad.boundary_pressure_nee(f, "right", rho_wall=1.0)
        if step >= case["obj_start"]:
            J = J + h[0]
    return J / (case["n_steps"] - case["obj_start"])


def test_composed_update_step_matches_fused_adjoint(ad):
    from vivsim_gb300 import adjoint
    off = np.random.default_rng(2).normal(0.0, 0.1, CASE["n_markers"])
    plan = adjoint.CylinderDrag(U0=0.05, offsets=off, dtype=DT, **CASE)
    J0 = plan.forward()
    gU0, gK, goff = plan.backward()
    K0 = plan.stiffness
    plan.close()
    U0 = torch.tensor(0.05, dtype=DT, device="cuda", requires_grad=True)
    K = torch.tensor(K0, dtype=DT, device="cuda", requires_grad=True)
    o = torch.tensor(off, dtype=DT, device="cuda", requires_grad=True)
    J = composed_drag(ad, U0, K, o, CASE)
    J.backward()
    print(f"\ncomposed vs fused adjoint: J {float(J):.15e} / {J0:.15e}; dU0 {float(U0.grad):.12e} / {gU0:.12e}; "
          f"dK {float(K.grad):.12e} / {gK:.12e}; doff {np.max(np.abs(o.grad.cpu().numpy() - goff)):.3e} "
          f"of {np.max(np.abs(goff)):.3e}")
    assert abs(float(J) - J0) <= 1e-10 * abs(J0), (float(J), J0)
    assert abs(float(U0.grad) - gU0) <= 1e-10 * abs(gU0), (float(U0.grad), gU0)
    assert abs(float(K.grad) - gK) <= 1e-10 * abs(gK), (float(K.grad), gK)
    go = o.grad.cpu().numpy()
    assert np.max(np.abs(go - goff)) <= 1e-10 * np.max(np.abs(goff)), np.max(np.abs(go - goff))
