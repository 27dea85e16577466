"""The reference's known-answer examples as regression tests of the fused step.

The reference validates itself with example scripts that compare against analytic
solutions: the Taylor-Green vortex (examples/2d/taylor_green_vortex.py), plane Couette
flow (examples/2d/couette_flow.py) and the ABC flow (examples/3d/abc_flow.py).  Here each
runs in the fused step with the example's parameters.  Its relative L2 error against the
analytic field must equal the oracle's own error for the same run to 1e-5.  Float32
rounding moves the error by far less than that.  For the 64^3 ABC run, which the NumPy
oracle would take minutes for, the kinetic energy must decay at the analytic rate.
"""

import math

import numpy as np
import pytest
import torch

from oracle import lbm2d as L2
from oracle import lbm3d as L3

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import vivsim_gb300
    vivsim_gb300.build()
    from vivsim_gb300 import solver
    return solver


def _run(S, step, f0, n):
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        sim = S.Simulation(step, torch.from_numpy(np.ascontiguousarray(f0)).cuda())
        sim.run(n, graph=True)
        torch.cuda.synchronize()
    step.check()
    return sim.f.cpu().numpy()


def _tgv(t, n=64, u0=0.02, nu=0.02):
    kx = ky = 2 * math.pi / n
    x = np.arange(n, dtype=np.float32)[:, None]
    y = np.arange(n, dtype=np.float32)[None, :]
    dec = np.exp(-nu * (kx * kx + ky * ky) * t)
    return np.stack([u0 * np.sin(kx * x) * np.cos(ky * y) * dec,
                     -u0 * np.cos(kx * x) * np.sin(ky * y) * dec]).astype(np.float32)


def test_taylor_green_vortex(S):
    """64 x 64, BGK, periodic, 4000 steps (examples/2d/taylor_green_vortex.py:19-31)."""
    n, nu, steps = 64, 0.02, 4000
    om = L2.get_omega(nu)
    f0 = L2.get_equilibrium(np.ones((n, n), np.float32), _tgv(0.0))
    f = _run(S, S.LatticeStep(9, (n, n), "bgk", om), f0, steps)
    _, u = L2.get_macroscopic(f)
    ut = _tgv(float(steps))
    err = np.linalg.norm(u - ut) / np.linalg.norm(ut)
    fo = f0
    for _ in range(steps):
        r, uo = L2.get_macroscopic(fo)
        fo = L2.streaming(L2.collision_bgk(fo, L2.get_equilibrium(r, uo), om))
    _, uo = L2.get_macroscopic(fo)
    err_o = np.linalg.norm(uo - ut) / np.linalg.norm(ut)
    assert err < 5e-3 and abs(err - err_o) < 1e-5, (err, err_o)


def test_couette_flow(S):
    """16 x 16, BGK, NEE bottom wall and moving NEE top wall, 12000 steps
    (examples/2d/couette_flow.py:21-47): the linear profile."""
    n, u0, nu, steps = 16, 0.08, 0.10, 12000
    om = L2.get_omega(nu)
    f0 = L2.get_equilibrium(np.ones((n, n), np.float32), np.zeros((2, n, n), np.float32))
    step = S.LatticeStep(9, (n, n), "bgk", om,
                         boundaries=[S.boundary("nee", "bottom"), S.boundary("nee", "top", ux_wall=u0)])
    f = _run(S, step, f0, steps)
    ut = np.broadcast_to(u0 * np.arange(n, dtype=np.float32) / (n - 1), (n, n))
    _, u = L2.get_macroscopic(f)
    err = np.linalg.norm(u[0] - ut) / np.linalg.norm(ut)
    fo = f0
    for _ in range(steps):
        r, uo = L2.get_macroscopic(fo)
        fo = L2.streaming(L2.collision_bgk(fo, L2.get_equilibrium(r, uo), om))
        fo = L2.boundary_nee(fo, "bottom")
        fo = L2.boundary_nee(fo, "top", ux_wall=u0)
    _, uo = L2.get_macroscopic(fo)
    err_o = np.linalg.norm(uo[0] - ut) / np.linalg.norm(ut)
    assert err < 1e-4 and abs(err - err_o) < 1e-5, (err, err_o)


def _abc(t, n, u0=0.02, nu=0.005):
    k = 2 * math.pi / n
    x = np.arange(n, dtype=np.float32)[:, None, None]
    y = np.arange(n, dtype=np.float32)[None, :, None]
    z = np.arange(n, dtype=np.float32)[None, None, :]
    dec = np.exp(-nu * k * k * t)
    u = [u0 * (np.sin(k * z) + np.cos(k * y)) * dec, u0 * (np.sin(k * x) + np.cos(k * z)) * dec,
         u0 * (np.sin(k * y) + np.cos(k * x)) * dec]
    return np.stack([np.broadcast_to(a, (n, n, n)) for a in u]).astype(np.float32)


def test_abc_flow_against_oracle(S):
    """D3Q19, regularised collision, periodic cube (examples/3d/abc_flow.py:21-60) at 32^3,
    300 steps: the same error against the analytic field as the oracle's run."""
    n, nu, steps = 32, 0.005, 300
    om = L3.get_omega(nu)
    f0 = L3.get_equilibrium(np.ones((n, n, n), np.float32), _abc(0.0, n))
    f = _run(S, S.LatticeStep(19, (n, n, n), "reg", om), f0, steps)
    ut = _abc(float(steps), n)
    _, u = L3.get_macroscopic(f)
    err = np.linalg.norm(u - ut) / np.linalg.norm(ut)
    fo = f0
    for _ in range(steps):
        r, uo = L3.get_macroscopic(fo)
        fo = L3.streaming(L3.collision_reg(fo, L3.get_equilibrium(r, uo), om))
    _, uo = L3.get_macroscopic(fo)
    err_o = np.linalg.norm(uo - ut) / np.linalg.norm(ut)
    assert err < 2e-2 and abs(err - err_o) < 1e-5, (err, err_o)


def test_abc_flow_energy_decay(S):
    """The example's 64^3, 2000-step run: kinetic energy decays as exp(-2 nu k^2 t) (3 %)."""
    n, nu, steps = 64, 0.005, 2000
    om = L3.get_omega(nu)
    u0 = _abc(0.0, n)
    f0 = L3.get_equilibrium(np.ones((n, n, n), np.float32), u0)
    f = _run(S, S.LatticeStep(19, (n, n, n), "reg", om), f0, steps)
    _, u = L3.get_macroscopic(f)
    ratio = float(np.sum(u.astype(np.float64) ** 2) / np.sum(u0.astype(np.float64) ** 2))
    k = 2 * math.pi / n
    exact = math.exp(-2 * nu * k * k * steps)
    assert abs(ratio / exact - 1) < 3e-2, (ratio, exact)


def test_flow_past_cylinder_force_coefficients(S):
    """examples/2d/flow_pass_cylinder.py:21-75 at its full size: D = 60 on a 30D x 20D grid,
    Re = 200, KBC, fixed immersed cylinder (240 markers, Peskin 4-point, MDF 3),
    force-corrected NEBB inflow and equilibrium outflow, 180 000 steps.  Over the second
    half the mean drag coefficient must be within 3 % of the literature value the example
    quotes (1.389), and the lift amplitude within 5 % of 0.718 (measured: 1.404 and
    0.713).  A 1e-4 transverse
    perturbation of the initial velocity starts the shedding (the example relies on
    round-off)."""
    D, U0, RE = 60, 0.05, 200
    nx, ny, cx, cy, M = 30 * D, 20 * D, 10 * D, 10 * D, 4 * D
    th = np.linspace(0, 2 * np.pi, M, endpoint=False)
    X = np.stack([cx + 0.5 * D * np.cos(th), cy + 0.5 * D * np.sin(th)], 1).astype(np.float32)
    ds = np.asarray(L2_get_ds(X), np.float64)
    om = L2.get_omega(U0 * D / RE)
    steps = int(30 * 5 / U0 * D)
    rng = np.random.default_rng(12)
    u = np.zeros((2, nx, ny), np.float32)
    u[0] = U0
    u[1] = 1e-4 * rng.standard_normal((nx, ny))
    f0 = L2.get_equilibrium(np.ones((nx, ny), np.float32), u)
    step = S.LatticeStep(9, (nx, ny), "kbc", om, forcing="edm",
                         boundaries=[S.boundary("nebb", "left", mode="force_corrected", ux_wall=U0),
                                     S.boundary("equilibrium", "right", ux_wall=U0)])
    body = S.RigidBody(step, X.astype(np.float64), ds, kernel="peskin4", n_iter=3, moving=False)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        sim = S.Simulation(step, torch.from_numpy(f0).cuda(), body)
        hist = sim.run(steps, force_history=True)
        torch.cuda.synchronize()
    step.check()
    h = hist.double().cpu().numpy()
    cd = h[steps // 2:, 0] * 2 / (D * U0 ** 2)
    cl = h[steps // 2:, 1] * 2 / (D * U0 ** 2)
    cd_mean, cl_max = float(np.mean(cd)), float(np.max(np.abs(cl)))
    print(f"Cd = {cd_mean:.4f} (1.389), max |Cl| = {cl_max:.4f} (0.718)")
    assert abs(cd_mean - 1.389) / 1.389 < 0.03, cd_mean
    assert abs(cl_max - 0.718) / 0.718 < 0.05, cl_max


def L2_get_ds(X):
    from oracle import ib as OIB
    return OIB.get_ds(X)
