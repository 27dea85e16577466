"""Fused time step (vs_step / vs_run / vs_run_graph) against the reference and the oracle.

Golden trajectories come from the reference's own functions chained as its examples do
(tests/golden/make_golden.py); larger cases compare with the oracle recipes.  Tolerance,
norm-relative per field: float32 1e-6 after one step, 1e-5 after a few steps (the fused
kernel contracts multiply-adds, the reference rounds each one); float64 1e-12.
"""

import math

import numpy as np
import pytest
import torch

from conftest import golden, rel_err
from oracle import dyn
from oracle import ib as OIB
from oracle import lbm2d as L2
from oracle import lbm3d as L3
from oracle import recipes

pytestmark = pytest.mark.gpu


def T(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def N(t):
    return t.detach().cpu().numpy()


def tol(mode, steps=1):
    if mode == "f64":
        return 1e-12
    return 1e-6 if steps <= 1 else 1e-5


@pytest.fixture(scope="module")
def S():
    import vivsim_gb300
    vivsim_gb300.build()
    from vivsim_gb300 import solver
    return solver


def test_cavity_golden(S, mode):
    G = golden(mode)
    dt = torch.float64 if mode == "f64" else torch.float32
    om = L2.get_omega(0.0256)
    bcs = [S.boundary("nee", "top", ux_wall=0.1), S.boundary("nee", "left"), S.boundary("nee", "right"),
           S.boundary("nee", "bottom")]
    step = S.LatticeStep(9, (16, 12), "bgk", om, dtype=dt, boundaries=bcs)
    sim = S.Simulation(step, T(G["cav.f0"]))
    done = 0
    for target in (1, 10, 30):
        sim.run(target - done)
        done = target
        err = rel_err(N(sim.f), G[f"cav.f{target}"])
        assert err <= tol(mode, target), (target, err)


def _viv_body(S, step, G, dt, mode):
    D, U0, M = 8.0, 0.05, 24
    area = math.pi * (D / 2) ** 2
    mass = area * 10.0
    fn = U0 / (5.0 * D)
    K = (2 * math.pi * fn) ** 2 * mass * (1 + 1 / 10.0)
    X = np.stack([G["viv.X0"], G["viv.Y0"]], axis=1)
    return S.RigidBody(step, X, math.pi * D / M, kernel="peskin4", radius=2, n_iter=3, moving=True,
                       free_dof=(False, True), mass=mass, stiffness=K, damping=0.0, added_mass_area=area)


@pytest.mark.parametrize("coll", ["kbc", "mrt", "reg", "bgk"])
def test_viv_golden(S, mode, coll):
    G = golden(mode)
    dt = torch.float64 if mode == "f64" else torch.float32
    nx, ny, U0 = 40, 24, 0.05
    om = L2.get_omega(U0 * 8.0 / 20.0)
    u = np.zeros((2, nx, ny), G["viv.X0"].dtype)
    u[0] = U0
    u[1] = G["viv.pert"]
    f0 = L2.get_equilibrium(np.ones((nx, ny), u.dtype), u)
    step = S.LatticeStep(9, (nx, ny), coll, om, dtype=dt, forcing="edm",
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=U0),
                                     S.boundary("nee", "right", mode="pressure", rho_wall=1.0)])
    body = _viv_body(S, step, G, dt, mode)
    sim = S.Simulation(step, T(f0), body)
    h1 = sim.run(1, force_history=True)
    st = body.state()
    assert rel_err(N(h1)[0, :2], G[f"viv.{coll}.h1"]) <= (1e-4 if mode == "f32" else 1e-10)
    assert rel_err(np.stack([st["a"][:2], st["v"][:2], st["d"][:2]]), G[f"viv.{coll}.body1"]) <= \
        (1e-4 if mode == "f32" else 1e-10)
    sim.run(5)
    err = rel_err(N(sim.f), G[f"viv.{coll}.f6"])
    assert err <= tol(mode, 6), err
    st = body.state()
    assert rel_err(st["h"][:2], G[f"viv.{coll}.h6"]) <= (1e-4 if mode == "f32" else 1e-9)


@pytest.mark.parametrize("coll", ["reg", "bgk", "kbc"])
def test_sphere_golden(S, mode, coll):
    G = golden(mode)
    dt = torch.float64 if mode == "f64" else torch.float32
    X = G["sph.X"]
    nx, ny, nz, D, U0, M = 16, 12, 12, 5.0, 0.05, 79
    om = L3.get_omega(U0 * D / 30.0)
    u = G["sph.pert"].copy()
    u[0] = u[0] + U0
    f0 = L3.get_equilibrium(np.ones((nx, ny, nz), X.dtype), u)
    step = S.LatticeStep(19, (nx, ny, nz), coll, om, dtype=dt, forcing="edm",
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=U0),
                                     S.boundary("nee", "right", mode="pressure", rho_wall=1.0)])
    body = S.RigidBody(step, X, 4 * math.pi * (D / 2) ** 2 / M, kernel="peskin4", n_iter=3, moving=False)
    sim = S.Simulation(step, T(f0), body)
    h = sim.run(4, force_history=True)
    assert rel_err(N(h)[0], G[f"sph.{coll}.h1"]) <= (1e-4 if mode == "f32" else 1e-9)
    assert rel_err(N(h)[3], G[f"sph.{coll}.h4"]) <= (1e-4 if mode == "f32" else 1e-9)
    err = rel_err(N(sim.f), G[f"sph.{coll}.f4"])
    assert err <= tol(mode, 4), err


def _forcing_case(S, forcing, dt):
    nx, ny = 20, 14
    gx = 1e-5
    om = L2.get_omega(0.1)
    g = np.zeros((2, nx, ny), np.float64 if dt == torch.float64 else np.float32)
    g[0] = gx
    rho = np.ones((nx, ny), g.dtype)
    u = np.zeros((2, nx, ny), g.dtype)
    f0 = L2.get_equilibrium(rho, u - g / 2)
    bcs = [S.boundary("nebb", "top", mode="force_corrected", gx_wall=gx),
           S.boundary("nebb", "bottom", mode="force_corrected", gx_wall=gx)]
    coll = "mrt" if forcing == "guo_mrt" else "bgk"
    step = S.LatticeStep(9, (nx, ny), coll, om, dtype=dt, forcing=forcing, g=(gx, 0.0), boundaries=bcs)
    obcs = [("fcnebb", "top", dict(gx_wall=gx)), ("fcnebb", "bottom", dict(gx_wall=gx))]
    return step, f0, g, om, obcs, coll


@pytest.mark.parametrize("forcing", ["edm", "guo_bgk", "guo_mrt"])
def test_body_force_recipes(S, forcing):
    """examples/2d/poiseuille_channel.py:82-143 recipes (uniform force, force-corrected NEBB)."""
    for dt in (torch.float32, torch.float64):
        step, f0, g, om, obcs, coll = _forcing_case(S, forcing, dt)
        sim = S.Simulation(step, T(f0))
        f = f0.copy()
        op = L2.get_mrt_collision_operator(om, f.dtype)
        for k in range(8):
            f = recipes.lbm_step_2d(f, coll, om, op, obcs, g=g, forcing=forcing)
        sim.run(8)
        assert rel_err(N(sim.f), f) <= (1e-5 if dt == torch.float32 else 1e-12)


def test_bounce_back_and_velocity_walls(S):
    """Fused bounce-back / specular faces and velocity-mode walls against the oracle."""
    nx, ny = 18, 16
    rng = np.random.default_rng(5)
    rho = 1 + 0.01 * rng.standard_normal((nx, ny))
    u = 0.02 * rng.standard_normal((2, nx, ny))
    f0 = L2.get_equilibrium(rho, u)
    om = 1.6
    bcs = [S.boundary("bounce_back", "top", ux_wall=0.05), S.boundary("specular_reflection", "bottom"),
           S.boundary("nebb", "left", mode="velocity", ux_wall=0.03),
           S.boundary("nee", "right", mode="pressure", rho_wall=1.0)]
    obcs = [("bb", "top", dict(ux_wall=0.05)), ("spec", "bottom", {}), ("vnebb", "left", dict(ux_wall=0.03)),
            ("pnee", "right", dict(rho_wall=1.0))]
    step = S.LatticeStep(9, (nx, ny), "kbc", om, dtype=torch.float64, boundaries=bcs)
    sim = S.Simulation(step, T(f0))
    f = f0.copy()
    for _ in range(5):
        f = recipes.lbm_step_2d(f, "kbc", om, None, obcs)
    sim.run(5)
    assert rel_err(N(sim.f), f) <= 1e-12


def test_viv_oracle_larger(S):
    """64 x 48 VIV case, KBC, 20 steps, float32, against the oracle recipe."""
    nx, ny, D, U0, M = 64, 48, 12.0, 0.05, 38
    om = L2.get_omega(U0 * D / 60.0)
    th = np.linspace(0, 2 * np.pi, M, endpoint=False)
    X0 = (20.0 + 0.5 * D * np.cos(th)).astype(np.float32)
    Y0 = (24.0 + 0.5 * D * np.sin(th)).astype(np.float32)
    rng = np.random.default_rng(0)
    u = np.zeros((2, nx, ny), np.float32)
    u[0] = U0
    u[1] = 1e-4 * rng.standard_normal((nx, ny))
    f0 = L2.get_equilibrium(np.ones((nx, ny), np.float32), u)
    area = math.pi * (D / 2) ** 2
    mass = 10 * area
    K = (2 * math.pi * U0 / (5 * D)) ** 2 * mass * 1.1
    ds = math.pi * D / M
    bcs = [("eq", "left", dict(ux_wall=U0)), ("pnee", "right", dict(rho_wall=1.0))]
    body_o = recipes.Body2D(X0, Y0, ds, mass, K, 0.0, area, free=(False, True), n_iter=3,
                            v=np.array([0, 1e-3], np.float32))
    step = S.LatticeStep(9, (nx, ny), "kbc", om, forcing="edm",
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=U0),
                                     S.boundary("nee", "right", mode="pressure", rho_wall=1.0)])
    body = S.RigidBody(step, np.stack([X0, Y0], 1), ds, moving=True, free_dof=(False, True), mass=mass,
                       stiffness=K, added_mass_area=area, v0=(0, 1e-3, 0))
    sim = S.Simulation(step, T(f0), body)
    f = f0
    for _ in range(20):
        f, h = recipes.ib_lbm_step_2d(f, body_o, "kbc", om, None, bcs)
    sim.run(20)
    assert rel_err(N(sim.f), f) <= 1e-5
    st = body.state()
    assert rel_err(st["d"][:2], body_o.d) <= 1e-4
    # h sums 38 marker forces of both signs (in a fixed tree on the GPU, serially in the
    # oracle); float32 rounding of u near the markers accumulates into it over 20 steps
    assert rel_err(st["h"][:2], h) <= 3e-4


def _chain_width(X, R=2):
    """Cyclic index distance bound of a rigid marker set (the plan's chain check)."""
    M, K = len(X), 0
    for i in range(M):
        for j in range(i + 1, M):
            if abs(X[i, 0] - X[j, 0]) < 2 * R + 1e-3 and abs(X[i, 1] - X[j, 1]) < 2 * R + 1e-3:
                K = max(K, min(j - i, M - (j - i)))
    return K


def _viv_small(S, X, steps, graph=False):
    nx, ny = 96, 64
    rng = np.random.default_rng(3)
    u = np.zeros((2, nx, ny), np.float32)
    u[0] = 0.05
    u[1] = 1e-3 * rng.standard_normal((nx, ny))
    f0 = T(L2.get_equilibrium(np.ones((nx, ny), np.float32), u))
    step = S.LatticeStep(9, (nx, ny), "kbc", 1.8, forcing="edm",
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=0.05),
                                     S.boundary("nee", "right", mode="pressure")])
    body = S.RigidBody(step, X, 0.94, moving=True, free_dof=(False, True), mass=500.0, stiffness=0.05,
                       added_mass_area=113.0, v0=(0, 2e-3, 0))
    sim = S.Simulation(step, f0, body)
    hist = sim.run(steps, graph=graph, force_history=True)
    return N(sim.f), body.state(), N(hist)


@pytest.mark.parametrize("form", ["single", "general"])
def test_viv_fsi_subiterations_golden(S, mode, form, monkeypatch):
    """FSI_ITER = 2 (examples/2d/vortex_induced_vibration.py:111-139) against the reference's
    golden trajectory, in the chain and the general form of the body kernel (sub-iterations
    run without the cluster form)."""
    monkeypatch.setenv("VIVSIM_GB300_BODY_SINGLE" if form == "single" else "VIVSIM_GB300_BODY_CSR", "1")
    G = golden(mode)
    dt = torch.float64 if mode == "f64" else torch.float32
    nx, ny, U0, D, M = 40, 24, 0.05, 8.0, 24
    om = L2.get_omega(U0 * D / 20.0)
    u = np.zeros((2, nx, ny), G["viv.X0"].dtype)
    u[0] = U0
    u[1] = G["viv.pert"]
    f0 = L2.get_equilibrium(np.ones((nx, ny), u.dtype), u)
    step = S.LatticeStep(9, (nx, ny), "kbc", om, dtype=dt, forcing="edm",
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=U0),
                                     S.boundary("nee", "right", mode="pressure", rho_wall=1.0)])
    area = math.pi * (D / 2) ** 2
    mass = area * 10.0
    K = (2 * math.pi * U0 / (5.0 * D)) ** 2 * mass * (1 + 1 / 10.0)
    X = np.stack([G["viv.X0"], G["viv.Y0"]], axis=1)
    body = S.RigidBody(step, X, math.pi * D / M, n_iter=3, moving=True, free_dof=(True, True), mass=mass,
                       stiffness=K, added_mass_area=area, v0=(0.0, 1e-2 * U0, 0.0), fsi_iter=2)
    sim = S.Simulation(step, T(f0), body)
    btol = 1e-4 if mode == "f32" else 1e-10
    h1 = sim.run(1, force_history=True)
    st = body.state()
    assert rel_err(N(sim.f), G["vivfsi.f1"]) <= tol(mode, 1)
    assert rel_err(N(h1)[0, :2], G["vivfsi.h1"]) <= btol
    assert rel_err(np.stack([st["a"][:2], st["v"][:2], st["d"][:2]]), G["vivfsi.body1"]) <= btol
    sim.run(5)
    st = body.state()
    assert rel_err(N(sim.f), G["vivfsi.f6"]) <= tol(mode, 6)
    assert rel_err(st["h"][:2], G["vivfsi.h6"]) <= btol
    assert rel_err(np.stack([st["a"][:2], st["v"][:2], st["d"][:2]]), G["vivfsi.body6"]) <= btol


def test_body_chain_form_equals_general_form(S, monkeypatch):
    """The body kernel's cluster form, its single-CTA chain form (neighbour search by marker
    index) and the general form (shared-memory sort) sum every node in the same order:
    identical bits over 30 moving steps."""
    th = np.linspace(0, 2 * np.pi, 40, endpoint=False)
    X = np.stack([30 + 6 * np.cos(th), 32 + 6 * np.sin(th)], 1).astype(np.float32).astype(np.float64)
    assert 2 * _chain_width(X) + 1 <= 31  # the chain form applies to this marker set
    fa, sa, ha = _viv_small(S, X, 30)  # cluster form (body + box in one launch)
    for env in ("VIVSIM_GB300_BODY_SINGLE", "VIVSIM_GB300_BODY_CSR"):
        monkeypatch.setenv(env, "1")
        fb, sb, hb = _viv_small(S, X, 30)
        monkeypatch.delenv(env)
        assert np.array_equal(fa, fb), env
        assert np.array_equal(ha, hb), env
        for k in ("a", "v", "d", "h"):
            assert np.array_equal(sa[k], sb[k]), (env, k)
    # and through graph replay
    with torch.cuda.stream(torch.cuda.Stream()):
        fg, sg, hg = _viv_small(S, X, 30, graph=True)
        torch.cuda.synchronize()
    assert np.array_equal(fa, fg)


def test_viv_shuffled_markers_general_form(S):
    """Markers in random order (no chain bound: the general body kernel) against the oracle."""
    nx, ny, D, U0, M = 64, 48, 12.0, 0.05, 38
    om = L2.get_omega(U0 * D / 60.0)
    th = np.linspace(0, 2 * np.pi, M, endpoint=False)
    perm = np.random.default_rng(5).permutation(M)
    X0 = (20.0 + 0.5 * D * np.cos(th)).astype(np.float32)[perm]
    Y0 = (24.0 + 0.5 * D * np.sin(th)).astype(np.float32)[perm]
    assert 2 * _chain_width(np.stack([X0, Y0], 1).astype(np.float64)) + 1 > 31
    rng = np.random.default_rng(0)
    u = np.zeros((2, nx, ny), np.float32)
    u[0] = U0
    u[1] = 1e-4 * rng.standard_normal((nx, ny))
    f0 = L2.get_equilibrium(np.ones((nx, ny), np.float32), u)
    area = math.pi * (D / 2) ** 2
    mass = 10 * area
    K = (2 * math.pi * U0 / (5 * D)) ** 2 * mass * 1.1
    ds = math.pi * D / M
    bcs = [("eq", "left", dict(ux_wall=U0)), ("pnee", "right", dict(rho_wall=1.0))]
    body_o = recipes.Body2D(X0, Y0, ds, mass, K, 0.0, area, free=(False, True), n_iter=3,
                            v=np.array([0, 1e-3], np.float32))
    step = S.LatticeStep(9, (nx, ny), "kbc", om, forcing="edm",
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=U0),
                                     S.boundary("nee", "right", mode="pressure", rho_wall=1.0)])
    body = S.RigidBody(step, np.stack([X0, Y0], 1), ds, moving=True, free_dof=(False, True), mass=mass,
                       stiffness=K, added_mass_area=area, v0=(0, 1e-3, 0))
    sim = S.Simulation(step, T(f0), body)
    f = f0
    for _ in range(10):
        f, h = recipes.ib_lbm_step_2d(f, body_o, "kbc", om, None, bcs)
    sim.run(10)
    assert rel_err(N(sim.f), f) <= 1e-5
    st = body.state()
    assert rel_err(st["d"][:2], body_o.d) <= 1e-4
    assert rel_err(st["h"][:2], h) <= 3e-4


def test_graph_replay_matches_eager_and_is_deterministic(S):
    nx, ny = 96, 64
    rng = np.random.default_rng(3)
    u = np.zeros((2, nx, ny), np.float32)
    u[0] = 0.05
    u[1] = 1e-3 * rng.standard_normal((nx, ny))
    f0 = T(L2.get_equilibrium(np.ones((nx, ny), np.float32), u))
    th = np.linspace(0, 2 * np.pi, 40, endpoint=False)
    X = np.stack([30 + 6 * np.cos(th), 32 + 6 * np.sin(th)], 1)

    def make():
        step = S.LatticeStep(9, (nx, ny), "kbc", 1.8, forcing="edm",
                             boundaries=[S.boundary("equilibrium", "left", ux_wall=0.05),
                                         S.boundary("nee", "right", mode="pressure")])
        body = S.RigidBody(step, X, 0.94, moving=True, free_dof=(False, True), mass=500.0, stiffness=0.05,
                           added_mass_area=113.0)
        return S.Simulation(step, f0, body), body

    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        a, ba = make()
        a.run(25)
        b, bb = make()
        b.run(25, graph=True)
        c, bc = make()
        c.run(25, graph=True)
    torch.cuda.synchronize()
    assert torch.equal(a.f, b.f)
    assert torch.equal(b.f, c.f)
    assert np.array_equal(ba.state()["d"], bb.state()["d"])


def test_sphere_oracle_larger(S):
    """32 x 24 x 24 D3Q19 regularised sphere, 3 steps, float32, against the oracle recipe."""
    nx, ny, nz, D, U0 = 32, 24, 24, 8.0, 0.05
    M = 201
    X = recipes.fibonacci_sphere(M, D / 2, (12.3, 11.8, 12.1)).astype(np.float32)
    om = L3.get_omega(U0 * D / 50.0)
    rng = np.random.default_rng(1)
    u = (1e-4 * rng.standard_normal((3, nx, ny, nz))).astype(np.float32)
    u[0] += U0
    f0 = L3.get_equilibrium(np.ones((nx, ny, nz), np.float32), u)
    ds = 4 * math.pi * (D / 2) ** 2 / M
    W, I = OIB.get_ib_stencil_3d(X, (nx, ny, nz))
    bcs = [("eq", "left", dict(ux_wall=U0)), ("pnee", "right", dict(rho_wall=1.0))]
    f = f0
    for _ in range(3):
        f, h = recipes.ib_lbm_step_3d(f, W, I, np.zeros((M, 3), np.float32), ds, "reg", om, None, bcs)
    step = S.LatticeStep(19, (nx, ny, nz), "reg", om, forcing="edm",
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=U0),
                                     S.boundary("nee", "right", mode="pressure", rho_wall=1.0)])
    body = S.RigidBody(step, X, ds, moving=False)
    sim = S.Simulation(step, T(f0), body)
    hist = sim.run(3, force_history=True)
    assert rel_err(N(sim.f), f) <= 1e-5
    assert rel_err(N(hist)[2], h) <= 1e-4


@pytest.mark.parametrize("dt", ["f32", "f64"])
def test_obstacle_mask_matches_oracle(S, dt):
    """Flow around masked obstacle cells (examples/2d/flow_through_text.py:71-78): KBC,
    streaming, NEE bottom and equilibrium top with uy = U0, obstacle bounce-back."""
    npdt = np.float32 if dt == "f32" else np.float64
    tdt = torch.float32 if dt == "f32" else torch.float64
    nx, ny, U0 = 48, 40, 0.05
    rng = np.random.default_rng(11)
    mask = np.zeros((nx, ny), bool)
    for cx, cy, r in ((15, 20, 4), (30, 12, 3), (33, 27, 5)):
        xx, yy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        mask |= (xx - cx) ** 2 + (yy - cy) ** 2 < r * r
    u = np.zeros((2, nx, ny), npdt)
    u[1] = U0
    u[0] = 1e-3 * rng.standard_normal((nx, ny))
    f0 = L2.get_equilibrium(np.ones((nx, ny), npdt), u).astype(npdt)
    om = npdt(1.8)
    f = f0
    for _ in range(30):
        rho, uu = L2.get_macroscopic(f)
        f = L2.collision_kbc(f, L2.get_equilibrium(rho, uu), om)
        f = L2.streaming(f)
        f = L2.boundary_nee(f, "bottom", uy_wall=U0)
        f = L2.boundary_equilibrium(f, "top", uy_wall=U0)
        f = L2.obstacle_bounce_back(f, mask)
    tol = 2e-5 if dt == "f32" else 1e-11
    mk = torch.from_numpy(mask).cuda()
    for how in ("run", "graph", "steps"):
        step = S.LatticeStep(9, (nx, ny), "kbc", float(om), dtype=tdt, obstacle_mask=mk,
                             boundaries=[S.boundary("nee", "bottom", uy_wall=U0),
                                         S.boundary("equilibrium", "top", uy_wall=U0)])
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            sim = S.Simulation(step, T(f0), None)
            if how == "steps":
                for _ in range(30):
                    sim.run(1)
            else:
                sim.run(30, graph=how == "graph")
            torch.cuda.synchronize()
        assert rel_err(N(sim.f), f) <= tol, how


def _sphere_run(S, moving, graph, steps=6):
    nx, ny, nz, D, U0 = 40, 32, 32, 10.0, 0.05
    M = 301
    X = recipes.fibonacci_sphere(M, D / 2, (14.3, 15.8, 16.1)).astype(np.float32).astype(np.float64)
    om = L3.get_omega(U0 * D / 50.0)
    rng = np.random.default_rng(7)
    u = (1e-4 * rng.standard_normal((3, nx, ny, nz))).astype(np.float32)
    u[0] += U0
    f0 = L3.get_equilibrium(np.ones((nx, ny, nz), np.float32), u)
    ds = 4 * math.pi * (D / 2) ** 2 / M
    step = S.LatticeStep(19, (nx, ny, nz), "reg", om, forcing="edm",
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=U0),
                                     S.boundary("nee", "right", mode="pressure", rho_wall=1.0)])
    if moving:
        vol = 4 / 3 * math.pi * (D / 2) ** 3
        body = S.RigidBody(step, X, ds, moving=True, free_dof=(True, True, False), mass=2 * vol, stiffness=0.05,
                           added_mass_area=vol, v0=(0, 2e-3, 0))
    else:
        body = S.RigidBody(step, X, ds, moving=False)
    with torch.cuda.stream(torch.cuda.Stream()):
        sim = S.Simulation(step, T(f0), body)
        hist = sim.run(steps, force_history=True, graph=graph)
        torch.cuda.synchronize()
    step.check()
    return N(sim.f), N(hist), body.state()


@pytest.mark.parametrize("moving", [False, True])
def test_sphere_fused_body_kernel_equals_phase_kernels(S, moving, monkeypatch):
    """The 3-D body step as one thread-block cluster (fixed bodies; 2 to 16 CTAs), as one
    cooperative launch (any number of CTAs) and as seven per-phase launches sums every
    marker and node in the same order: identical bits, eager and in graph replay, for a
    fixed and a moving sphere."""
    monkeypatch.setenv("VIVSIM_GB300_BODY3D_CLUSTER", "0")
    monkeypatch.setenv("VIVSIM_GB300_BODY3D_CTAS", "0")
    fa, ha, sa = _sphere_run(S, moving, False)
    variants = [("0", "7"), ("0", "64"), ("0", None)]
    if not moving:
        variants += [("2", None), ("8", None), (None, None)]
    for cluster, ctas in variants:
        for name, val in (("VIVSIM_GB300_BODY3D_CLUSTER", cluster), ("VIVSIM_GB300_BODY3D_CTAS", ctas)):
            if val is None:
                monkeypatch.delenv(name, raising=False)
            else:
                monkeypatch.setenv(name, val)
        for graph in (False, True):
            fb, hb, sb = _sphere_run(S, moving, graph)
            assert np.array_equal(fa, fb), (cluster, ctas, graph)
            assert np.array_equal(ha, hb), (cluster, ctas, graph)
            for k in ("a", "v", "d", "h"):
                assert np.array_equal(sa[k], sb[k]), (cluster, ctas, graph, k)


@pytest.mark.parametrize("dt", ["f32", "f64"])
def test_moving_sphere_3d_matches_oracle(S, dt):
    """A spring-mounted sphere moving through a D3Q19 channel (the 3-D moving-body step of
    examples/3d/oscillating_cylinder.py:228-283 with a sphere): markers follow the body, the
    stencil and its CSR are rebuilt every step; Newmark on y (and x), added mass."""
    npdt = np.float32 if dt == "f32" else np.float64
    tdt = torch.float32 if dt == "f32" else torch.float64
    nx, ny, nz, D, U0 = 32, 28, 24, 6.0, 0.05
    M = 113
    X = recipes.fibonacci_sphere(M, D / 2, (11.3, 13.8, 12.1)).astype(np.float32).astype(npdt)
    om = L3.get_omega(U0 * D / 50.0)
    rng = np.random.default_rng(5)
    u = (1e-4 * rng.standard_normal((3, nx, ny, nz))).astype(npdt)
    u[0] += U0
    f = L3.get_equilibrium(np.ones((nx, ny, nz), npdt), u).astype(npdt)
    f0 = f.copy()
    ds = 4 * math.pi * (D / 2) ** 2 / M
    vol = 4 / 3 * math.pi * (D / 2) ** 3
    mass, K = 2 * vol, 0.05
    free = (True, True, False)
    a, v, d = np.zeros(3, npdt), np.array([0, 2e-3, 0], npdt), np.zeros(3, npdt)
    bcs = [("eq", "left", dict(ux_wall=U0)), ("pnee", "right", dict(rho_wall=1.0))]
    dsv = npdt(ds)
    for _ in range(8):
        rho, uu = L3.get_macroscopic(f)
        f = L3.collision_reg(f, L3.get_equilibrium(rho, uu), npdt(om))
        W, I = OIB.get_ib_stencil_3d(X + d, (nx, ny, nz))
        g, mh = OIB.multi_direct_forcing(uu, W, I, np.repeat(v[None, :], M, axis=0), dsv, 3)
        h = mh[0].copy()
        for i in range(1, M):
            h = h + mh[i]
        h = h + a * npdt(vol)
        an, vn, dn = a.copy(), v.copy(), d.copy()
        for k in range(3):
            if free[k]:
                an[k], vn[k], dn[k] = dyn.newmark(a[k], v[k], d[k], h[k], mass, K, 0.0)
        a, v, d = an, vn, dn
        f = L3.forcing_edm(f, g, uu)
        f_post = f
        f = L3.streaming(f)
        f = recipes._apply_bcs(L3, recipes._BC3, f_post, f, bcs)
    step = S.LatticeStep(19, (nx, ny, nz), "reg", om, dtype=tdt, forcing="edm",
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=U0),
                                     S.boundary("nee", "right", mode="pressure", rho_wall=1.0)])
    body = S.RigidBody(step, X, ds, moving=True, free_dof=free, mass=mass, stiffness=K, added_mass_area=vol,
                       v0=(0, 2e-3, 0))
    sim = S.Simulation(step, T(f0), body)
    sim.run(8)
    st = body.state()
    tol = 2e-5 if dt == "f32" else 1e-10
    assert rel_err(N(sim.f), f) <= tol
    assert rel_err(st["d"], d) <= (1e-4 if dt == "f32" else 1e-9)
    step.check()


@pytest.mark.parametrize("scheme", ["nee", "eq", "nebb"])
def test_characteristic_outflow_golden(S, mode, scheme):
    """Outflow wall state from boundary_characteristic of the step's input moments, imposed
    by NEE / equilibrium / NEBB, against the reference's functions chained the same way."""
    G = golden(mode)
    dt = torch.float64 if mode == "f64" else torch.float32
    om, u0 = (float(x) for x in G["cbc2.omega"])
    kind = {"nee": "nee", "eq": "equilibrium", "nebb": "nebb"}[scheme]
    bcs = [S.boundary("equilibrium", "left", ux_wall=u0), S.boundary(kind, "right", mode="characteristic")]
    for graph in (False, True):
        step = S.LatticeStep(9, (24, 16), "kbc", om, dtype=dt, boundaries=bcs)
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            sim = S.Simulation(step, T(G["cbc2.f0"]))
            sim.run(1, graph=graph)
            f1 = N(sim.f)
            sim.run(7, graph=graph)
            torch.cuda.synchronize()
        assert rel_err(f1, G[f"cbc2.{scheme}.f1"]) <= tol(mode, 1), graph
        assert rel_err(N(sim.f), G[f"cbc2.{scheme}.f8"]) <= tol(mode, 8), graph


def test_characteristic_outflow_golden_3d(S, mode):
    G = golden(mode)
    dt = torch.float64 if mode == "f64" else torch.float32
    om, u0 = (float(x) for x in G["cbc2.omega"])
    step = S.LatticeStep(19, (12, 8, 8), "bgk", om, dtype=dt,
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=u0),
                                     S.boundary("nee", "right", mode="characteristic")])
    sim = S.Simulation(step, T(G["cbc3.f0"]))
    sim.run(1)
    assert rel_err(N(sim.f), G["cbc3.f1"]) <= tol(mode, 1)
    sim.run(3)
    assert rel_err(N(sim.f), G["cbc3.f4"]) <= tol(mode, 4)


@pytest.mark.parametrize("graph", [False, True])
def test_viv_characteristic_outflow_matches_oracle(S, graph):
    """The 64 x 48 VIV case with a characteristic NEE outflow instead of the pressure NEE:
    the moving body's kernels and the outflow's moments kernel share the step."""
    nx, ny, D, U0, M = 64, 48, 12.0, 0.05, 38
    om = L2.get_omega(U0 * D / 60.0)
    th = np.linspace(0, 2 * np.pi, M, endpoint=False)
    X0 = (20.0 + 0.5 * D * np.cos(th)).astype(np.float32)
    Y0 = (24.0 + 0.5 * D * np.sin(th)).astype(np.float32)
    rng = np.random.default_rng(5)
    u = np.zeros((2, nx, ny), np.float32)
    u[0] = U0
    u[1] = 1e-4 * rng.standard_normal((nx, ny))
    f0 = L2.get_equilibrium(np.ones((nx, ny), np.float32), u)
    area = math.pi * (D / 2) ** 2
    mass = 10 * area
    K = (2 * math.pi * U0 / (5 * D)) ** 2 * mass * 1.1
    ds = math.pi * D / M
    bcs = [("eq", "left", dict(ux_wall=U0)), ("cbc", "right", dict(scheme="nee"))]
    body_o = recipes.Body2D(X0, Y0, ds, mass, K, 0.0, area, free=(False, True), n_iter=3,
                            v=np.array([0, 1e-3], np.float32))
    step = S.LatticeStep(9, (nx, ny), "kbc", om, forcing="edm",
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=U0),
                                     S.boundary("nee", "right", mode="characteristic")])
    body = S.RigidBody(step, np.stack([X0, Y0], 1), ds, moving=True, free_dof=(False, True), mass=mass,
                       stiffness=K, added_mass_area=area, v0=(0, 1e-3, 0))
    f = f0
    for _ in range(20):
        f, h = recipes.ib_lbm_step_2d(f, body_o, "kbc", om, None, bcs)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        sim = S.Simulation(step, T(f0), body)
        sim.run(20, graph=graph)
        torch.cuda.synchronize()
    assert rel_err(N(sim.f), f) <= 1e-5
    st = body.state()
    assert rel_err(st["d"][:2], body_o.d) <= 1e-4
    assert rel_err(st["h"][:2], h) <= 3e-4


def _rotating_ellipse(S, npdt, steps, graph=False):
    """Ellipse (semi-axes 8 and 4) free to move in y and to turn against a torsional spring,
    KBC, equilibrium inflow, pressure-NEE outflow; fused run and oracle run."""
    tdt = torch.float32 if npdt == np.float32 else torch.float64
    nx, ny, U0, M = 64, 48, 0.05, 40
    om = L2.get_omega(U0 * 16.0 / 60.0)
    th = np.linspace(0, 2 * np.pi, M, endpoint=False)
    X0 = (24.0 + 8.0 * np.cos(th)).astype(npdt)
    Y0 = (24.0 + 4.0 * np.sin(th)).astype(npdt)
    rng = np.random.default_rng(8)
    u = np.zeros((2, nx, ny), npdt)
    u[0] = U0
    u[1] = 1e-4 * rng.standard_normal((nx, ny))
    f0 = L2.get_equilibrium(np.ones((nx, ny), npdt), u).astype(npdt)
    area = math.pi * 8 * 4
    mass = 10 * area
    inertia = mass * (64 + 16) / 4
    K = (2 * math.pi * U0 / 80) ** 2 * mass
    Kr = (2 * math.pi * U0 / 60) ** 2 * inertia
    ds = 1.2
    bcs = [("eq", "left", dict(ux_wall=U0)), ("pnee", "right", dict(rho_wall=1.0))]
    body_o = recipes.Body2D(X0, Y0, ds, mass, K, 0.0, area, free=(False, True, True), n_iter=3,
                            v=np.array([0, 1e-3, 2e-3], npdt), center=(24.0, 24.0), inertia=inertia, rot_k=Kr,
                            rot_c=0.0, rot_added=0.5 * inertia)
    f = f0
    hist_o = []
    for _ in range(steps):
        f, h = recipes.ib_lbm_step_2d(f, body_o, "kbc", om, None, bcs)
        hist_o.append(h)
    step = S.LatticeStep(9, (nx, ny), "kbc", om, dtype=tdt, forcing="edm",
                         boundaries=[S.boundary("equilibrium", "left", ux_wall=U0),
                                     S.boundary("nee", "right", mode="pressure", rho_wall=1.0)])
    body = S.RigidBody(step, np.stack([X0, Y0], 1), ds, moving=True, free_dof=(False, True, True), mass=mass,
                       stiffness=K, added_mass_area=area, v0=(0, 1e-3, 2e-3), center=(24.0, 24.0),
                       inertia=inertia, rot_stiffness=Kr, added_inertia=0.5 * inertia)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        sim = S.Simulation(step, T(f0), body)
        hist = sim.run(steps, graph=graph, force_history=True)
        torch.cuda.synchronize()
    return (N(sim.f), body.state(), N(hist)), (f, body_o, np.array(hist_o))


@pytest.mark.parametrize("dt", ["f32", "f64"])
def test_rotating_body_matches_oracle(S, dt, monkeypatch):
    """A body with a free rotation (get_markers_coords_3dof / get_markers_velocity_3dof /
    get_torque_to_obj) in the fused step against the oracle, in each body-kernel form; the
    three forms give identical bits."""
    npdt = np.float32 if dt == "f32" else np.float64
    tf, tst, th = (1e-5, 1e-4, 1e-3) if dt == "f32" else (1e-11, 1e-10, 1e-9)
    runs = {}
    for form, env in (("cluster", None), ("single", "VIVSIM_GB300_BODY_SINGLE"), ("general", "VIVSIM_GB300_BODY_CSR")):
        if env:
            monkeypatch.setenv(env, "1")
        (fg, st, hist), (fo, body_o, hist_o) = _rotating_ellipse(S, npdt, 20)
        if env:
            monkeypatch.delenv(env)
        assert rel_err(fg, fo) <= tf, form
        assert rel_err(st["d"], body_o.d) <= tst, form
        assert abs(st["d"][2]) > 1e-3, "the body must have turned"
        assert rel_err(hist, hist_o) <= th, form
        runs[form] = (fg, hist)
    for form in ("single", "general"):
        assert np.array_equal(runs["cluster"][0], runs[form][0]), form
        assert np.array_equal(runs["cluster"][1], runs[form][1]), form
    (fgr, _, _), _ = _rotating_ellipse(S, npdt, 20, graph=True)
    assert np.array_equal(runs["cluster"][0], fgr)


def test_watchdog_reports_nonfinite_populations(S):
    """A NaN planted in the input populations (a host-side fault) reaches the plan's status
    word through the watchdog scan; a clean run reports nothing."""
    from vivsim_gb300 import _lib as V
    nx, ny = 64, 48
    u = np.zeros((2, nx, ny), np.float32)
    u[0] = 0.05
    f0 = L2.get_equilibrium(np.ones((nx, ny), np.float32), u)
    bad = f0.copy()
    bad[3, 10, 20] = np.nan
    for graph in (False, True):
        step = S.LatticeStep(9, (nx, ny), "bgk", 1.5, watchdog_every=5,
                             boundaries=[S.boundary("equilibrium", "left", ux_wall=0.05)])
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            S.Simulation(step, T(f0)).run(12, graph=graph)
            step.check()  # clean
            S.Simulation(step, T(bad)).run(12, graph=graph)
            with pytest.raises(V.VivsimError) as err:
                step.check()
            assert err.value.status == V.VS_ERR_NONFINITE
            step.check()  # the status word was reset
    t = torch.ones(1000, device="cuda", dtype=torch.float64)
    assert S.check_finite(t)
    t[777] = float("inf")
    assert not S.check_finite(t)


def test_checkpoint_resume_is_bit_exact(S, tmp_path):
    """save() after 12 steps, load() into a fresh plan, 18 more steps: the same bits as 30
    uninterrupted steps (moving body, cluster form, lazy faces)."""
    th = np.linspace(0, 2 * np.pi, 40, endpoint=False)
    X = np.stack([30 + 6 * np.cos(th), 32 + 6 * np.sin(th)], 1)
    fa, sa, _ = _viv_small(S, X, 30)
    nx, ny = 96, 64
    rng = np.random.default_rng(3)
    u = np.zeros((2, nx, ny), np.float32)
    u[0] = 0.05
    u[1] = 1e-3 * rng.standard_normal((nx, ny))
    f0 = T(L2.get_equilibrium(np.ones((nx, ny), np.float32), u))

    def make():
        step = S.LatticeStep(9, (nx, ny), "kbc", 1.8, forcing="edm",
                             boundaries=[S.boundary("equilibrium", "left", ux_wall=0.05),
                                         S.boundary("nee", "right", mode="pressure")])
        body = S.RigidBody(step, X, 0.94, moving=True, free_dof=(False, True), mass=500.0, stiffness=0.05,
                           added_mass_area=113.0, v0=(0, 2e-3, 0))
        return step, body

    step, body = make()
    sim = S.Simulation(step, f0, body)
    sim.run(12)
    sim.save(tmp_path / "ck.npz")
    step2, body2 = make()
    sim2 = S.Simulation(step2, torch.zeros_like(f0), body2)
    sim2.load(tmp_path / "ck.npz")
    sim2.run(18)
    assert np.array_equal(N(sim2.f), fa)
    st = body2.state()
    for k in ("a", "v", "d"):
        assert np.array_equal(st[k], sa[k]), k


def test_bounded_wait_reports_timeout(S):
    """A bounded device wait on a barrier that nothing completes gives up and reports
    VS_ERR_TIMEOUT; the context stays usable for the next launches."""
    from vivsim_gb300 import _lib as V
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    V.call("vs_selftest_bounded_wait", 4096, V.ptr(status), V.stream())
    assert int(status.item()) == V.VS_ERR_TIMEOUT
    t = torch.ones(64, device="cuda")
    assert S.check_finite(t)


def _viv_case_run(S, case_kw, chunks, watchdog=0, graph=False):
    """The benchmark VIV configuration (vivsim_gb300.configs.viv2d with case_kw), run as
    consecutive vs_run calls of the given lengths; populations, body state and forces."""
    from vivsim_gb300 import configs
    case = configs.viv2d(**case_kw)
    bcs = [S.boundary(k, loc, mode=m, **kw) for (k, loc, m, kw) in case["boundaries"]]
    step = S.LatticeStep(9, case["shape"], case["collision"], case["omega"], forcing="edm", boundaries=bcs,
                         watchdog_every=watchdog)
    b = case["body"]
    body = S.RigidBody(step, b["markers"], b["ds"], moving=True, free_dof=b["free_dof"], mass=b["mass"],
                       stiffness=b["stiffness"], added_mass_area=b["added_mass_area"])
    sim = S.Simulation(step, T(case["f0"]), body)
    persistent = sim.persistent(max(chunks))
    hists = []
    with torch.cuda.stream(torch.cuda.Stream()):
        for n in chunks:
            hists.append(N(sim.run(n, graph=graph, force_history=True)))
        torch.cuda.synchronize()
    step.check()
    return N(sim.f), body.state(), np.concatenate(hists), persistent


@pytest.mark.parametrize("collision", ["kbc", "bgk", "mrt", "reg"])
def test_persistent_run_equals_step_launches(S, monkeypatch, collision):
    """The persistent run (one cooperative launch: the body's cluster beside groups of grid
    tiles, a barrier per step) and the launch-per-step form give identical bits on the
    benchmark VIV case, over runs of odd and even lengths in a row (prediction slots and
    deferred boundaries carried across calls)."""
    kw = dict(nx=256, ny=128, D=20.0, center=(64.0, 64.0), n_markers=63, collision=collision)
    chunks = [7, 12, 1, 30]
    monkeypatch.setenv("VIVSIM_GB300_RUN_FORM", "persistent")
    fa, sa, ha, pa = _viv_case_run(S, kw, chunks)
    monkeypatch.delenv("VIVSIM_GB300_RUN_FORM")
    fb, sb, hb, pb = _viv_case_run(S, kw, chunks)
    assert pa and not pb
    assert np.array_equal(fa, fb)
    assert np.array_equal(ha, hb)
    for k in ("a", "v", "d", "h"):
        assert np.array_equal(sa[k], sb[k]), k


def test_persistent_run_full_size_and_watchdog(S, monkeypatch):
    """At the benchmark size (1024 x 512, 126 markers) with the watchdog splitting the run
    into launches of 9 steps, and through vs_run_graph: identical bits to the per-step form."""
    monkeypatch.setenv("VIVSIM_GB300_RUN_FORM", "persistent")
    fa, sa, ha, pa = _viv_case_run(S, {}, [40, 25], watchdog=9)
    fg, sg, hg, pg = _viv_case_run(S, {}, [40, 25], graph=True)
    monkeypatch.delenv("VIVSIM_GB300_RUN_FORM")
    fb, sb, hb, pb = _viv_case_run(S, {}, [40, 25])
    assert pa and pg and not pb
    for f, h, s in ((fa, ha, sa), (fg, hg, sg)):
        assert np.array_equal(f, fb)
        assert np.array_equal(h, hb)
        for k in ("a", "v", "d", "h"):
            assert np.array_equal(s[k], sb[k]), k


def test_run_form_tuner(S):
    """Simulation.tune times the run forms that apply (launches per step; the persistent
    run) and keeps the faster; runs then give the same bits whichever it chose."""
    from vivsim_gb300 import configs
    kw = dict(nx=256, ny=128, D=20.0, center=(64.0, 64.0), n_markers=63)
    _, _, a = configs.build_solver(configs.viv2d(**kw))
    times = a.tune(trial_steps=20)
    assert set(times) == {"steps", "persistent"}, times
    assert a.step.run_form == min(times, key=times.get)
    _, _, b = configs.build_solver(configs.viv2d(**kw))
    b.step.set_run_form("persistent" if a.step.run_form == "steps" else "steps")
    with torch.cuda.stream(torch.cuda.Stream()):
        b.run(80, graph=True)  # the tuner advanced a by 4 x 20 steps
        a.run(30, graph=True)
        b.run(30, graph=True)
        torch.cuda.synchronize()
    assert np.array_equal(N(a.f), N(b.f))
    with pytest.raises(ValueError):
        a.step.set_run_form("fast")
