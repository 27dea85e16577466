"""Pin the oracle: every oracle function against golden vectors from the reference's own code.

The golden vectors come from running the reference vivsim source (through a NumPy
backend for its JAX calls) in float32 (``jax_enable_x64`` off) and float64 (on).
Tolerances are norm-relative (max|a-b| / max|b|): float64 1e-12, float32 2e-6 for
single operators and 2e-5 for multi-step recipes (summation order of ``einsum``
contractions is the only difference).
"""

import math

import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import dyn, ib
from oracle import lbm2d as L2
from oracle import lbm3d as L3
from oracle import recipes
from oracle.lattice import Q9_C as Q9_C_
from oracle.lattice import Q9_FACES, Q19_FACES
from oracle.lattice import Q9_OPP as Q9_OPP_
from oracle.lattice import Q19_C as Q19_C_
from oracle.lattice import Q19_OPP as Q19_OPP_

TOL = {"f32": 2e-6, "f64": 1e-12}
TOL_RECIPE = {"f32": 2e-5, "f64": 1e-11}


def check(mode, got, key, tol=None):
    G = golden(mode)
    err = rel_err(got, G[key])
    assert err <= (tol or TOL[mode]), f"{key}: rel err {err:.3e}"


def test_d2_basic(mode):
    G = golden(mode)
    f = G["d2.f"]
    check(mode, L2.streaming(f), "d2.streaming")
    r, u = L2.get_macroscopic(f)
    check(mode, r, "d2.macro.rho")
    check(mode, u, "d2.macro.u")
    feq = L2.get_equilibrium(G["d2.rho_in"], G["d2.u_in"])
    check(mode, feq, "d2.equilibrium")
    om = 1.7
    check(mode, L2.collision_bgk(f, feq, om), "d2.bgk")
    check(mode, L2.collision_kbc(f, feq, om), "d2.kbc")
    check(mode, L2.collision_reg(f, feq, om), "d2.reg")
    dt = f.dtype
    check(mode, L2.get_mrt_collision_operator(om, dt), "d2.mrt_op")
    check(mode, L2.collision_mrt(f, feq, G["d2.mrt_op"]), "d2.mrt")
    g, u0 = G["d2.g"], G["d2.u_in"]
    check(mode, L2.get_guo_forcing_term(g, u0), "d2.guo_term")
    check(mode, L2.forcing_edm(f, g, u0), "d2.edm")
    check(mode, L2.forcing_guo_bgk(f, g, u0, om), "d2.guo_bgk")
    check(mode, L2.get_mrt_forcing_operator(om, dt), "d2.mrt_fop")
    check(mode, L2.forcing_guo_mrt(f, g, u0, G["d2.mrt_fop"]), "d2.guo_mrt")
    check(mode, L2.get_velocity_correction(g, G["d2.rho_in"]), "d2.vel_corr")
    check(mode, L2.obstacle_bounce_back(f, G["d2.mask"]), "d2.obb")


@pytest.mark.parametrize("loc", ["left", "right", "top", "bottom"])
def test_d2_boundaries(mode, loc):
    G = golden(mode)
    f, fp = G["d2.f"], G["d2.f_pre"]
    wall = (slice(None),) + Q9_FACES[loc].wall

    def cw(out, key):
        rest = np.ones(f.shape[1:], bool)
        rest[Q9_FACES[loc].wall] = False
        assert np.array_equal(out[:, rest], f[:, rest])
        check(mode, out[wall], key)

    kw = dict(rho_wall=1.02, ux_wall=0.03, uy_wall=-0.01)
    cw(L2.boundary_nee(f, loc, **kw), f"d2.nee.{loc}")
    cw(L2.boundary_nebb(f, loc, **kw), f"d2.nebb.{loc}")
    cw(L2.boundary_equilibrium(f, loc, **kw), f"d2.eq.{loc}")
    vk = dict(ux_wall=0.04, uy_wall=0.01)
    cw(L2.boundary_velocity_nee(f, loc, **vk), f"d2.vnee.{loc}")
    cw(L2.boundary_velocity_nebb(f, loc, **vk), f"d2.vnebb.{loc}")
    cw(L2.boundary_velocity_equilibrium(f, loc, **vk), f"d2.veq.{loc}")
    cw(L2.boundary_pressure_nee(f, loc, rho_wall=1.01), f"d2.pnee.{loc}")
    cw(L2.boundary_pressure_nebb(f, loc, rho_wall=1.01), f"d2.pnebb.{loc}")
    cw(L2.boundary_pressure_equilibrium(f, loc, rho_wall=1.01), f"d2.peq.{loc}")
    fk = dict(rho_wall=1.0, ux_wall=0.05, uy_wall=0.002, gx_wall=1e-4, gy_wall=-2e-4)
    cw(L2.boundary_force_corrected_nee(f, loc, **fk), f"d2.fcnee.{loc}")
    cw(L2.boundary_force_corrected_nebb(f, loc, **fk), f"d2.fcnebb.{loc}")
    cw(L2.boundary_force_corrected_equilibrium(f, loc, **fk), f"d2.fceq.{loc}")
    cw(L2.boundary_bounce_back(fp, f, loc, ux_wall=0.02, uy_wall=0.01), f"d2.bb.{loc}")
    cw(L2.boundary_specular_reflection(fp, f, loc, ux_wall=0.02, uy_wall=0.01), f"d2.spec.{loc}")
    rc, uc = L2.boundary_characteristic(G["d2.rho_in"], G["d2.u_in"], loc)
    check(mode, rc, f"d2.cbc.{loc}.rho")
    check(mode, uc, f"d2.cbc.{loc}.u")


def test_d3_basic(mode):
    G = golden(mode)
    f = G["d3.f"]
    check(mode, L3.streaming(f), "d3.streaming")
    r, u = L3.get_macroscopic(f)
    check(mode, r, "d3.macro.rho")
    check(mode, u, "d3.macro.u")
    feq = L3.get_equilibrium(G["d3.rho_in"], G["d3.u_in"])
    check(mode, feq, "d3.equilibrium")
    assert np.array_equal(L3.SECOND_ORDER_PROJECTION, G["d3.projection"].astype(np.float32))
    om = 1.9
    check(mode, L3.collision_bgk(f, feq, om), "d3.bgk")
    check(mode, L3.collision_kbc(f, feq, om), "d3.kbc")
    check(mode, L3.collision_reg(f, feq, om), "d3.reg")
    dt = f.dtype
    check(mode, L3.get_mrt_collision_operator(om, dt), "d3.mrt_op")
    check(mode, L3.collision_mrt(f, feq, G["d3.mrt_op"]), "d3.mrt")
    g, u0 = G["d3.g"], G["d3.u_in"]
    check(mode, L3.get_guo_forcing_term(g, u0), "d3.guo_term")
    check(mode, L3.forcing_edm(f, g, u0), "d3.edm")
    check(mode, L3.forcing_guo_bgk(f, g, u0, om), "d3.guo_bgk")
    check(mode, L3.get_mrt_forcing_operator(om, dt), "d3.mrt_fop")
    check(mode, L3.forcing_guo_mrt(f, g, u0, G["d3.mrt_fop"]), "d3.guo_mrt")
    check(mode, L3.obstacle_bounce_back(f, G["d3.mask"]), "d3.obb")


@pytest.mark.parametrize("loc", ["left", "right", "bottom", "top", "back", "front"])
def test_d3_boundaries(mode, loc):
    G = golden(mode)
    f, fp = G["d3.f"], G["d3.f_pre"]
    wall = (slice(None),) + Q19_FACES[loc].wall

    def cw(out, key):
        check(mode, out[wall], key)

    kw = dict(rho_wall=1.02, ux_wall=0.03, uy_wall=-0.01, uz_wall=0.02)
    cw(L3.boundary_nee(f, loc, **kw), f"d3.nee.{loc}")
    cw(L3.boundary_nebb(f, loc, **kw), f"d3.nebb.{loc}")
    cw(L3.boundary_equilibrium(f, loc, **kw), f"d3.eq.{loc}")
    vk = dict(ux_wall=0.04, uy_wall=0.01, uz_wall=-0.02)
    cw(L3.boundary_velocity_nee(f, loc, **vk), f"d3.vnee.{loc}")
    cw(L3.boundary_velocity_nebb(f, loc, **vk), f"d3.vnebb.{loc}")
    cw(L3.boundary_velocity_equilibrium(f, loc, **vk), f"d3.veq.{loc}")
    cw(L3.boundary_pressure_nee(f, loc, rho_wall=1.01), f"d3.pnee.{loc}")
    cw(L3.boundary_pressure_nebb(f, loc, rho_wall=1.01), f"d3.pnebb.{loc}")
    cw(L3.boundary_pressure_equilibrium(f, loc, rho_wall=1.01), f"d3.peq.{loc}")
    fk = dict(rho_wall=1.0, ux_wall=0.05, uy_wall=0.002, uz_wall=-0.001,
              gx_wall=1e-4, gy_wall=-2e-4, gz_wall=3e-4)
    cw(L3.boundary_force_corrected_nee(f, loc, **fk), f"d3.fcnee.{loc}")
    cw(L3.boundary_force_corrected_nebb(f, loc, **fk), f"d3.fcnebb.{loc}")
    cw(L3.boundary_force_corrected_equilibrium(f, loc, **fk), f"d3.fceq.{loc}")
    bk = dict(ux_wall=0.02, uy_wall=0.01, uz_wall=-0.01)
    cw(L3.boundary_bounce_back(fp, f, loc, **bk), f"d3.bb.{loc}")
    cw(L3.boundary_specular_reflection(fp, f, loc, **bk), f"d3.spec.{loc}")
    rc, uc = L3.boundary_characteristic(G["d3.rho_in"], G["d3.u_in"], loc)
    check(mode, rc, f"d3.cbc.{loc}.rho")
    check(mode, uc, f"d3.cbc.{loc}.u")


def test_ib_ops(mode):
    G = golden(mode)
    r = G["ib.r"]
    check(mode, ib.kernel_peskin_3pt(r), "ib.k_peskin3")
    check(mode, ib.kernel_peskin_4pt(r), "ib.k_peskin4")
    check(mode, ib.kernel_cosine_4pt(r), "ib.k_cosine4")
    mx, my = G["ib2.mx"], G["ib2.my"]
    for name in ("peskin4", "peskin3", "cosine4"):
        W, I = ib.get_ib_stencil(mx, my, 24, ib.KERNELS[name], 2)
        assert np.array_equal(I, G[f"ib2.I.{name}"])
        check(mode, W, f"ib2.W.{name}")
    W, I = ib.get_ib_stencil(mx, my, 24, ib.kernel_peskin_3pt, 1)
    assert np.array_equal(I, G["ib2.I.r1"])
    check(mode, W, "ib2.W.r1")
    W, I = G["ib2.W.peskin4"], G["ib2.I.peskin4"]
    check(mode, ib.interpolate(G["ib2.ugrid"], W, I), "ib2.interp")
    check(mode, ib.spread(G["ib2.Fm"], G["ib2.grid0"], W, I), "ib2.spread")
    g, h = ib.multi_direct_forcing(G["ib2.ugrid"], W, I, G["ib2.ut"], G["ib2.ds"], 3)
    check(mode, g, "ib2.mdf.g")
    check(mode, h, "ib2.mdf.h")
    g, h = ib.multi_direct_forcing(G["ib2.ugrid"], W, I, G["ib2.ut"], 1.3, 5)
    check(mode, g, "ib2.mdf5.g")
    check(mode, h, "ib2.mdf5.h")
    X = np.stack([mx, my], axis=1)
    check(mode, ib.get_ds(X), "ib2.ds_curve")
    check(mode, ib.get_ds(X, closed=False), "ib2.ds_open")
    W3, I3 = ib.get_ib_stencil_3d(G["ib3.X"], (16, 14, 12))
    assert np.array_equal(I3, G["ib3.I"])
    check(mode, W3, "ib3.W")
    W3c, I3c = ib.get_ib_stencil_3d(G["ib3.X"], (16, 14, 12), ib.kernel_cosine_4pt)
    assert np.array_equal(I3c, G["ib3.I.cosine4"])
    check(mode, W3c, "ib3.W.cosine4")
    check(mode, ib.interpolate(G["ib3.ugrid"], W3, I3), "ib3.interp")
    z = np.zeros((3, 16, 14, 12), dtype=W3.dtype)
    check(mode, ib.spread(G["ib3.Fm"], z, W3, I3), "ib3.spread")
    g, h = ib.multi_direct_forcing(G["ib3.ugrid"], W3, I3, G["ib3.ut"], 0.9, 3)
    check(mode, g, "ib3.mdf.g")
    check(mode, h, "ib3.mdf.h")


def test_dyn(mode):
    G = golden(mode)
    dt = G["d2.f"].dtype
    check(mode, np.array(dyn.newmark(0.01, -0.02, 0.3, 1.5, 12.0, 3.0, 0.4), dtype=dt), "dyn.scalar")
    a, v, d, h = G["dyn.vec.in"]
    check(mode, np.stack(dyn.newmark(a, v, d, h, 12.0, 3.0, 0.4)), "dyn.vec")
    a, v, d, h = G["dyn.mat.in"]
    check(mode, np.stack(dyn.newmark(a, v, d, h, G["dyn.mat.m"], G["dyn.mat.k"], G["dyn.mat.c"])), "dyn.mat")
    mx, my = G["ib2.mx"], G["ib2.my"]
    dv = G["dyn.vec.in"][2]
    check(mode, np.stack(dyn.get_markers_coords_2dof(mx, my, dv)), "dyn.coords2")
    d3 = G["dyn.mat.in"][2]
    v3 = G["dyn.mat.in"][1]
    x3, y3 = dyn.get_markers_coords_3dof(mx, my, 14.3, 11.7, d3)
    check(mode, np.stack([x3, y3]), "dyn.coords3")
    check(mode, dyn.get_markers_velocity_3dof(x3, y3, 14.3, 11.7, d3, v3), "dyn.vel3")
    check(mode, dyn.get_force_to_obj(G["ib2.Fm"]), "dyn.force")
    check(mode, dyn.get_torque_to_obj(x3, y3, 14.3, 11.7, d3, G["ib2.Fm"]), "dyn.torque")


def test_recipe_cavity(mode):
    G = golden(mode)
    f = G["cav.f0"].copy()
    om = L2.get_omega(0.0256)
    for step in range(1, 31):
        f = recipes.cavity_step(f, om, 0.1)
        if step in (1, 10, 30):
            check(mode, f, f"cav.f{step}", TOL_RECIPE[mode])


def _viv_body(G, dt):
    D, U0 = 8.0, 0.05
    M = 24
    area = math.pi * (D / 2) ** 2
    mass = area * 10.0
    fn = U0 / (5.0 * D)
    K = (2 * math.pi * fn) ** 2 * mass * (1 + 1 / 10.0)
    return recipes.Body2D(G["viv.X0"], G["viv.Y0"], math.pi * D / M, mass, K, 0.0, area,
                          free=(False, True), n_iter=3)


@pytest.mark.parametrize("coll", ["kbc", "mrt", "reg", "bgk"])
def test_recipe_viv(mode, coll):
    G = golden(mode)
    dt = G["viv.X0"].dtype
    nx, ny, U0 = 40, 24, 0.05
    om = L2.get_omega(U0 * 8.0 / 20.0)
    u = np.zeros((2, nx, ny), dt)
    u[0] = U0
    u[1] = G["viv.pert"]
    f = L2.get_equilibrium(np.ones((nx, ny), dt), u)
    body = _viv_body(G, dt)
    op = L2.get_mrt_collision_operator(om, dt)
    bcs = [("eq", "left", dict(ux_wall=U0)), ("pnee", "right", dict(rho_wall=1.0))]
    for step in range(1, 7):
        f, h = recipes.ib_lbm_step_2d(f, body, coll, om, op, bcs)
        if step == 1:
            r, uu = L2.get_macroscopic(f)
            check(mode, r, f"viv.{coll}.rho1", TOL_RECIPE[mode])
            check(mode, uu, f"viv.{coll}.u1", TOL_RECIPE[mode])
        if step in (1, 6):
            check(mode, h, f"viv.{coll}.h{step}", 1e-4 if mode == "f32" else 1e-10)
            check(mode, np.stack([body.a, body.v, body.d]), f"viv.{coll}.body{step}",
                  1e-4 if mode == "f32" else 1e-10)
    check(mode, f, f"viv.{coll}.f6", TOL_RECIPE[mode])


def test_recipe_viv_fsi_subiterations(mode):
    """FSI_ITER = 2 (examples/2d/vortex_induced_vibration.py:111-139), both translations free."""
    G = golden(mode)
    dt = G["viv.X0"].dtype
    nx, ny, U0, D, M = 40, 24, 0.05, 8.0, 24
    om = L2.get_omega(U0 * D / 20.0)
    u = np.zeros((2, nx, ny), dt)
    u[0] = U0
    u[1] = G["viv.pert"]
    f = L2.get_equilibrium(np.ones((nx, ny), dt), u)
    area = math.pi * (D / 2) ** 2
    mass = area * 10.0
    K = (2 * math.pi * U0 / (5.0 * D)) ** 2 * mass * (1 + 1 / 10.0)
    body = recipes.Body2D(G["viv.X0"], G["viv.Y0"], math.pi * D / M, mass, K, 0.0, area, free=(True, True),
                          n_iter=3, v=np.array([0.0, 1e-2 * U0], dt), fsi_iter=2)
    bcs = [("eq", "left", dict(ux_wall=U0)), ("pnee", "right", dict(rho_wall=1.0))]
    for step in range(1, 7):
        f, h = recipes.ib_lbm_step_2d(f, body, "kbc", om, None, bcs)
        if step in (1, 6):
            check(mode, f, f"vivfsi.f{step}", TOL_RECIPE[mode])
            check(mode, h, f"vivfsi.h{step}", 1e-4 if mode == "f32" else 1e-10)
            check(mode, np.stack([body.a, body.v, body.d]), f"vivfsi.body{step}", 1e-4 if mode == "f32" else 1e-10)


@pytest.mark.parametrize("coll", ["reg", "bgk", "kbc"])
def test_recipe_sphere(mode, coll):
    G = golden(mode)
    X = G["sph.X"]
    dt = X.dtype
    nx, ny, nz, D, U0, M = 16, 12, 12, 5.0, 0.05, 79
    om = L3.get_omega(U0 * D / 30.0)
    W, I = ib.get_ib_stencil_3d(X, (nx, ny, nz))
    ds = 4 * math.pi * (D / 2) ** 2 / M
    u = G["sph.pert"].copy()
    u[0] = u[0] + U0
    f = L3.get_equilibrium(np.ones((nx, ny, nz), dt), u)
    bcs = [("eq", "left", dict(ux_wall=U0)), ("pnee", "right", dict(rho_wall=1.0))]
    for step in range(1, 5):
        f, h = recipes.ib_lbm_step_3d(f, W, I, np.zeros((M, 3), dt), ds, coll, om, None, bcs)
        if step == 1:
            r, uu = L3.get_macroscopic(f)
            check(mode, r, f"sph.{coll}.rho1", TOL_RECIPE[mode])
            check(mode, uu, f"sph.{coll}.u1", TOL_RECIPE[mode])
        if step in (1, 4):
            check(mode, h, f"sph.{coll}.h{step}", 1e-4 if mode == "f32" else 1e-10)
    check(mode, f, f"sph.{coll}.f4", TOL_RECIPE[mode])


POST_FIELDS = ("velocity_magnitude", "velocity_gradient", "vorticity", "vorticity_magnitude", "divergence",
               "strain_rate", "strain_rate_magnitude", "kinetic_energy", "mean_kinetic_energy", "enstrophy",
               "mean_enstrophy", "q_criterion")


def test_post_oracle(mode):
    from oracle import post
    G = golden(mode)
    for tag in ("p2", "p3"):
        u = G[f"{tag}.u"]
        for name in POST_FIELDS:
            err = rel_err(np.asarray(getattr(post, name)(u)), G[f"{tag}.{name}"])
            assert err <= TOL[mode], f"{tag}.{name}: {err:.3e}"
    assert rel_err(post.pressure(G["p.rho"]), G["p.pressure"]) <= TOL[mode]


REFINE_DIRS = ("left", "right", "up", "down")


def test_multigrid_oracle(mode):
    """Transfers are copies and one 4-term average: bit-exact against the reference."""
    from oracle import multigrid as mg
    G = golden(mode)
    for d in REFINE_DIRS:
        ff, fc = G[f"mg.{d}.ff"], G[f"mg.{d}.fc"]
        assert np.array_equal(mg.fine_to_coarse(ff, fc, d), G[f"mg.{d}.f2c"]), d
        assert np.array_equal(mg.coarse_to_fine(fc, ff, d), G[f"mg.{d}.c2f"]), d
    assert np.array_equal(mg.coarse_to_fine(G["mg.bc.fc"], G["mg.bc.ff"], "right"), G["mg.bc.c2f"])
    om = [mg.get_omega(nu, lv) for nu in (0.004, 0.02, 0.1) for lv in (-2, -1, 0, 1, 2, 3)]
    assert np.array_equal(np.array(om), G["mg.omega"])
    shapes = [mg.init_grid(w, h, lv, bx, by)[0].shape[1:] for w, h, lv, bx, by in
              ((16, 8, 0, 1, 0), (16, 8, 1, 0, 0), (16, 8, -1, 0, 2), (10, 6, 2, 1, 1))]
    assert np.array_equal(np.array(shapes), G["mg.init"])
    assert mg.coord_to_indices(10.5, 7.25, 2, 3, 2) == (34, 17)


def test_recipe_refined_channel(mode):
    G = golden(mode)
    fc, ff = G["rc.fc0"], G["rc.ff0"]
    om_c, om_f, u0 = G["rc.omega"]
    for s in range(6):
        fc, ff = recipes.refined_channel_cycle(fc, ff, float(om_c), float(om_f), float(u0))
        if s in (0, 5):
            check(mode, fc, f"rc.fc{s + 1}", TOL_RECIPE[mode])
            check(mode, ff, f"rc.ff{s + 1}", TOL_RECIPE[mode])


@pytest.mark.parametrize("scheme", ["nee", "eq", "nebb"])
def test_recipe_characteristic_outflow_2d(mode, scheme):
    G = golden(mode)
    om, u0 = (float(x) for x in G["cbc2.omega"])
    f = G["cbc2.f0"]
    bcs = [("eq", "left", dict(ux_wall=u0)), ("cbc", "right", dict(scheme=scheme))]
    for step in range(1, 9):
        f = recipes.lbm_step_2d(f, "kbc", om, bcs=bcs)
        if step in (1, 8):
            check(mode, f, f"cbc2.{scheme}.f{step}", TOL_RECIPE[mode])


def test_recipe_characteristic_outflow_3d(mode):
    G = golden(mode)
    om, u0 = (float(x) for x in G["cbc2.omega"])
    f = G["cbc3.f0"]
    bcs = [("eq", "left", dict(ux_wall=u0)), ("cbc", "right", dict(scheme="nee"))]
    for step in range(1, 5):
        f = recipes.lbm_step_3d(f, "bgk", om, bcs=bcs)
        if step in (1, 4):
            check(mode, f, f"cbc3.f{step}", TOL_RECIPE[mode])


def test_oracle_known_answers():
    """The oracle on two of the reference's known-answer examples (CPU, a few seconds):
    the Taylor-Green vortex decay (examples/2d/taylor_green_vortex.py, 64^2, 4000 steps)
    and Couette flow (examples/2d/couette_flow.py, 16^2, 12000 steps) against their
    analytic fields."""
    n, u0, nu = 64, 0.02, 0.02
    k = 2 * math.pi / n
    x = np.arange(n, dtype=np.float32)[:, None]
    y = np.arange(n, dtype=np.float32)[None, :]

    def tgv(t):
        dec = np.exp(-nu * 2 * k * k * t)
        return np.stack([u0 * np.sin(k * x) * np.cos(k * y) * dec,
                         -u0 * np.cos(k * x) * np.sin(k * y) * dec]).astype(np.float32)
    om = L2.get_omega(nu)
    f = L2.get_equilibrium(np.ones((n, n), np.float32), tgv(0.0))
    for _ in range(4000):
        r, u = L2.get_macroscopic(f)
        f = L2.streaming(L2.collision_bgk(f, L2.get_equilibrium(r, u), om))
    _, u = L2.get_macroscopic(f)
    ut = tgv(4000.0)
    assert np.linalg.norm(u - ut) / np.linalg.norm(ut) < 3e-3
    n, u0, nu = 16, 0.08, 0.10
    om = L2.get_omega(nu)
    f = L2.get_equilibrium(np.ones((n, n), np.float32), np.zeros((2, n, n), np.float32))
    for _ in range(12000):
        r, u = L2.get_macroscopic(f)
        f = L2.streaming(L2.collision_bgk(f, L2.get_equilibrium(r, u), om))
        f = L2.boundary_nee(f, "bottom")
        f = L2.boundary_nee(f, "top", ux_wall=u0)
    _, u = L2.get_macroscopic(f)
    ut = np.broadcast_to(u0 * np.arange(n, dtype=np.float32) / (n - 1), (n, n))
    assert np.linalg.norm(u[0] - ut) / np.linalg.norm(ut) < 1e-4


def test_threaded_cpu_step_equals_the_serial_recipes():
    """The CPU baseline's thread-parallel step (oracle/threaded.py) gives the serial
    recipes' bits: VIV with a moving body, the cavity, and a D3Q19 channel."""
    from oracle.threaded import ThreadedStep
    from vivsim_gb300 import configs
    viv = configs.viv2d(nx=96, ny=64, D=12.0, center=(30.0, 32.0), n_markers=38, seed=5)
    b = viv["body"]
    X = b["markers"].astype(np.float32)
    body = recipes.Body2D(X[:, 0], X[:, 1], b["ds"], b["mass"], b["stiffness"], b["damping"], b["added_mass_area"],
                          free=b["free_dof"][:2], kernel=b["kernel"], n_iter=b["n_iter"])
    t = ThreadedStep(viv, threads=4)
    f = viv["f0"].copy()
    for _ in range(3):
        t()
        f, _ = recipes.ib_lbm_step_2d(f, body, viv["collision"], viv["omega"], None, t.bcs)
    assert np.array_equal(t.f, f)
    assert np.array_equal(t.body.d, body.d) and np.array_equal(t.body.v, body.v)
    t.close()
    cav = configs.cavity(n=32)
    t = ThreadedStep(cav, threads=3)
    f = cav["f0"].copy()
    for _ in range(3):
        t()
        f = recipes.lbm_step_2d(f, cav["collision"], cav["omega"], None, t.bcs)
    assert np.array_equal(t.f, f)
    t.close()
    n = (12, 8, 6)
    rng = np.random.default_rng(3)
    u = (0.02 * rng.standard_normal((3,) + n)).astype(np.float32)
    f0 = L3.get_equilibrium(np.ones(n, np.float32), u)
    ch = dict(q=19, collision="reg", omega=1.7, body=None, f0=f0,
              boundaries=[("equilibrium", "left", "given", dict(ux_wall=0.03)),
                          ("nee", "right", "pressure", dict(rho_wall=1.0))])
    t = ThreadedStep(ch, threads=4)
    f = f0.copy()
    for _ in range(3):
        t()
        f = recipes.lbm_step_3d(f, "reg", 1.7, None, t.bcs)
    assert np.array_equal(t.f, f)
    t.close()
    sph = configs.sphere3d(nx=32, ny=24, nz=24, D=8.0, center=(12.0, 12.0, 12.0), n_markers=200)
    t = ThreadedStep(sph, threads=4)
    b = sph["body"]
    X = b["markers"].astype(np.float32)
    W, I = ib.get_ib_stencil_3d(X, sph["shape"])
    f = sph["f0"].copy()
    for _ in range(2):
        t()
        f, _ = recipes.ib_lbm_step_3d(f, W, I, np.zeros((X.shape[0], 3), np.float32), b["ds"], sph["collision"],
                                      sph["omega"], None, t.bcs, b["n_iter"])
    assert np.array_equal(t.f, f)
    t.close()


@pytest.mark.parametrize("coll", ["bgk", "kbc", "reg", "mrt"])
def test_oracle_collisions_conserve_mass_and_momentum(coll):
    """Every collision of the oracle keeps each node's density and momentum (float64 data).
    The lattice weights are float32 values, as in the reference under x64, so the
    equilibrium's moments match rho and rho u only to about 1e-8."""
    rng = np.random.default_rng(6)
    for L, q, shape in ((L2, 9, (6, 5)), (L3, 19, (4, 3, 5))):
        d = len(shape)
        rho = 1 + 0.05 * rng.standard_normal(shape)
        u = 0.05 * rng.standard_normal((d,) + shape)
        feq = L.get_equilibrium(rho, u)
        f = feq + 0.01 * rng.standard_normal((q,) + shape) * feq
        op = L.get_mrt_collision_operator(1.7, np.float64) if coll == "mrt" else None
        fo = recipes._collide(L, f, L.get_equilibrium(*L.get_macroscopic(f)), coll, 1.7, op)
        r0, u0 = L.get_macroscopic(f)
        r1, u1 = L.get_macroscopic(fo)
        assert np.max(np.abs(r1 - r0)) < 1e-7, (coll, q)
        assert np.max(np.abs(r1 * u1 - r0 * u0)) < 1e-7, (coll, q)


def test_oracle_streaming_is_a_permutation():
    """Streaming moves every population to its neighbour and back again."""
    rng = np.random.default_rng(8)
    for L, C, opp, shape in ((L2, Q9_C_, Q9_OPP_, (7, 5)), (L3, Q19_C_, Q19_OPP_, (4, 5, 3))):
        f = rng.random((len(opp),) + shape)
        g = L.streaming(f)
        back = L.streaming(g[list(opp)])[list(opp)]
        assert np.array_equal(back, f)
        assert np.allclose(g.sum(axis=tuple(range(1, g.ndim))), f.sum(axis=tuple(range(1, f.ndim))))


def test_oracle_drift_measurement():
    """oracle.drift: the perturbed start differs from the original by exactly one float32 ulp
    in population 0 at every 97th node; after a few cavity steps the float32 run sits within
    float32 rounding of the float64 run, and the one-ulp float64 pair stays far closer."""
    import subprocess
    import sys
    from conftest import ROOT
    from oracle.drift import perturbed
    f0 = np.random.default_rng(0).uniform(0.01, 0.2, (9, 20, 30)).astype(np.float32)
    fp = perturbed(f0)
    flat0, flatp = f0.reshape(9, -1), fp.reshape(9, -1)
    changed = np.nonzero(flat0 != flatp)
    assert set(changed[0]) == {0} and np.array_equal(changed[1], np.arange(0, 600, 97))
    assert np.all(flatp[0, ::97] == np.nextafter(flat0[0, ::97], np.float32(2.0)))
    out = subprocess.run([sys.executable, "-m", "oracle.drift", "--case", "cavity", "--steps", "3", "--perturb"],
                         cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    import json
    d = json.loads(out.stdout.strip().splitlines()[-1])
    assert d["steps"] == 3
    assert 0.0 < d["oracle32_vs_64_u"] < 1e-5 and 0.0 < d["oracle32_vs_64_rho"] < 1e-5
    assert d["perturbed64_vs_64_u"] < 1e-6
