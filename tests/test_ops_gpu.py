"""Per-operator CUDA kernels against the golden vectors of the reference's own functions.

Every array function of vivsim_gb300.{lbm, lbm3d, ib, ib3d, dyn} runs through the C ABI
on the GPU and is compared with the reference output (float32 and float64).  Tolerance,
norm-relative (max|a-b| / max|b|): float32 2e-6, float64 1e-12; stencil indices exact.
"""

import math

import numpy as np
import pytest
import torch

from conftest import golden, rel_err
from oracle.lattice import Q9_FACES, Q19_FACES

pytestmark = pytest.mark.gpu
TOL = {"f32": 2e-6, "f64": 1e-12}


def T(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def N(t):
    return t.detach().cpu().numpy()


def check(mode, got, key, tol=None):
    err = rel_err(N(got) if isinstance(got, torch.Tensor) else got, golden(mode)[key])
    assert err <= (tol or TOL[mode]), f"{key}: rel err {err:.3e}"


@pytest.fixture(scope="module")
def vs():
    import vivsim_gb300
    vivsim_gb300.build()
    from vivsim_gb300 import dyn, ib, ib3d, lbm, lbm3d
    return dict(lbm=lbm, lbm3d=lbm3d, ib=ib, ib3d=ib3d, dyn=dyn)


def test_d2_basic(vs, mode):
    lbm = vs["lbm"]
    G = golden(mode)
    f = T(G["d2.f"])
    check(mode, lbm.streaming(f), "d2.streaming")
    r, u = lbm.get_macroscopic(f)
    check(mode, r, "d2.macro.rho")
    check(mode, u, "d2.macro.u")
    feq = lbm.get_equilibrium(T(G["d2.rho_in"]), T(G["d2.u_in"]))
    check(mode, feq, "d2.equilibrium")
    om = 1.7
    check(mode, lbm.collision_bgk(f, feq, om), "d2.bgk")
    check(mode, lbm.collision_kbc(f, feq, om), "d2.kbc")
    check(mode, lbm.collision_reg(f, feq, om), "d2.reg")
    check(mode, lbm.get_mrt_collision_operator(om, f.dtype).numpy(), "d2.mrt_op")
    check(mode, lbm.collision_mrt(f, feq, G["d2.mrt_op"]), "d2.mrt")
    g, u0 = T(G["d2.g"]), T(G["d2.u_in"])
    check(mode, lbm.get_guo_forcing_term(g, u0), "d2.guo_term")
    check(mode, lbm.forcing_edm(f, g, u0), "d2.edm")
    check(mode, lbm.forcing_guo_bgk(f, g, u0, om), "d2.guo_bgk")
    check(mode, lbm.forcing_guo_mrt(f, g, u0, G["d2.mrt_fop"]), "d2.guo_mrt")
    check(mode, lbm.get_velocity_correction(g, T(G["d2.rho_in"])), "d2.vel_corr")
    check(mode, lbm.obstacle_bounce_back(f, T(G["d2.mask"])), "d2.obb")


@pytest.mark.parametrize("loc", ["left", "right", "top", "bottom"])
def test_d2_boundaries(vs, mode, loc):
    lbm = vs["lbm"]
    G = golden(mode)
    fn, fpn = G["d2.f"], G["d2.f_pre"]
    f, fp = T(fn), T(fpn)
    wall = (slice(None),) + Q9_FACES[loc].wall
    rest = np.ones(fn.shape[1:], bool)
    rest[Q9_FACES[loc].wall] = False

    def cw(out, key):
        o = N(out)
        assert np.array_equal(o[:, rest], fn[:, rest]), key
        check(mode, o[wall], key)

    kw = dict(rho_wall=1.02, ux_wall=0.03, uy_wall=-0.01)
    cw(lbm.boundary_nee(f, loc, **kw), f"d2.nee.{loc}")
    cw(lbm.boundary_nebb(f, loc, **kw), f"d2.nebb.{loc}")
    cw(lbm.boundary_equilibrium(f, loc, **kw), f"d2.eq.{loc}")
    vk = dict(ux_wall=0.04, uy_wall=0.01)
    cw(lbm.boundary_velocity_nee(f, loc, **vk), f"d2.vnee.{loc}")
    cw(lbm.boundary_velocity_nebb(f, loc, **vk), f"d2.vnebb.{loc}")
    cw(lbm.boundary_velocity_equilibrium(f, loc, **vk), f"d2.veq.{loc}")
    cw(lbm.boundary_pressure_nee(f, loc, rho_wall=1.01), f"d2.pnee.{loc}")
    cw(lbm.boundary_pressure_nebb(f, loc, rho_wall=1.01), f"d2.pnebb.{loc}")
    cw(lbm.boundary_pressure_equilibrium(f, loc, rho_wall=1.01), f"d2.peq.{loc}")
    fk = dict(rho_wall=1.0, ux_wall=0.05, uy_wall=0.002, gx_wall=1e-4, gy_wall=-2e-4)
    cw(lbm.boundary_force_corrected_nee(f, loc, **fk), f"d2.fcnee.{loc}")
    cw(lbm.boundary_force_corrected_nebb(f, loc, **fk), f"d2.fcnebb.{loc}")
    cw(lbm.boundary_force_corrected_equilibrium(f, loc, **fk), f"d2.fceq.{loc}")
    cw(lbm.boundary_bounce_back(fp, f, loc, ux_wall=0.02, uy_wall=0.01), f"d2.bb.{loc}")
    cw(lbm.boundary_specular_reflection(fp, f, loc, ux_wall=0.02, uy_wall=0.01), f"d2.spec.{loc}")
    rc, uc = lbm.boundary_characteristic(T(G["d2.rho_in"]), T(G["d2.u_in"]), loc)
    check(mode, rc, f"d2.cbc.{loc}.rho")
    check(mode, uc, f"d2.cbc.{loc}.u")


def test_d3_basic(vs, mode):
    lbm3d = vs["lbm3d"]
    G = golden(mode)
    f = T(G["d3.f"])
    check(mode, lbm3d.streaming(f), "d3.streaming")
    r, u = lbm3d.get_macroscopic(f)
    check(mode, r, "d3.macro.rho")
    check(mode, u, "d3.macro.u")
    feq = lbm3d.get_equilibrium(T(G["d3.rho_in"]), T(G["d3.u_in"]))
    check(mode, feq, "d3.equilibrium")
    om = 1.9
    check(mode, lbm3d.collision_bgk(f, feq, om), "d3.bgk")
    check(mode, lbm3d.collision_kbc(f, feq, om), "d3.kbc")
    check(mode, lbm3d.collision_reg(f, feq, om), "d3.reg")
    check(mode, lbm3d.get_mrt_collision_operator(om, f.dtype).numpy(), "d3.mrt_op")
    check(mode, lbm3d.collision_mrt(f, feq, G["d3.mrt_op"]), "d3.mrt")
    g, u0 = T(G["d3.g"]), T(G["d3.u_in"])
    check(mode, lbm3d.get_guo_forcing_term(g, u0), "d3.guo_term")
    check(mode, lbm3d.forcing_edm(f, g, u0), "d3.edm")
    check(mode, lbm3d.forcing_guo_bgk(f, g, u0, om), "d3.guo_bgk")
    check(mode, lbm3d.forcing_guo_mrt(f, g, u0, G["d3.mrt_fop"]), "d3.guo_mrt")
    check(mode, lbm3d.obstacle_bounce_back(f, T(G["d3.mask"])), "d3.obb")


@pytest.mark.parametrize("loc", ["left", "right", "bottom", "top", "back", "front"])
def test_d3_boundaries(vs, mode, loc):
    lbm3d = vs["lbm3d"]
    G = golden(mode)
    f, fp = T(G["d3.f"]), T(G["d3.f_pre"])
    wall = (slice(None),) + Q19_FACES[loc].wall

    def cw(out, key):
        check(mode, N(out)[wall], key)

    kw = dict(rho_wall=1.02, ux_wall=0.03, uy_wall=-0.01, uz_wall=0.02)
    cw(lbm3d.boundary_nee(f, loc, **kw), f"d3.nee.{loc}")
    cw(lbm3d.boundary_nebb(f, loc, **kw), f"d3.nebb.{loc}")
    cw(lbm3d.boundary_equilibrium(f, loc, **kw), f"d3.eq.{loc}")
    vk = dict(ux_wall=0.04, uy_wall=0.01, uz_wall=-0.02)
    cw(lbm3d.boundary_velocity_nee(f, loc, **vk), f"d3.vnee.{loc}")
    cw(lbm3d.boundary_velocity_nebb(f, loc, **vk), f"d3.vnebb.{loc}")
    cw(lbm3d.boundary_velocity_equilibrium(f, loc, **vk), f"d3.veq.{loc}")
    cw(lbm3d.boundary_pressure_nee(f, loc, rho_wall=1.01), f"d3.pnee.{loc}")
    cw(lbm3d.boundary_pressure_nebb(f, loc, rho_wall=1.01), f"d3.pnebb.{loc}")
    cw(lbm3d.boundary_pressure_equilibrium(f, loc, rho_wall=1.01), f"d3.peq.{loc}")
    fk = dict(rho_wall=1.0, ux_wall=0.05, uy_wall=0.002, uz_wall=-0.001, gx_wall=1e-4, gy_wall=-2e-4, gz_wall=3e-4)
    cw(lbm3d.boundary_force_corrected_nee(f, loc, **fk), f"d3.fcnee.{loc}")
    cw(lbm3d.boundary_force_corrected_nebb(f, loc, **fk), f"d3.fcnebb.{loc}")
    cw(lbm3d.boundary_force_corrected_equilibrium(f, loc, **fk), f"d3.fceq.{loc}")
    bk = dict(ux_wall=0.02, uy_wall=0.01, uz_wall=-0.01)
    cw(lbm3d.boundary_bounce_back(fp, f, loc, **bk), f"d3.bb.{loc}")
    cw(lbm3d.boundary_specular_reflection(fp, f, loc, **bk), f"d3.spec.{loc}")
    rc, uc = lbm3d.boundary_characteristic(T(G["d3.rho_in"]), T(G["d3.u_in"]), loc)
    check(mode, rc, f"d3.cbc.{loc}.rho")
    check(mode, uc, f"d3.cbc.{loc}.u")


def test_ib_ops(vs, mode):
    ib, ib3d = vs["ib"], vs["ib3d"]
    G = golden(mode)
    r = T(G["ib.r"])
    check(mode, ib.kernel_peskin_3pt(r), "ib.k_peskin3")
    check(mode, ib.kernel_peskin_4pt(r), "ib.k_peskin4")
    check(mode, ib.kernel_cosine_4pt(r), "ib.k_cosine4", 1e-6 if mode == "f32" else 1e-12)
    mx, my = T(G["ib2.mx"]), T(G["ib2.my"])
    for name, k in (("peskin4", ib.kernel_peskin_4pt), ("peskin3", ib.kernel_peskin_3pt),
                    ("cosine4", ib.kernel_cosine_4pt)):
        W, I = ib.get_ib_stencil(mx, my, 24, kernel=k, stencil_radius=2)
        assert np.array_equal(N(I), G[f"ib2.I.{name}"]), name
        check(mode, W, f"ib2.W.{name}", 1e-6 if mode == "f32" else 1e-12)
    W1, I1 = ib.get_ib_stencil(mx, my, 24, kernel=ib.kernel_peskin_3pt, stencil_radius=1)
    assert np.array_equal(N(I1), G["ib2.I.r1"])
    check(mode, W1, "ib2.W.r1")
    W, I = T(G["ib2.W.peskin4"]), T(G["ib2.I.peskin4"])
    check(mode, ib.interpolate(T(G["ib2.ugrid"]), W, I), "ib2.interp")
    check(mode, ib.spread(T(G["ib2.Fm"]), T(G["ib2.grid0"]), W, I), "ib2.spread")
    g, h = ib.multi_direct_forcing(T(G["ib2.ugrid"]), W, I, T(G["ib2.ut"]), T(G["ib2.ds"]), n_iter=3)
    check(mode, g, "ib2.mdf.g")
    check(mode, h, "ib2.mdf.h")
    g, h = ib.multi_direct_forcing(T(G["ib2.ugrid"]), W, I, T(G["ib2.ut"]), 1.3, n_iter=5)
    check(mode, g, "ib2.mdf5.g")
    check(mode, h, "ib2.mdf5.h")
    W3, I3 = ib3d.get_ib_stencil(T(G["ib3.X"]), (16, 14, 12), kernel=ib3d.kernel_peskin_4pt)
    assert np.array_equal(N(I3), G["ib3.I"])
    check(mode, W3, "ib3.W", 1e-6 if mode == "f32" else 1e-12)
    W3c, I3c = ib3d.get_ib_stencil(T(G["ib3.X"]), (16, 14, 12), kernel=ib3d.kernel_cosine_4pt)
    assert np.array_equal(N(I3c), G["ib3.I.cosine4"])
    check(mode, W3c, "ib3.W.cosine4", 1e-6 if mode == "f32" else 1e-12)
    W3, I3 = T(G["ib3.W"]), T(G["ib3.I"])
    check(mode, ib3d.interpolate(T(G["ib3.ugrid"]), W3, I3), "ib3.interp")
    z = torch.zeros((3, 16, 14, 12), dtype=W3.dtype, device="cuda")
    check(mode, ib3d.spread(T(G["ib3.Fm"]), z, W3, I3), "ib3.spread")
    g, h = ib3d.multi_direct_forcing(T(G["ib3.ugrid"]), W3, I3, T(G["ib3.ut"]), 0.9, n_iter=3)
    check(mode, g, "ib3.mdf.g")
    check(mode, h, "ib3.mdf.h")


def test_spread_is_deterministic(vs, mode):
    """Two spreads of the same input are bitwise identical (no floating-point atomics)."""
    ib = vs["ib"]
    G = golden(mode)
    W, I = T(G["ib2.W.peskin4"]), T(G["ib2.I.peskin4"])
    a = ib.spread(T(G["ib2.Fm"]), T(G["ib2.grid0"]), W, I)
    b = ib.spread(T(G["ib2.Fm"]), T(G["ib2.grid0"]), W, I)
    assert torch.equal(a, b)


def test_dyn(vs, mode):
    dyn = vs["dyn"]
    G = golden(mode)
    a, v, d, h = (T(x) for x in G["dyn.vec.in"])
    check(mode, torch.stack(dyn.newmark(a, v, d, h, 12.0, 3.0, 0.4)), "dyn.vec")
    a, v, d, h = (T(x) for x in G["dyn.mat.in"])
    out = dyn.newmark(a, v, d, h, T(G["dyn.mat.m"]), T(G["dyn.mat.k"]), T(G["dyn.mat.c"]))
    check(mode, torch.stack(out), "dyn.mat", 1e-5 if mode == "f32" else 1e-12)
    mx, my = T(G["ib2.mx"]), T(G["ib2.my"])
    dv = T(G["dyn.vec.in"][2])
    check(mode, torch.stack(dyn.get_markers_coords_2dof(mx, my, dv)), "dyn.coords2")
    d3, v3 = T(G["dyn.mat.in"][2]), T(G["dyn.mat.in"][1])
    x3, y3 = dyn.get_markers_coords_3dof(mx, my, 14.3, 11.7, d3)
    check(mode, torch.stack([x3, y3]), "dyn.coords3", 1e-6 if mode == "f32" else 1e-12)
    check(mode, dyn.get_markers_velocity_3dof(x3, y3, 14.3, 11.7, d3, v3), "dyn.vel3", 1e-6 if mode == "f32" else 1e-12)
    check(mode, dyn.get_force_to_obj(T(G["ib2.Fm"])), "dyn.force")
    check(mode, dyn.get_torque_to_obj(x3, y3, 14.3, 11.7, d3, T(G["ib2.Fm"])), "dyn.torque",
          1e-5 if mode == "f32" else 1e-12)
    s = np.array(dyn.newmark(0.01, -0.02, 0.3, 1.5, 12.0, 3.0, 0.4))
    assert rel_err(s, G["dyn.scalar"].astype(np.float64)) < (1e-6 if mode == "f32" else 1e-15)


def test_cpu_tensor_is_rejected(vs):
    with pytest.raises(ValueError, match="CUDA"):
        vs["lbm"].streaming(torch.zeros((9, 4, 4)))
