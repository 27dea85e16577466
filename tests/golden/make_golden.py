"""Generate golden vectors by running the reference vivsim source on NumPy.

JAX is not installed here, so the reference package is imported through the
NumPy-backed JAX stand-in in ``tests/golden/_jaxshim`` (see its docstring for the
semantics it reproduces).  Every output below is produced by the reference's own
functions; the step recipes chain them exactly as the reference's examples do
(cited per recipe).  Run once where the reference source is present:

    python tests/golden/make_golden.py --reference /path/to/vivsim-checkout

It writes ``tests/golden/golden_f32.npz`` (``jax_enable_x64`` off) and
``tests/golden/golden_f64.npz`` (``jax_enable_x64`` on).  The inputs are stored next
to the outputs, so the tests never need the reference.
"""

import argparse
import math
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def fibonacci_sphere(n, radius, center):
    k = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * k / n)
    theta = math.pi * (1 + 5 ** 0.5) * k
    return np.stack([center[0] + radius * np.cos(theta) * np.sin(phi),
                     center[1] + radius * np.sin(theta) * np.sin(phi),
                     center[2] + radius * np.cos(phi)], axis=1)


def random_state_2d(rng, nx, ny, dt):
    rho = 1 + 0.05 * rng.standard_normal((nx, ny))
    u = 0.05 * rng.standard_normal((2, nx, ny))
    return rho.astype(dt), u.astype(dt)


def generate(mode, jax, jnp, lbm, lbm3d, ib, ib3d, dyn):
    jax.config.update("jax_enable_x64", mode == "f64")
    dt = np.float64 if mode == "f64" else np.float32
    rng = np.random.default_rng(20261203)
    G = {}

    def put(key, val):
        G[key] = np.asarray(val)

    def put_wall(key, f_in, wall, out):
        """Store the wall slice only, after checking every other node is unchanged."""
        out = np.asarray(out)
        rest = np.ones(out.shape[1:], dtype=bool)
        rest[wall] = False
        assert np.array_equal(out[:, rest], np.asarray(f_in)[:, rest]), key
        G[key] = out[(slice(None),) + wall]

    def A(x):
        return jnp.asarray(np.asarray(x, dtype=dt))

    from vivsim.lbm.lattice import D2Q9
    from vivsim.lbm3d.lattice import D3Q19
    W2 = {k: v.wall for k, v in D2Q9.boundary_spec.items()}
    W3F = {k: v.wall for k, v in D3Q19.boundary_spec.items()}

    # ------------------------------------------------------------- D2Q9 ops
    NX, NY = 12, 10
    rho0, u0 = random_state_2d(rng, NX, NY, dt)
    feq0 = np.asarray(lbm.get_equilibrium(A(rho0), A(u0)))
    f = (feq0 * (1 + 0.05 * rng.standard_normal(feq0.shape))).astype(dt)
    f_pre = (feq0 * (1 + 0.05 * rng.standard_normal(feq0.shape))).astype(dt)
    g = (1e-3 * rng.standard_normal((2, NX, NY))).astype(dt)
    mask = rng.random((NX, NY)) < 0.2
    put("d2.f", f); put("d2.f_pre", f_pre); put("d2.g", g); put("d2.mask", mask)
    put("d2.rho_in", rho0); put("d2.u_in", u0)
    F = A(f)
    put("d2.streaming", lbm.streaming(F))
    r, u = lbm.get_macroscopic(F)
    put("d2.macro.rho", r); put("d2.macro.u", u)
    feq = lbm.get_equilibrium(A(rho0), A(u0))
    put("d2.equilibrium", feq)
    om = 1.7
    put("d2.bgk", lbm.collision_bgk(F, feq, om))
    put("d2.kbc", lbm.collision_kbc(F, feq, om))
    put("d2.reg", lbm.collision_reg(F, feq, om))
    op = lbm.get_mrt_collision_operator(om)
    put("d2.mrt_op", op)
    put("d2.mrt", lbm.collision_mrt(F, feq, op))
    put("d2.guo_term", lbm.get_guo_forcing_term(A(g), A(u0)))
    put("d2.edm", lbm.forcing_edm(F, A(g), A(u0)))
    put("d2.guo_bgk", lbm.forcing_guo_bgk(F, A(g), A(u0), om))
    fop = lbm.get_mrt_forcing_operator(om)
    put("d2.mrt_fop", fop)
    put("d2.guo_mrt", lbm.forcing_guo_mrt(F, A(g), A(u0), fop))
    put("d2.vel_corr", lbm.get_velocity_correction(A(g), A(rho0)))
    for loc in ("left", "right", "top", "bottom"):
        put_wall(f"d2.nee.{loc}", F, W2[loc], lbm.boundary_nee(F, loc, rho_wall=1.02, ux_wall=0.03, uy_wall=-0.01))
        put_wall(f"d2.nebb.{loc}", F, W2[loc], lbm.boundary_nebb(F, loc, rho_wall=1.02, ux_wall=0.03, uy_wall=-0.01))
        put_wall(f"d2.eq.{loc}", F, W2[loc], lbm.boundary_equilibrium(F, loc, rho_wall=1.02, ux_wall=0.03, uy_wall=-0.01))
        put_wall(f"d2.vnee.{loc}", F, W2[loc], lbm.boundary_velocity_nee(F, loc, ux_wall=0.04, uy_wall=0.01))
        put_wall(f"d2.vnebb.{loc}", F, W2[loc], lbm.boundary_velocity_nebb(F, loc, ux_wall=0.04, uy_wall=0.01))
        put_wall(f"d2.veq.{loc}", F, W2[loc], lbm.boundary_velocity_equilibrium(F, loc, ux_wall=0.04, uy_wall=0.01))
        put_wall(f"d2.pnee.{loc}", F, W2[loc], lbm.boundary_pressure_nee(F, loc, rho_wall=1.01))
        put_wall(f"d2.pnebb.{loc}", F, W2[loc], lbm.boundary_pressure_nebb(F, loc, rho_wall=1.01))
        put_wall(f"d2.peq.{loc}", F, W2[loc], lbm.boundary_pressure_equilibrium(F, loc, rho_wall=1.01))
        kw = dict(rho_wall=1.0, ux_wall=0.05, uy_wall=0.002, gx_wall=1e-4, gy_wall=-2e-4)
        put_wall(f"d2.fcnee.{loc}", F, W2[loc], lbm.boundary_force_corrected_nee(F, loc, **kw))
        put_wall(f"d2.fcnebb.{loc}", F, W2[loc], lbm.boundary_force_corrected_nebb(F, loc, **kw))
        put_wall(f"d2.fceq.{loc}", F, W2[loc], lbm.boundary_force_corrected_equilibrium(F, loc, **kw))
        put_wall(f"d2.bb.{loc}", F, W2[loc], lbm.boundary_bounce_back(A(f_pre), F, loc, ux_wall=0.02, uy_wall=0.01))
        put_wall(f"d2.spec.{loc}", F, W2[loc], lbm.boundary_specular_reflection(A(f_pre), F, loc, ux_wall=0.02, uy_wall=0.01))
        rc, uc = lbm.boundary_characteristic(A(rho0), A(u0), loc)
        put(f"d2.cbc.{loc}.rho", rc); put(f"d2.cbc.{loc}.u", uc)
    put("d2.obb", lbm.obstacle_bounce_back(F, jnp.asarray(mask)))

    # ------------------------------------------------------------ D3Q19 ops
    NX3, NY3, NZ3 = 6, 5, 4
    rho3 = (1 + 0.05 * rng.standard_normal((NX3, NY3, NZ3))).astype(dt)
    u3 = (0.05 * rng.standard_normal((3, NX3, NY3, NZ3))).astype(dt)
    feq3 = np.asarray(lbm3d.get_equilibrium(A(rho3), A(u3)))
    f3 = (feq3 * (1 + 0.05 * rng.standard_normal(feq3.shape))).astype(dt)
    f3_pre = (feq3 * (1 + 0.05 * rng.standard_normal(feq3.shape))).astype(dt)
    g3 = (1e-3 * rng.standard_normal((3, NX3, NY3, NZ3))).astype(dt)
    mask3 = rng.random((NX3, NY3, NZ3)) < 0.2
    put("d3.f", f3); put("d3.f_pre", f3_pre); put("d3.g", g3); put("d3.mask", mask3)
    put("d3.rho_in", rho3); put("d3.u_in", u3)
    F3 = A(f3)
    put("d3.streaming", lbm3d.streaming(F3))
    r3, uu3 = lbm3d.get_macroscopic(F3)
    put("d3.macro.rho", r3); put("d3.macro.u", uu3)
    feq3j = lbm3d.get_equilibrium(A(rho3), A(u3))
    put("d3.equilibrium", feq3j)
    om3 = 1.9
    put("d3.bgk", lbm3d.collision_bgk(F3, feq3j, om3))
    put("d3.kbc", lbm3d.collision_kbc(F3, feq3j, om3))
    put("d3.reg", lbm3d.collision_reg(F3, feq3j, om3))
    from vivsim.lbm3d.collision import reg as _reg3
    put("d3.projection", _reg3._SECOND_ORDER_PROJECTION)
    op3 = lbm3d.get_mrt_collision_operator(om3)
    put("d3.mrt_op", op3)
    put("d3.mrt", lbm3d.collision_mrt(F3, feq3j, op3))
    put("d3.guo_term", lbm3d.get_guo_forcing_term(A(g3), A(u3)))
    put("d3.edm", lbm3d.forcing_edm(F3, A(g3), A(u3)))
    put("d3.guo_bgk", lbm3d.forcing_guo_bgk(F3, A(g3), A(u3), om3))
    fop3 = lbm3d.get_mrt_forcing_operator(om3)
    put("d3.mrt_fop", fop3)
    put("d3.guo_mrt", lbm3d.forcing_guo_mrt(F3, A(g3), A(u3), fop3))
    for loc in ("left", "right", "bottom", "top", "back", "front"):
        kw = dict(rho_wall=1.02, ux_wall=0.03, uy_wall=-0.01, uz_wall=0.02)
        put_wall(f"d3.nee.{loc}", F3, W3F[loc], lbm3d.boundary_nee(F3, loc, **kw))
        put_wall(f"d3.nebb.{loc}", F3, W3F[loc], lbm3d.boundary_nebb(F3, loc, **kw))
        put_wall(f"d3.eq.{loc}", F3, W3F[loc], lbm3d.boundary_equilibrium(F3, loc, **kw))
        vk = dict(ux_wall=0.04, uy_wall=0.01, uz_wall=-0.02)
        put_wall(f"d3.vnee.{loc}", F3, W3F[loc], lbm3d.boundary_velocity_nee(F3, loc, **vk))
        put_wall(f"d3.vnebb.{loc}", F3, W3F[loc], lbm3d.boundary_velocity_nebb(F3, loc, **vk))
        put_wall(f"d3.veq.{loc}", F3, W3F[loc], lbm3d.boundary_velocity_equilibrium(F3, loc, **vk))
        put_wall(f"d3.pnee.{loc}", F3, W3F[loc], lbm3d.boundary_pressure_nee(F3, loc, rho_wall=1.01))
        put_wall(f"d3.pnebb.{loc}", F3, W3F[loc], lbm3d.boundary_pressure_nebb(F3, loc, rho_wall=1.01))
        put_wall(f"d3.peq.{loc}", F3, W3F[loc], lbm3d.boundary_pressure_equilibrium(F3, loc, rho_wall=1.01))
        fk = dict(rho_wall=1.0, ux_wall=0.05, uy_wall=0.002, uz_wall=-0.001,
                  gx_wall=1e-4, gy_wall=-2e-4, gz_wall=3e-4)
        put_wall(f"d3.fcnee.{loc}", F3, W3F[loc], lbm3d.boundary_force_corrected_nee(F3, loc, **fk))
        put_wall(f"d3.fcnebb.{loc}", F3, W3F[loc], lbm3d.boundary_force_corrected_nebb(F3, loc, **fk))
        put_wall(f"d3.fceq.{loc}", F3, W3F[loc], lbm3d.boundary_force_corrected_equilibrium(F3, loc, **fk))
        bk = dict(ux_wall=0.02, uy_wall=0.01, uz_wall=-0.01)
        put_wall(f"d3.bb.{loc}", F3, W3F[loc], lbm3d.boundary_bounce_back(A(f3_pre), F3, loc, **bk))
        put_wall(f"d3.spec.{loc}", F3, W3F[loc], lbm3d.boundary_specular_reflection(A(f3_pre), F3, loc, **bk))
        rc, uc = lbm3d.boundary_characteristic(A(rho3), A(u3), loc)
        put(f"d3.cbc.{loc}.rho", rc); put(f"d3.cbc.{loc}.u", uc)
    put("d3.obb", lbm3d.obstacle_bounce_back(F3, jnp.asarray(mask3)))

    # ----------------------------------------------------------------- IB ops
    r = np.linspace(-2.6, 2.6, 105).astype(dt)
    put("ib.r", r)
    put("ib.k_peskin3", ib.kernel_peskin_3pt(A(r)))
    put("ib.k_peskin4", ib.kernel_peskin_4pt(A(r)))
    put("ib.k_cosine4", ib.kernel_cosine_4pt(A(r)))
    GX, GY = 30, 24
    M = 20
    th = np.linspace(0, 2 * np.pi, M, endpoint=False)
    mx = (14.3 + 5.2 * np.cos(th)).astype(dt)
    my = (11.7 + 5.2 * np.sin(th)).astype(dt)
    put("ib2.mx", mx); put("ib2.my", my)
    for kname, kfn in (("peskin4", ib.kernel_peskin_4pt), ("peskin3", ib.kernel_peskin_3pt),
                       ("cosine4", ib.kernel_cosine_4pt)):
        W, I = ib.get_ib_stencil(A(mx), A(my), GY, kernel=kfn, stencil_radius=2)
        put(f"ib2.W.{kname}", W); put(f"ib2.I.{kname}", I)
    W1, I1 = ib.get_ib_stencil(A(mx), A(my), GY, kernel=ib.kernel_peskin_3pt, stencil_radius=1)
    put("ib2.W.r1", W1); put("ib2.I.r1", I1)
    W, I = ib.get_ib_stencil(A(mx), A(my), GY)
    ugrid = (0.05 * rng.standard_normal((2, GX, GY))).astype(dt)
    put("ib2.ugrid", ugrid)
    put("ib2.interp", ib.interpolate(A(ugrid), W, I))
    Fm = (1e-2 * rng.standard_normal((M, 2))).astype(dt)
    grid0 = (1e-3 * rng.standard_normal((2, GX, GY))).astype(dt)
    put("ib2.Fm", Fm); put("ib2.grid0", grid0)
    put("ib2.spread", ib.spread(A(Fm), A(grid0), W, I))
    ut = (0.01 * rng.standard_normal((M, 2))).astype(dt)
    ds = (0.5 + rng.random(M)).astype(dt)
    put("ib2.ut", ut); put("ib2.ds", ds)
    gg, hh = ib.multi_direct_forcing(A(ugrid), W, I, A(ut), A(ds), n_iter=3)
    put("ib2.mdf.g", gg); put("ib2.mdf.h", hh)
    gg, hh = ib.multi_direct_forcing(A(ugrid), W, I, A(ut), 1.3, n_iter=5)
    put("ib2.mdf5.g", gg); put("ib2.mdf5.h", hh)
    put("ib2.ds_curve", ib.get_ds(A(np.stack([mx, my], axis=1))))
    put("ib2.ds_open", ib.get_ds(A(np.stack([mx, my], axis=1)), closed=False))

    G3 = (16, 14, 12)
    X3 = fibonacci_sphere(30, 3.3, (7.6, 6.9, 5.8)).astype(dt)
    put("ib3.X", X3)
    W3, I3 = ib3d.get_ib_stencil(A(X3), G3, kernel=ib3d.kernel_peskin_4pt)
    put("ib3.W", W3); put("ib3.I", I3)
    W3c, I3c = ib3d.get_ib_stencil(A(X3), G3, kernel=ib3d.kernel_cosine_4pt)
    put("ib3.W.cosine4", W3c); put("ib3.I.cosine4", I3c)
    u3g = (0.05 * rng.standard_normal((3,) + G3)).astype(dt)
    put("ib3.ugrid", u3g)
    put("ib3.interp", ib3d.interpolate(A(u3g), W3, I3))
    Fm3 = (1e-2 * rng.standard_normal((30, 3))).astype(dt)
    put("ib3.Fm", Fm3)
    put("ib3.spread", ib3d.spread(A(Fm3), jnp.zeros((3,) + G3, dtype=dt), W3, I3))
    ut3 = (0.01 * rng.standard_normal((30, 3))).astype(dt)
    put("ib3.ut", ut3)
    gg, hh = ib3d.multi_direct_forcing(A(u3g), W3, I3, A(ut3), 0.9, n_iter=3)
    put("ib3.mdf.g", gg); put("ib3.mdf.h", hh)

    # -------------------------------------------------------------------- dyn
    a, v, d, h = 0.01, -0.02, 0.3, 1.5
    put("dyn.scalar", np.array(dyn.newmark(a, v, d, h, 12.0, 3.0, 0.4), dtype=dt))
    av = np.array([1e-3, -2e-3], dtype=dt); vv = np.array([0.01, 0.02], dtype=dt)
    dv = np.array([0.5, -0.25], dtype=dt); hv = np.array([2.0, -1.0], dtype=dt)
    put("dyn.vec.in", np.stack([av, vv, dv, hv]))
    put("dyn.vec", np.stack(dyn.newmark(A(av), A(vv), A(dv), A(hv), 12.0, 3.0, 0.4)))
    m3 = np.diag([10.0, 11.0, 5.0]).astype(dt); k3 = np.array([[3, .1, 0], [.1, 2, 0], [0, 0, 1]], dtype=dt)
    c3 = np.diag([0.1, 0.2, 0.05]).astype(dt)
    a3 = np.array([1e-3, 2e-3, -1e-3], dtype=dt); v3 = np.array([.01, -.02, .003], dtype=dt)
    d3 = np.array([.1, .2, .05], dtype=dt); h3 = np.array([1.0, -0.5, 0.2], dtype=dt)
    put("dyn.mat.in", np.stack([a3, v3, d3, h3])); put("dyn.mat.m", m3); put("dyn.mat.k", k3); put("dyn.mat.c", c3)
    put("dyn.mat", np.stack(dyn.newmark(A(a3), A(v3), A(d3), A(h3), A(m3), A(k3), A(c3))))
    x2, y2 = dyn.get_markers_coords_2dof(A(mx), A(my), A(dv))
    put("dyn.coords2", np.stack([x2, y2]))
    x3, y3 = dyn.get_markers_coords_3dof(A(mx), A(my), 14.3, 11.7, A(d3))
    put("dyn.coords3", np.stack([x3, y3]))
    put("dyn.vel3", dyn.get_markers_velocity_3dof(x3, y3, 14.3, 11.7, A(d3), A(v3)))
    put("dyn.force", dyn.get_force_to_obj(A(Fm)))
    put("dyn.torque", dyn.get_torque_to_obj(x3, y3, 14.3, 11.7, A(d3), A(Fm)))

    # --------------------------------------------------------------- recipes
    recipes_2d(put, jnp, lbm, ib, dyn, dt, rng)
    recipes_3d(put, jnp, lbm3d, ib3d, dt, rng)
    post_golden(put, jnp, dt)
    refine_golden(put, jnp, lbm, dt)
    cbc_golden(put, jnp, lbm, lbm3d, dt)
    return G


POST_FIELDS = ("velocity_magnitude", "velocity_gradient", "vorticity", "vorticity_magnitude", "divergence",
               "strain_rate", "strain_rate_magnitude", "kinetic_energy", "mean_kinetic_energy", "enstrophy",
               "mean_enstrophy", "q_criterion")


def post_golden(put, jnp, dt):
    """vivsim/post.py on random 2-D and 3-D velocity fields (its own seed, so the other
    vectors do not move)."""
    from vivsim import post
    rng = np.random.default_rng(777)
    u2 = rng.normal(0.0, 0.05, (2, 12, 10)).astype(dt)
    u3 = rng.normal(0.0, 0.05, (3, 8, 7, 6)).astype(dt)
    rho = (1 + 0.01 * rng.normal(0.0, 1.0, (12, 10))).astype(dt)
    for tag, u in (("p2", u2), ("p3", u3)):
        put(f"{tag}.u", u)
        for name in POST_FIELDS:
            put(f"{tag}.{name}", getattr(post, name)(jnp.asarray(u)))
    put("p.rho", rho)
    put("p.pressure", post.pressure(jnp.asarray(rho)))


REFINE_SHAPES = {  # (fine, coarse) populations shapes per direction, plus a broadcast case
    "left": ((9, 5, 12), (9, 7, 6)), "right": ((9, 4, 10), (9, 6, 5)),
    "up": ((9, 12, 5), (9, 6, 7)), "down": ((9, 10, 3), (9, 5, 4)),
}


def refine_golden(put, jnp, lbm, dt):
    """vivsim/multigrid.py: the two transfers in every direction, get_omega over levels, and
    a two-level channel run of the transfers (its own seed, so the other vectors do not move).
    The channel's order of operations restates oracle/recipes.py:refined_channel_cycle: the
    reference ships the transfers without a driver."""
    from vivsim import multigrid as mg
    rng = np.random.default_rng(4242)
    for d, (sf, sc) in REFINE_SHAPES.items():
        ff = rng.uniform(0.0, 0.2, sf).astype(dt)
        fc = rng.uniform(0.0, 0.2, sc).astype(dt)
        put(f"mg.{d}.ff", ff)
        put(f"mg.{d}.fc", fc)
        put(f"mg.{d}.f2c", mg.fine_to_coarse(jnp.asarray(ff), jnp.asarray(fc), d))
        put(f"mg.{d}.c2f", mg.coarse_to_fine(jnp.asarray(fc), jnp.asarray(ff), d))
    # a coarse line of length 1 broadcasts onto every fine node
    ff = rng.uniform(0.0, 0.2, (9, 3, 7)).astype(dt)
    fc = rng.uniform(0.0, 0.2, (9, 4, 1)).astype(dt)
    put("mg.bc.ff", ff)
    put("mg.bc.fc", fc)
    put("mg.bc.c2f", mg.coarse_to_fine(jnp.asarray(fc), jnp.asarray(ff), "right"))
    put("mg.omega", np.array([mg.get_omega(nu, lv) for nu in (0.004, 0.02, 0.1) for lv in (-2, -1, 0, 1, 2, 3)]))
    put("mg.init", np.array([mg.init_grid(w, h, lv, bx, by)[0].shape[1:] for w, h, lv, bx, by in
                             ((16, 8, 0, 1, 0), (16, 8, 1, 0, 0), (16, 8, -1, 0, 2), (10, 6, 2, 1, 1))]))
    # two-level channel: coarse 16 x 16 (+1 buffer column), fine 8 x 16 at level 1
    nu, u0, H = 0.02, 0.05, 16
    om_c, om_f = mg.get_omega(nu, 0), mg.get_omega(nu, 1)
    uc = np.zeros((2, 17, H), dt)
    uc[0] = u0
    uc[1] = rng.normal(0.0, 1e-3, (17, H))
    uf = np.zeros((2, 16, 2 * H), dt)
    uf[0] = u0
    uf[1] = rng.normal(0.0, 1e-3, (16, 2 * H))
    fc = lbm.get_equilibrium(jnp.ones((17, H), dtype=dt), jnp.asarray(uc))
    ff = lbm.get_equilibrium(jnp.ones((16, 2 * H), dtype=dt), jnp.asarray(uf))
    put("rc.fc0", fc)
    put("rc.ff0", ff)
    put("rc.omega", np.array([om_c, om_f, u0]))
    for s in range(6):
        rho, u = lbm.get_macroscopic(fc)
        fc = lbm.streaming(lbm.collision_bgk(fc, lbm.get_equilibrium(rho, u), om_c))
        fc = lbm.boundary_equilibrium(fc, "left", ux_wall=u0)
        for _ in range(2):
            rho, u = lbm.get_macroscopic(ff)
            ff = lbm.streaming(lbm.collision_bgk(ff, lbm.get_equilibrium(rho, u), om_f))
            ff = mg.coarse_to_fine(fc, ff, "right")
            ff = lbm.boundary_pressure_nee(ff, "right")
        fc = mg.fine_to_coarse(ff, fc, "left")
        if s in (0, 5):
            put(f"rc.fc{s + 1}", fc)
            put(f"rc.ff{s + 1}", ff)


def cbc_golden(put, jnp, lbm, lbm3d, dt):
    """Channels whose outflow takes its wall state from boundary_characteristic
    (lbm/boundary/cbc.py:14-53, lbm3d/boundary/cbc.py:16-51) of the step's input moments and
    imposes it with NEE / equilibrium / NEBB (its own seed, so the other vectors do not
    move).  The reference uses the condition in no example; this recipe takes the moments
    the step already has (get_macroscopic before colliding)."""
    rng = np.random.default_rng(9090)
    nu, u0 = 0.02, 0.05
    om = lbm.get_omega(nu)
    nx, ny = 24, 16
    rho0 = (1 + 0.02 * rng.normal(0.0, 1.0, (nx, ny))).astype(dt)
    u = np.zeros((2, nx, ny), dt)
    u[0] = u0 + 0.01 * rng.normal(0.0, 1.0, (nx, ny))
    u[1] = 0.01 * rng.normal(0.0, 1.0, (nx, ny))
    f0 = lbm.get_equilibrium(jnp.asarray(rho0), jnp.asarray(u))
    put("cbc2.f0", f0)
    put("cbc2.omega", np.array([om, u0]))
    for scheme in ("nee", "eq", "nebb"):
        wall = {"nee": lbm.boundary_nee, "eq": lbm.boundary_equilibrium, "nebb": lbm.boundary_nebb}[scheme]
        f = f0
        for step in range(1, 9):
            rho, uu = lbm.get_macroscopic(f)
            f = lbm.streaming(lbm.collision_kbc(f, lbm.get_equilibrium(rho, uu), om))
            f = lbm.boundary_equilibrium(f, "left", ux_wall=u0)
            rn, un = lbm.boundary_characteristic(rho, uu, "right")
            f = wall(f, "right", rho_wall=rn, ux_wall=un[0], uy_wall=un[1])
            if step in (1, 8):
                put(f"cbc2.{scheme}.f{step}", f)
    nx, ny, nz = 12, 8, 8
    rho0 = (1 + 0.02 * rng.normal(0.0, 1.0, (nx, ny, nz))).astype(dt)
    u = np.zeros((3, nx, ny, nz), dt)
    u[0] = u0 + 0.01 * rng.normal(0.0, 1.0, (nx, ny, nz))
    u[1:] = 0.01 * rng.normal(0.0, 1.0, (2, nx, ny, nz))
    f = lbm3d.get_equilibrium(jnp.asarray(rho0), jnp.asarray(u))
    put("cbc3.f0", f)
    for step in range(1, 5):
        rho, uu = lbm3d.get_macroscopic(f)
        f = lbm3d.streaming(lbm3d.collision_bgk(f, lbm3d.get_equilibrium(rho, uu), om))
        f = lbm3d.boundary_equilibrium(f, "left", ux_wall=u0)
        rn, un = lbm3d.boundary_characteristic(rho, uu, "right")
        f = lbm3d.boundary_nee(f, "right", rho_wall=rn, ux_wall=un[0], uy_wall=un[1], uz_wall=un[2])
        if step in (1, 4):
            put(f"cbc3.f{step}", f)


def recipes_2d(put, jnp, lbm, ib, dyn, dt, rng):
    # Lid-driven cavity, examples/2d/lid_driven_cavity.py:55-63 (BGK + four NEE walls)
    nx, ny, nu, ulid = 16, 12, 0.0256, 0.1
    om = lbm.get_omega(nu)
    f = lbm.get_equilibrium(jnp.ones((nx, ny)), jnp.zeros((2, nx, ny)))
    put("cav.f0", f)
    for step in range(1, 31):
        rho, u = lbm.get_macroscopic(f)
        feq = lbm.get_equilibrium(rho, u)
        f = lbm.collision_bgk(f, feq, om)
        f = lbm.streaming(f)
        f = lbm.boundary_nee(f, loc="top", ux_wall=ulid)
        f = lbm.boundary_nee(f, loc="left")
        f = lbm.boundary_nee(f, loc="right")
        f = lbm.boundary_nee(f, loc="bottom")
        if step in (1, 10, 30):
            put(f"cav.f{step}", f)

    # Cylinder VIV, examples/2d/vortex_induced_vibration.py:96-148 with a full-grid
    # stencil, equilibrium inflow and pressure-NEE outflow, transverse (y) spring only.
    nx, ny, D, U0, Re, M = 40, 24, 8.0, 0.05, 20.0, 24
    nu = U0 * D / Re
    om = lbm.get_omega(nu)
    cx, cy = 12.0, 12.0
    th = jnp.linspace(0, 2 * jnp.pi, M, endpoint=False)
    X0 = cx + 0.5 * D * jnp.cos(th)
    Y0 = cy + 0.5 * D * jnp.sin(th)
    ds = math.pi * D / M
    area = math.pi * (D / 2) ** 2
    mass = area * 10.0
    fn = U0 / (5.0 * D)
    K = (2 * math.pi * fn) ** 2 * mass * (1 + 1 / 10.0)
    put("viv.X0", X0); put("viv.Y0", Y0)
    pert = (1e-4 * rng.standard_normal((nx, ny))).astype(dt)
    put("viv.pert", pert)
    for coll in ("kbc", "mrt", "reg", "bgk"):
        u = jnp.zeros((2, nx, ny))
        u = u.at[0].set(U0)
        u = u.at[1].set(jnp.asarray(pert))
        f = lbm.get_equilibrium(jnp.ones((nx, ny)), u)
        d = jnp.zeros(2); v = jnp.zeros(2); a = jnp.zeros(2)
        mrt_op = lbm.get_mrt_collision_operator(om)
        for step in range(1, 7):
            rho, u = lbm.get_macroscopic(f)
            feq = lbm.get_equilibrium(rho, u)
            if coll == "kbc":
                f = lbm.collision_kbc(f, feq, om)
            elif coll == "mrt":
                f = lbm.collision_mrt(f, feq, mrt_op)
            elif coll == "reg":
                f = lbm.collision_reg(f, feq, om)
            else:
                f = lbm.collision_bgk(f, feq, om)
            mxx, myy = dyn.get_markers_coords_2dof(X0, Y0, d)
            W, I = ib.get_ib_stencil(mxx, myy, ny, kernel=ib.kernel_peskin_4pt, stencil_radius=2)
            mv = jnp.repeat(v[None, :], M, axis=0)
            g, mh = ib.multi_direct_forcing(u, W, I, mv, ds, n_iter=3)
            h = dyn.get_force_to_obj(mh)
            h += a * area
            ay, vy, dy = dyn.newmark(a[1], v[1], d[1], h[1], mass, K, 0.0)
            a = jnp.zeros(2).at[1].set(ay)
            v = jnp.zeros(2).at[1].set(vy)
            d = jnp.zeros(2).at[1].set(dy)
            f = lbm.forcing_edm(f, g, u)
            f = lbm.streaming(f)
            f = lbm.boundary_equilibrium(f, loc="left", ux_wall=U0)
            f = lbm.boundary_pressure_nee(f, loc="right", rho_wall=1.0)
            if step == 1:
                rr, uu = lbm.get_macroscopic(f)
                put(f"viv.{coll}.rho1", rr); put(f"viv.{coll}.u1", uu)
            if step in (1, 6):
                if step == 6:
                    put(f"viv.{coll}.f{step}", f)
                put(f"viv.{coll}.h{step}", h)
                put(f"viv.{coll}.body{step}", jnp.stack([a, v, d]))

    # Fluid-structure sub-iterations, examples/2d/vortex_induced_vibration.py:111-139 with
    # FSI_ITER = 2: each pass places the markers with the latest (a, v, d) and restarts the
    # 2-DOF Newmark update from the step's saved state.  Full-grid stencil, KBC, equilibrium
    # inflow, pressure-NEE outflow, both translations free.
    u = jnp.zeros((2, nx, ny))
    u = u.at[0].set(U0)
    u = u.at[1].set(jnp.asarray(pert))
    f = lbm.get_equilibrium(jnp.ones((nx, ny)), u)
    d = jnp.zeros(2); v = jnp.zeros(2).at[1].set(1e-2 * U0); a = jnp.zeros(2)
    for step in range(1, 7):
        rho, u = lbm.get_macroscopic(f)
        feq = lbm.get_equilibrium(rho, u)
        f = lbm.collision_kbc(f, feq, om)
        a_old, v_old, d_old = a, v, d
        for _ in range(2):
            mxx, myy = dyn.get_markers_coords_2dof(X0, Y0, d)
            W, I = ib.get_ib_stencil(mxx, myy, ny, kernel=ib.kernel_peskin_4pt, stencil_radius=2)
            mv = jnp.repeat(v[None, :], M, axis=0)
            g, mh = ib.multi_direct_forcing(u, W, I, mv, ds, n_iter=3)
            h = dyn.get_force_to_obj(mh)
            h += a * area
            a, v, d = dyn.newmark_2dof(a_old, v_old, d_old, h, mass, K, 0.0)
        f = lbm.forcing_edm(f, g, u)
        f = lbm.streaming(f)
        f = lbm.boundary_equilibrium(f, loc="left", ux_wall=U0)
        f = lbm.boundary_pressure_nee(f, loc="right", rho_wall=1.0)
        if step in (1, 6):
            put(f"vivfsi.f{step}", f)
            put(f"vivfsi.h{step}", h)
            put(f"vivfsi.body{step}", jnp.stack([a, v, d]))

    # Windowed IB region as in examples/2d/vortex_induced_vibration.py:104-146 (2-DOF,
    # force-corrected NEBB inflow, equilibrium outflow, dynamic window).
    nx, ny, D, U0 = 40, 28, 8.0, 0.05
    om = lbm.get_omega(U0 * D / 30.0)
    cx, cy, pad = 13.0, 14.0, 3
    M = 24
    th = jnp.linspace(0, 2 * jnp.pi, M, endpoint=False)
    X0 = cx + 0.5 * D * jnp.cos(th)
    Y0 = cy + 0.5 * D * jnp.sin(th)
    ds = math.pi * D / M
    area = math.pi * (D / 2) ** 2
    mass = area * 5.0
    K = 2e-3
    x0i, y0i = int(cx - 0.5 * D - pad), int(cy - 0.5 * D - pad)
    S = int(D + 2 * pad)
    u = jnp.zeros((2, nx, ny)).at[0].set(U0)
    f = lbm.get_equilibrium(jnp.ones((nx, ny)), u)
    d = jnp.zeros(2); v = jnp.zeros(2).at[1].set(1e-2 * U0); a = jnp.zeros(2)
    for step in range(1, 7):
        rho, u = lbm.get_macroscopic(f)
        feq = lbm.get_equilibrium(rho, u)
        f = lbm.collision_reg(f, feq, om)
        ibx = (x0i + d[0]).astype(jnp.int32)
        iby = (y0i + d[1]).astype(jnp.int32)
        import jax
        ib_u = jax.lax.dynamic_slice(u, (0, ibx, iby), (2, S, S))
        ib_f = jax.lax.dynamic_slice(f, (0, ibx, iby), (9, S, S))
        mxx, myy = dyn.get_markers_coords_2dof(X0, Y0, d)
        W, I = ib.get_ib_stencil(mxx - ibx, myy - iby, S)
        mv = jnp.repeat(v[None, :], M, axis=0)
        g, mh = ib.multi_direct_forcing(ib_u, W, I, mv, ds, n_iter=1)
        h = dyn.get_force_to_obj(mh)
        h += a * area
        a, v, d = dyn.newmark(a, v, d, h, mass, K, 0.0)
        ib_f = lbm.forcing_edm(ib_f, g, ib_u)
        f = jax.lax.dynamic_update_slice(f, ib_f, (0, ibx, iby))
        f = lbm.streaming(f)
        f = lbm.boundary_force_corrected_nebb(f, loc="left", ux_wall=U0)
        f = lbm.boundary_equilibrium(f, loc="right", ux_wall=U0)
    put("vivw.f6", f); put("vivw.h6", h); put("vivw.body6", jnp.stack([a, v, d]))


def recipes_3d(put, jnp, lbm3d, ib3d, dt, rng):
    # Fixed sphere, examples/3d/flow_past_sphere.py:139-180 with a full-grid static
    # stencil, equilibrium inflow and pressure-NEE outflow.
    nx, ny, nz, D, U0, Re, M = 16, 12, 12, 5.0, 0.05, 30.0, 79
    om = lbm3d.get_omega(U0 * D / Re)
    X = fibonacci_sphere(M, D / 2, (6.2, 6.1, 5.9)).astype(dt)
    ds = 4 * math.pi * (D / 2) ** 2 / M
    put("sph.X", X)
    W, I = ib3d.get_ib_stencil(jnp.asarray(X), (nx, ny, nz), kernel=ib3d.kernel_peskin_4pt)
    pert = (1e-4 * rng.standard_normal((3, nx, ny, nz))).astype(dt)
    put("sph.pert", pert)
    for coll in ("reg", "bgk", "kbc"):
        u = jnp.asarray(pert)
        u = u.at[0].add(U0)
        f = lbm3d.get_equilibrium(jnp.ones((nx, ny, nz)), u)
        for step in range(1, 5):
            rho, u = lbm3d.get_macroscopic(f)
            feq = lbm3d.get_equilibrium(rho, u)
            if coll == "reg":
                f = lbm3d.collision_reg(f, feq, om)
            elif coll == "kbc":
                f = lbm3d.collision_kbc(f, feq, om)
            else:
                f = lbm3d.collision_bgk(f, feq, om)
            g, mh = ib3d.multi_direct_forcing(u, W, I, jnp.zeros((M, 3)), ds, n_iter=3)
            f = lbm3d.forcing_edm(f, g, u)
            f = lbm3d.streaming(f)
            f = lbm3d.boundary_equilibrium(f, loc="left", ux_wall=U0)
            f = lbm3d.boundary_pressure_nee(f, loc="right", rho_wall=1.0)
            if step == 1:
                rr, uu = lbm3d.get_macroscopic(f)
                put(f"sph.{coll}.rho1", rr); put(f"sph.{coll}.u1", uu)
            if step in (1, 4):
                if step == 4:
                    put(f"sph.{coll}.f{step}", f)
                put(f"sph.{coll}.h{step}", jnp.sum(mh, axis=0))


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--reference", required=True, help="checkout of haimingz/vivsim")
    args = ap.parse_args()
    sys.path.insert(0, os.path.join(HERE, "_jaxshim"))
    sys.path.insert(0, args.reference)
    warnings.filterwarnings("ignore", category=RuntimeWarning)
    import jax
    import jax.numpy as jnp
    from vivsim import dyn, ib, ib3d, lbm, lbm3d

    for mode in ("f32", "f64"):
        G = generate(mode, jax, jnp, lbm, lbm3d, ib, ib3d, dyn)
        path = os.path.join(HERE, f"golden_{mode}.npz")
        np.savez_compressed(path, **G)
        print(f"wrote {path}: {len(G)} arrays, {os.path.getsize(path) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
