"""Composed IB-LBM time steps built from the oracle operators (test infrastructure only).

Each recipe chains the oracle functions in the order of the reference's example
``update_step`` it cites.  The reference itself has no driver: users write this
sequence inside ``jax.jit`` + ``lax.scan``.
"""

import math

import numpy as np

from . import dyn, ib
from . import lbm2d as L2
from . import lbm3d as L3

_BC2 = {
    "nee": L2.boundary_nee, "nebb": L2.boundary_nebb, "eq": L2.boundary_equilibrium,
    "vnee": L2.boundary_velocity_nee, "vnebb": L2.boundary_velocity_nebb,
    "veq": L2.boundary_velocity_equilibrium, "pnee": L2.boundary_pressure_nee,
    "pnebb": L2.boundary_pressure_nebb, "peq": L2.boundary_pressure_equilibrium,
    "fcnee": L2.boundary_force_corrected_nee, "fcnebb": L2.boundary_force_corrected_nebb,
    "fceq": L2.boundary_force_corrected_equilibrium,
}
_BC3 = {
    "nee": L3.boundary_nee, "nebb": L3.boundary_nebb, "eq": L3.boundary_equilibrium,
    "vnee": L3.boundary_velocity_nee, "vnebb": L3.boundary_velocity_nebb,
    "veq": L3.boundary_velocity_equilibrium, "pnee": L3.boundary_pressure_nee,
    "pnebb": L3.boundary_pressure_nebb, "peq": L3.boundary_pressure_equilibrium,
    "fcnee": L3.boundary_force_corrected_nee, "fcnebb": L3.boundary_force_corrected_nebb,
    "fceq": L3.boundary_force_corrected_equilibrium,
}


def _collide(L, f, feq, kind, omega, mrt_op):
    if kind == "bgk":
        return L.collision_bgk(f, feq, omega)
    if kind == "kbc":
        return L.collision_kbc(f, feq, omega)
    if kind == "reg":
        return L.collision_reg(f, feq, omega)
    if kind == "mrt":
        return L.collision_mrt(f, feq, mrt_op)
    raise ValueError(kind)


def _apply_bcs(L, table, f_post, f, bcs, moments=None):
    """Face boundaries in order.  ``("cbc", loc, {"scheme": s})`` is a characteristic outflow:
    the wall state from boundary_characteristic of the step's input moments (rho, u),
    imposed by scheme s ("nee", "nebb" or "eq")."""
    for name, loc, kw in bcs:
        if name == "cbc":
            rho, u = moments
            rn, un = L.boundary_characteristic(rho, u, loc)
            vel = dict(ux_wall=un[0], uy_wall=un[1])
            if un.shape[0] == 3:
                vel["uz_wall"] = un[2]
            f = table[kw["scheme"]](f, loc, rho_wall=rn, **vel)
        elif name == "bb":
            f = L.boundary_bounce_back(f_post, f, loc, **kw)
        elif name == "spec":
            f = L.boundary_specular_reflection(f_post, f, loc, **kw)
        else:
            f = table[name](f, loc, **kw)
    return f


def cavity_step(f, omega, u_lid):
    """examples/2d/lid_driven_cavity.py:55-63: BGK, stream, NEE top(lid)/left/right/bottom."""
    rho, u = L2.get_macroscopic(f)
    f = L2.collision_bgk(f, L2.get_equilibrium(rho, u), omega)
    f = L2.streaming(f)
    f = L2.boundary_nee(f, "top", ux_wall=u_lid)
    f = L2.boundary_nee(f, "left")
    f = L2.boundary_nee(f, "right")
    return L2.boundary_nee(f, "bottom")


def lbm_step_2d(f, collision, omega=None, mrt_op=None, bcs=(), g=None, forcing="edm"):
    """Plain D2Q9 step with an optional body-force field (examples/2d/poiseuille_channel.py:82-143)."""
    rho, u = L2.get_macroscopic(f)
    moments = (rho, u)  # a characteristic wall reads get_macroscopic's u, before any correction
    if g is not None and forcing in ("guo_bgk", "guo_mrt"):
        u = u + L2.get_velocity_correction(g, rho)
    feq = L2.get_equilibrium(rho, u)
    f = _collide(L2, f, feq, collision, omega, mrt_op)
    if g is not None:
        if forcing == "edm":
            f = L2.forcing_edm(f, g, u)
        elif forcing == "guo_bgk":
            f = L2.forcing_guo_bgk(f, g, u, omega)
        else:
            f = L2.forcing_guo_mrt(f, g, u, L2.get_mrt_forcing_operator(omega, f.dtype))
    f_post = f
    f = L2.streaming(f)
    return _apply_bcs(L2, _BC2, f_post, f, bcs, moments)


class Body2D:
    """Rigid body carried between steps: markers relative to a displacement d.

    ``free`` has two entries (x, y translation) or three; a free third DOF is the rotation
    angle about ``center`` (dyn.get_markers_coords_3dof), integrated with ``inertia``,
    ``rot_k``, ``rot_c`` and the added inertia ``rot_added``.  ``fsi_iter`` is the number of
    fluid-structure sub-iterations per step (examples/2d/vortex_induced_vibration.py:114-139).
    """

    def __init__(self, X0, Y0, ds, mass, stiffness, damping, area, free=(False, True),
                 kernel="peskin4", radius=2, n_iter=3, d=None, v=None, a=None, center=None, inertia=0.0,
                 rot_k=0.0, rot_c=0.0, rot_added=0.0, fsi_iter=1):
        self.fsi_iter = int(fsi_iter)
        self.X0, self.Y0 = np.asarray(X0), np.asarray(Y0)
        self.ds, self.mass, self.k, self.c, self.area = ds, mass, stiffness, damping, area
        self.free = tuple(bool(x) for x in free)
        self.rot = len(self.free) > 2 and self.free[2]
        self.center = center
        self.inertia, self.rot_k, self.rot_c, self.rot_added = inertia, rot_k, rot_c, rot_added
        self.kernel, self.radius, self.n_iter = kernel, radius, n_iter
        dt = self.X0.dtype
        nd = 3 if self.rot else 2
        self.d = np.zeros(nd, dt) if d is None else np.asarray(d, dt)
        self.v = np.zeros(nd, dt) if v is None else np.asarray(v, dt)
        self.a = np.zeros(nd, dt) if a is None else np.asarray(a, dt)


def ib_lbm_step_2d(f, body, collision, omega=None, mrt_op=None, bcs=()):
    """One VIV step, examples/2d/vortex_induced_vibration.py:96-148.

    Full-grid stencil (the IB window of the example covers the whole grid); the free
    degrees of freedom of ``body`` advance with Newmark, fixed ones stay zero.
    Returns ``(f_next, h)`` and updates ``body`` in place.
    """
    ny = f.shape[2]
    rho, u = L2.get_macroscopic(f)
    feq = L2.get_equilibrium(rho, u)
    f = _collide(L2, f, feq, collision, omega, mrt_op)
    g, h = body_forces_2d(u, body, ny)
    f = L2.forcing_edm(f, g, u)
    f_post = f
    f = L2.streaming(f)
    return _apply_bcs(L2, _BC2, f_post, f, bcs, (rho, u)), h


def body_forces_2d(u, body, ny):
    """The immersed-boundary part of ib_lbm_step_2d (examples/2d/vortex_induced_vibration.py:
    108-141): marker kinematics, stencil, MDF, body force (and torque) and the Newmark
    update of ``body``, repeated ``body.fsi_iter`` times: each pass places the markers with
    the latest state and restarts Newmark from the step's saved one (:111-139).  Returns the
    last pass's grid force g and body force h."""
    M = body.X0.shape[0]
    a_old, v_old, d_old = body.a, body.v, body.d
    a, v, d = a_old, v_old, d_old
    for _ in range(body.fsi_iter):
        if body.rot:  # markers turn with d[2] about the initial centre (dyn.py:84-120)
            cx, cy = body.center
            mx, my = dyn.get_markers_coords_3dof(body.X0, body.Y0, cx, cy, d)
            mv = dyn.get_markers_velocity_3dof(mx, my, cx, cy, d, v)
        else:
            mx, my = dyn.get_markers_coords_2dof(body.X0, body.Y0, d)
            mv = np.repeat(v[None, :], M, axis=0)
        W, I = ib.get_ib_stencil(mx, my, ny, ib.KERNELS[body.kernel], body.radius)
        g, mh = ib.multi_direct_forcing(u, W, I, mv, body.ds, body.n_iter)
        h = dyn.get_force_to_obj(mh)
        h = h + a[:2] * body.area
        if body.rot:  # torque (dyn.py:139-154) plus added inertia
            tq = dyn.get_torque_to_obj(mx, my, cx, cy, d, mh)
            h = np.concatenate([h, np.asarray([tq + a[2] * body.rot_added], h.dtype)])
        a, v, d = a_old.copy(), v_old.copy(), d_old.copy()
        for k in range(len(body.d)):
            if body.free[k]:
                m, kk, c = (body.mass, body.k, body.c) if k < 2 else (body.inertia, body.rot_k, body.rot_c)
                a[k], v[k], d[k] = dyn.newmark(a_old[k], v_old[k], d_old[k], h[k], m, kk, c)
    body.a, body.v, body.d = a, v, d
    return g, h


def lbm_step_3d(f, collision, omega=None, mrt_op=None, bcs=()):
    """Plain D3Q19 step (examples/3d/abc_flow.py update loop)."""
    rho, u = L3.get_macroscopic(f)
    f = _collide(L3, f, L3.get_equilibrium(rho, u), collision, omega, mrt_op)
    f_post = f
    f = L3.streaming(f)
    return _apply_bcs(L3, _BC3, f_post, f, bcs, (rho, u))


def ib_lbm_step_3d(f, W, I, marker_u, ds, collision, omega=None, mrt_op=None, bcs=(), n_iter=3):
    """Fixed-body 3D step with a static stencil, examples/3d/flow_past_sphere.py:139-180.

    Returns ``(f_next, h)`` with ``h`` the total force on the body.
    """
    rho, u = L3.get_macroscopic(f)
    f = _collide(L3, f, L3.get_equilibrium(rho, u), collision, omega, mrt_op)
    g, mh = ib.multi_direct_forcing(u, W, I, marker_u, ds, n_iter)
    f = L3.forcing_edm(f, g, u)
    f_post = f
    f = L3.streaming(f)
    h = mh[0].copy()
    for i in range(1, mh.shape[0]):
        h = h + mh[i]
    return _apply_bcs(L3, _BC3, f_post, f, bcs, (rho, u)), h


def fibonacci_sphere(n, radius, center):
    """Marker cloud on a sphere: golden-angle spiral, equal area per marker."""
    k = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * k / n)
    theta = math.pi * (1 + 5 ** 0.5) * k
    return np.stack([center[0] + radius * np.cos(theta) * np.sin(phi),
                     center[1] + radius * np.sin(theta) * np.sin(phi),
                     center[2] + radius * np.cos(phi)], axis=1)


def refined_channel_cycle(fc, ff, omega_c, omega_f, u0):
    """One coarse step of a two-level channel built from vivsim/multigrid.py's transfers.

    The coarse block (level 0, one buffer column on its right) has the equilibrium inflow
    ux = u0 on its left; the fine block (level 1) continues it to the right and ends in a
    pressure-NEE outflow; y is periodic in both.  The reference ships the transfers but no
    driver that uses them, so the order is this recipe's: the coarse block steps
    (collide, stream, inflow); the fine block takes two steps, each followed by
    coarse_to_fine(.., 'right') from the new coarse state and the outflow; then
    fine_to_coarse(.., 'left') refills the coarse buffer column.
    """
    from . import multigrid as mg
    rho, u = L2.get_macroscopic(fc)
    fc = L2.streaming(L2.collision_bgk(fc, L2.get_equilibrium(rho, u), omega_c))
    fc = L2.boundary_equilibrium(fc, "left", ux_wall=u0)
    for _ in range(2):
        rho, u = L2.get_macroscopic(ff)
        ff = L2.streaming(L2.collision_bgk(ff, L2.get_equilibrium(rho, u), omega_f))
        ff = mg.coarse_to_fine(fc, ff, "right")
        ff = L2.boundary_pressure_nee(ff, "right")
    return mg.fine_to_coarse(ff, fc, "left"), ff
