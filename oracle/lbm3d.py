"""D3Q19 operators — NumPy restatement of vivsim/lbm3d (test infrastructure only).

Arrays are SoA, C-order ``(19, NX, NY, NZ)``.  Contractions the reference writes as
``einsum`` are written as explicit sums in population order.
"""

import numpy as np

from .lattice import Q19_C, Q19_CS2, Q19_FACES, Q19_OPP, Q19_W


def _seq(terms):
    out = terms[0]
    for t in terms[1:]:
        out = out + t
    return out


def _w(dt, ndim):
    return Q19_W.astype(dt).reshape((19,) + (1,) * ndim)


# ------------------------------------------------------------------ basic ops

def streaming(f):
    """Periodic D3Q19 shift by c_i (vivsim/lbm3d/basic.py:52-87)."""
    out = np.empty_like(f)
    for i in range(19):
        out[i] = np.roll(f[i], shift=tuple(int(v) for v in Q19_C[i]), axis=(0, 1, 2))
    return out


def get_macroscopic(f):
    """rho = sum f; u = c^T f / rho (lbm3d/basic.py:90-106)."""
    rho = _seq([f[i] for i in range(19)])
    mom = []
    for d in range(3):
        terms = [f[i] if Q19_C[i, d] > 0 else -f[i] for i in range(19) if Q19_C[i, d] != 0]
        mom.append(_seq(terms))
    u = np.stack(mom) / rho[None]
    return rho, u


def _uc(u, dt):
    """uc_q = sum_d c_qd u_d, in d order (the einsum of lbm3d/basic.py:121)."""
    out = []
    for q in range(19):
        acc = None
        for d in range(3):
            cq = int(Q19_C[q, d])
            if cq == 0:
                continue
            t = u[d] if cq > 0 else -u[d]
            acc = t if acc is None else acc + t
        out.append(np.zeros_like(u[0]) if acc is None else acc)
    return np.stack(out).astype(dt, copy=False)


def get_equilibrium(rho, u):
    """feq = rho w (1 + cu/cs2 + (cu)^2/(2 cs2^2) - u^2/(2 cs2)) (lbm3d/basic.py:109-130)."""
    dt = np.result_type(rho, u)
    ndim = np.ndim(rho)
    uc = _uc(u, dt)
    usq = (u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]
    return (rho[None] * _w(dt, ndim)) * (
        ((1 + uc / Q19_CS2) + (0.5 * (uc * uc)) / (Q19_CS2 ** 2)) - (0.5 * usq[None]) / Q19_CS2)


def collision_bgk(f, feq, omega):
    """(1 - omega) f + omega feq (lbm3d/basic.py:133-146)."""
    return (1 - omega) * f + omega * feq


def get_omega(nu):
    """(lbm3d/basic.py:149-152)."""
    return 1 / (3 * nu + 0.5)


def get_velocity_correction(g, rho=1):
    """(lbm3d/basic.py:155-167)."""
    return g * 0.5 / rho


# ---------------------------------------------------- second-order projection
# vivsim/lbm3d/collision/reg.py:10-32 declares this 19x19 float32 matrix literally.  It
# is the Hermite projector P_qr = w_q / (2 cs^4) (c_qa c_qb - cs^2 d_ab)(c_ra c_rb - ...)
# restricted to the entries the reference lists; rebuilt here from that formula and
# rounded to float32 like the reference's table.

def _projection_table():
    c = Q19_C.astype(np.float64)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    cs2 = 1.0 / 3.0
    P = np.zeros((19, 19))
    for q in range(19):
        Hq = np.outer(c[q], c[q]) - cs2 * np.eye(3)
        for r in range(19):
            Hr = np.outer(c[r], c[r])
            P[q, r] = w[q] / (2 * cs2 * cs2) * np.sum(Hq * Hr)
    return P.astype(np.float32)


SECOND_ORDER_PROJECTION = _projection_table()


def get_second_order_projection(fneq):
    """P fneq, summed over r in population order (lbm3d/collision/reg.py:35-41)."""
    P = SECOND_ORDER_PROJECTION.astype(fneq.dtype)
    return np.stack([_seq([P[q, r] * fneq[r] for r in range(19)]) for q in range(19)])


def collision_reg(f, feq, omega):
    """feq + (1 - omega) P fneq (lbm3d/collision/reg.py:44-62)."""
    return feq + (1 - omega) * get_second_order_projection(f - feq)


def collision_kbc(f, feq, omega):
    """KBC with the second-order projection as shear part (lbm3d/collision/kbc.py:8-42)."""
    fneq = f - feq
    shear = get_second_order_projection(fneq)
    high = fneq - shear
    inv_feq = 1.0 / (feq + 1e-20)
    inner_sh = _seq([(high[i] * shear[i]) * inv_feq[i] for i in range(19)])
    inner_hh = _seq([(high[i] * high[i]) * inv_feq[i] for i in range(19)])
    half_gamma = 1.0 / omega - ((1.0 - 1.0 / omega) * inner_sh) / (inner_hh + 1e-20)
    return f - omega * (shear + half_gamma[None] * high)


# MRT basis, lbm3d/collision/mrt.py:7-29
MRT_M = np.array([
    [1] * 19,
    [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
    [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1],
    [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1],
    [0, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2],
    [0, 2, 2, -1, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2],
    [0, 0, 0, 1, 1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1],
    [0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1],
    [0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1],
], dtype=np.float32)
MRT_M_INV = np.linalg.inv(MRT_M)


def get_mrt_relaxation_diag(omega):
    """Diagonal of S (lbm3d/collision/mrt.py:34-77)."""
    return [0.0, 0.0, 0.0, 0.0, 1.1] + [omega] * 5 + [1.2] * 6 + [1.4] * 3


def get_mrt_collision_operator(omega, dtype=np.float32):
    """M^-1 S M in ``dtype`` (lbm3d/collision/mrt.py:80-85)."""
    dt = np.dtype(dtype)
    S = np.diag(np.array(get_mrt_relaxation_diag(omega), dtype=dt))
    return (MRT_M_INV.astype(dt) @ S) @ MRT_M.astype(dt)


def get_mrt_forcing_operator(omega, dtype=np.float32):
    """M^-1 (I - S/2) M (lbm3d/forcing/guo.py:58-68)."""
    dt = np.dtype(dtype)
    S = np.diag(np.array(get_mrt_relaxation_diag(omega), dtype=dt))
    return (MRT_M_INV.astype(dt) @ (np.eye(19, dtype=dt) - 0.5 * S)) @ MRT_M.astype(dt)


def _matvec(op, v):
    op = op.astype(v.dtype)
    return np.stack([_seq([op[i, j] * v[j] for j in range(19)]) for i in range(19)])


def collision_mrt(f, feq, mrt_collision_matrix):
    """f + op (feq - f) (lbm3d/collision/mrt.py:88-98)."""
    return f + _matvec(mrt_collision_matrix, feq - f)


# -------------------------------------------------------------------- forcing

def get_guo_forcing_term(g, u):
    """Guo lattice force, D3Q19 closed form (lbm3d/forcing/guo.py:13-38)."""
    ux, uy, uz = u
    gx, gy, gz = g
    vp = np.stack([np.zeros_like(ux), ux, -ux, uy, -uy, uz, -uz,
                   ux + uy, -ux + uy, ux - uy, -ux - uy,
                   ux + uz, -ux + uz, ux - uz, -ux - uz,
                   uy + uz, -uy + uz, uy - uz, -uy - uz])
    fp = np.stack([np.zeros_like(gx), gx, -gx, gy, -gy, gz, -gz,
                   gx + gy, -gx + gy, gx - gy, -gx - gy,
                   gx + gz, -gx + gz, gx - gz, -gx - gz,
                   gy + gz, -gy + gz, gy - gz, -gy - gz])
    fv = (gx * ux + gy * uy) + gz * uz
    dt = np.result_type(g, u)
    return _w(dt, u.ndim - 1) * (3.0 * (fp - fv[None]) + (9.0 * fp) * vp)


def forcing_edm(f, g, u):
    """(lbm3d/forcing/edm.py:6-26)."""
    return f + get_guo_forcing_term(g, u)


def forcing_guo_bgk(f, g, u, omega):
    """(lbm3d/forcing/guo.py:41-55)."""
    return f + get_guo_forcing_term(g, u) * (1 - 0.5 * omega)


def forcing_guo_mrt(f, g, u, mrt_forcing_operator):
    """(lbm3d/forcing/guo.py:71-87)."""
    return f + _matvec(mrt_forcing_operator, get_guo_forcing_term(g, u))


# ----------------------------------------------------------------- boundaries

def _face_shape(f, loc):
    na = Q19_FACES[loc].normal_axis
    return tuple(f.shape[1 + ax] for ax in range(3) if ax != na)


def broadcast_wall_values(f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0):
    """(lbm3d/boundary/_helpers.py:19-34)."""
    shp = _face_shape(f, loc)
    dt = f.dtype

    def full(v):
        return np.full(shp, v, dtype=dt) if np.ndim(v) == 0 else np.asarray(v, dtype=dt)

    return full(rho_wall), np.stack([full(ux_wall), full(uy_wall), full(uz_wall)])


def _rho_wall_numerator(f, loc):
    """sum f_zero + 2 sum f_out at the wall (lbm3d/boundary/_helpers.py:37-44)."""
    s = Q19_FACES[loc]
    w = s.wall
    return _seq([f[(i,) + w] for i in s.zero_dirs]) + 2.0 * _seq([f[(i,) + w] for i in s.out_dirs])


def get_signed_wall_velocity(loc, ux_wall=0, uy_wall=0, uz_wall=0):
    """(lbm3d/boundary/_helpers.py:47-56)."""
    s = Q19_FACES[loc]
    vel = [ux_wall, uy_wall, uz_wall]
    return s.normal_sign * vel[s.normal_axis], [s.normal_sign * vel[a] for a in s.tangential_axes]


def get_rho_wall_from_velocity(f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
    """(lbm3d/boundary/_helpers.py:59-66)."""
    un, _ = get_signed_wall_velocity(loc, ux_wall, uy_wall, uz_wall)
    return _rho_wall_numerator(f, loc) / (1 - un)


def get_wall_velocity_from_pressure(f, loc, rho_wall=1):
    """(lbm3d/boundary/_helpers.py:69-81)."""
    s = Q19_FACES[loc]
    rw = np.full(_face_shape(f, loc), rho_wall, dtype=f.dtype)
    nvs = 1 - _rho_wall_numerator(f, loc) / rw
    _, u_nb = get_macroscopic(f[(slice(None),) + s.neighbor])
    vel = [u_nb[0], u_nb[1], u_nb[2]]
    vel[s.normal_axis] = s.normal_sign * nvs
    return tuple(vel)


def get_corrected_wall_velocity(ux_wall, uy_wall, uz_wall, rho_wall=1, gx_wall=0, gy_wall=0, gz_wall=0):
    """(lbm3d/boundary/_helpers.py:84-92)."""
    return (ux_wall - get_velocity_correction(gx_wall, rho_wall),
            uy_wall - get_velocity_correction(gy_wall, rho_wall),
            uz_wall - get_velocity_correction(gz_wall, rho_wall))


def _set_wall(f, loc, vals):
    out = f.copy()
    out[(slice(None),) + Q19_FACES[loc].wall] = vals
    return out


def boundary_nee(f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0):
    """(lbm3d/boundary/nee.py:13-32)."""
    s = Q19_FACES[loc]
    rw, uw = broadcast_wall_values(f, loc, rho_wall, ux_wall, uy_wall, uz_wall)
    feq_wall = get_equilibrium(rw, uw)
    f_nb = f[(slice(None),) + s.neighbor]
    rho_nb, u_nb = get_macroscopic(f_nb)
    return _set_wall(f, loc, feq_wall + (f_nb - get_equilibrium(rho_nb, u_nb)))


def boundary_nebb(f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0):
    """feq-difference NEBB (lbm3d/boundary/nebb.py:13-32)."""
    s = Q19_FACES[loc]
    rw, uw = broadcast_wall_values(f, loc, rho_wall, ux_wall, uy_wall, uz_wall)
    feq_wall = get_equilibrium(rw, uw)
    wall = f[(slice(None),) + s.wall]
    new = wall.copy()
    for i in s.in_dirs:
        o = Q19_OPP[i]
        new[i] = (wall[o] + feq_wall[i]) - feq_wall[o]
    return _set_wall(f, loc, new)


def boundary_equilibrium(f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0):
    """(lbm3d/boundary/eq.py:13-26)."""
    rw, uw = broadcast_wall_values(f, loc, rho_wall, ux_wall, uy_wall, uz_wall)
    return _set_wall(f, loc, get_equilibrium(rw, uw))


def _wrap_velocity(fn):
    def wrapped(f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
        rw = get_rho_wall_from_velocity(f, loc, ux_wall, uy_wall, uz_wall)
        return fn(f, loc, rho_wall=rw, ux_wall=ux_wall, uy_wall=uy_wall, uz_wall=uz_wall)
    return wrapped


def _wrap_pressure(fn):
    def wrapped(f, loc, rho_wall=1):
        ux, uy, uz = get_wall_velocity_from_pressure(f, loc, rho_wall)
        return fn(f, loc, rho_wall=rho_wall, ux_wall=ux, uy_wall=uy, uz_wall=uz)
    return wrapped


def _wrap_force_corrected(fn):
    def wrapped(f, loc, rho_wall=1, ux_wall=0, uy_wall=0, uz_wall=0, gx_wall=0, gy_wall=0, gz_wall=0):
        ux, uy, uz = get_corrected_wall_velocity(ux_wall, uy_wall, uz_wall, rho_wall, gx_wall, gy_wall, gz_wall)
        return fn(f, loc, rho_wall=rho_wall, ux_wall=ux, uy_wall=uy, uz_wall=uz)
    return wrapped


boundary_velocity_nee = _wrap_velocity(boundary_nee)
boundary_pressure_nee = _wrap_pressure(boundary_nee)
boundary_force_corrected_nee = _wrap_force_corrected(boundary_nee)
boundary_velocity_nebb = _wrap_velocity(boundary_nebb)
boundary_pressure_nebb = _wrap_pressure(boundary_nebb)
boundary_force_corrected_nebb = _wrap_force_corrected(boundary_nebb)
boundary_velocity_equilibrium = _wrap_velocity(boundary_equilibrium)
boundary_pressure_equilibrium = _wrap_pressure(boundary_equilibrium)
boundary_force_corrected_equilibrium = _wrap_force_corrected(boundary_equilibrium)


def boundary_bounce_back(f_before_stream, f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
    """Momentum-corrected bounce-back (lbm3d/boundary/bb.py:8-34)."""
    s = Q19_FACES[loc]
    dt = f.dtype
    pre = f_before_stream[(slice(None),) + s.wall]
    rho_w = _seq([pre[i] for i in range(19)]).astype(dt)
    _, uw = broadcast_wall_values(f, loc, 1, ux_wall, uy_wall, uz_wall)
    new = f[(slice(None),) + s.wall].copy()
    for i, o in zip(s.in_dirs, s.out_dirs):
        cu = None
        for d in range(3):
            cq = int(Q19_C[i, d])
            if cq == 0:
                continue
            t = uw[d] if cq > 0 else -uw[d]
            cu = t if cu is None else cu + t
        if cu is None:
            cu = np.zeros_like(rho_w)
        wi = Q19_W.astype(dt)[i]
        corr = (((2.0 * wi) * rho_w) * cu) / Q19_CS2
        new[i] = pre[o] + corr
    return _set_wall(f, loc, new)


def boundary_specular_reflection(f_before_stream, f, loc, ux_wall=0, uy_wall=0, uz_wall=0):
    """Identical to bounce-back in the reference's D3Q19 code (lbm3d/boundary/bb.py:37-53)."""
    return boundary_bounce_back(f_before_stream, f, loc, ux_wall, uy_wall, uz_wall)


def obstacle_bounce_back(f, mask):
    """(lbm3d/boundary/bb.py:56-59)."""
    out = f.copy()
    out[:, mask] = f[:, mask][list(Q19_OPP)]
    return out


def boundary_characteristic(rho, u, loc="right"):
    """(lbm3d/boundary/cbc.py:16-51)."""
    if loc not in Q19_FACES:
        raise ValueError("loc must be one of: 'left', 'right', 'bottom', 'top', 'back', 'front'")
    s = Q19_FACES[loc]
    na = s.normal_axis
    ta = s.tangential_axes
    sg = s.normal_sign
    cs = np.sqrt(np.asarray(Q19_CS2, dtype=rho.dtype))
    idx = [0, 1, 2] if sg > 0 else [-1, -2, -3]
    rb = [np.take(rho, i, axis=na) for i in idx]
    ub = [np.take(u[na], i, axis=na) for i in idx]
    ut0 = np.take(u[ta[0]], idx[0], axis=na)
    ut1 = np.take(u[ta[1]], idx[0], axis=na)
    dc = -0.5 * sg
    drho = dc * ((3 * rb[0] - 4 * rb[1]) + rb[2])
    dun = dc * ((3 * ub[0] - 4 * ub[1]) + ub[2])
    char_out = dun - ((sg * cs) / rb[0]) * drho
    l_out = (ub[0] - sg * cs) * char_out
    rho_next = rb[0] - ((0.5 * rb[0]) / cs) * l_out
    un_next = ub[0] - 0.5 * l_out
    vel = [None, None, None]
    vel[na] = un_next
    vel[ta[0]] = ut0
    vel[ta[1]] = ut1
    return rho_next, np.stack(vel)
