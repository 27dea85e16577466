"""D2Q9 operators — NumPy restatement of vivsim/lbm (test infrastructure only).

Arrays are SoA, C-order ``(9, NX, NY)``.  Reductions over populations are written as
explicit left-to-right sums so their rounding order is fixed.
"""

import numpy as np

from .lattice import Q9_C, Q9_DOWN, Q9_FACES, Q9_LEFT, Q9_OPP, Q9_RIGHT, Q9_UP, Q9_W


def _seq(terms):
    out = terms[0]
    for t in terms[1:]:
        out = out + t
    return out


def _w(dt, ndim):
    return Q9_W.astype(dt).reshape((9,) + (1,) * ndim)


# ------------------------------------------------------------------ basic ops

def streaming(f):
    """Periodic D2Q9 shift by c_i (vivsim/lbm/basic.py:60-85)."""
    out = np.empty_like(f)
    for i in range(9):
        out[i] = np.roll(f[i], shift=(int(Q9_C[i, 0]), int(Q9_C[i, 1])), axis=(0, 1))
    return out


def get_macroscopic(f):
    """rho = sum f; u = (sum right - sum left, sum up - sum down) / rho (lbm/basic.py:88-111)."""
    rho = _seq([f[i] for i in range(9)])
    u = np.zeros((2,) + rho.shape, dtype=f.dtype)
    u[0] = (_seq([f[i] for i in Q9_RIGHT]) - _seq([f[i] for i in Q9_LEFT])) / rho
    u[1] = (_seq([f[i] for i in Q9_UP]) - _seq([f[i] for i in Q9_DOWN])) / rho
    return rho, u


def get_equilibrium(rho, u):
    """feq_i = rho w_i (1 + 3 cu + 4.5 cu^2 - 1.5 u^2) (lbm/basic.py:114-135)."""
    dt = np.result_type(rho, u)
    ndim = np.ndim(rho)
    c = Q9_C.astype(dt).reshape((9, 2) + (1,) * ndim)
    uc = u[None, 0] * c[:, 0] + u[None, 1] * c[:, 1]
    usq = u[0] * u[0] + u[1] * u[1]
    return (rho * _w(dt, ndim)) * (((1 + 3 * uc) + 4.5 * (uc * uc)) - 1.5 * usq)


def collision_bgk(f, feq, omega):
    """(1 - omega) f + omega feq (lbm/basic.py:138-156)."""
    return (1 - omega) * f + omega * feq


def get_omega(nu):
    """omega = 1 / (3 nu + 0.5) (lbm/basic.py:159-172)."""
    return 1 / (3 * nu + 0.5)


def get_velocity_correction(g, rho=1):
    """g * 0.5 / rho (lbm/basic.py:175-194)."""
    return g * 0.5 / rho


# ----------------------------------------------------------------- collisions

def collision_kbc(f, feq, omega):
    """Entropic KBC step (lbm/collision/kbc.py:10-60)."""
    fneq = f - feq
    nsd = ((fneq[1] - fneq[2]) + fneq[3]) - fneq[4]
    ssd = ((fneq[5] - fneq[6]) + fneq[7]) - fneq[8]
    shear = np.zeros_like(fneq)
    for k, i in enumerate(range(1, 5)):
        shear[i] = ((1, -1, 1, -1)[k] * nsd) / 4.0
    for k, i in enumerate(range(5, 9)):
        shear[i] = ((1, -1, 1, -1)[k] * ssd) / 4.0
    high = fneq - shear
    den = feq + 1e-20
    inner_sh = _seq([(high[i] * shear[i]) / den[i] for i in range(9)])
    inner_hh = _seq([(high[i] * high[i]) / den[i] for i in range(9)])
    half_gamma = 1.0 / omega - ((1.0 - 1.0 / omega) * inner_sh) / (inner_hh + 1e-20)
    return f - omega * (shear + half_gamma[None] * high)


# MRT basis, lbm/collision/mrt.py:9-23 (Gram-Schmidt D2Q9 moments)
MRT_M = np.array([
    [1, 1, 1, 1, 1, 1, 1, 1, 1],
    [-4, -1, -1, -1, -1, 2, 2, 2, 2],
    [4, -2, -2, -2, -2, 1, 1, 1, 1],
    [0, 1, 0, -1, 0, 1, -1, -1, 1],
    [0, -2, 0, 2, 0, 1, -1, -1, 1],
    [0, 0, 1, 0, -1, 1, 1, -1, -1],
    [0, 0, -2, 0, 2, 1, 1, -1, -1],
    [0, 1, -1, 1, -1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 1, -1, 1, -1],
])
MRT_M_INV = np.linalg.inv(MRT_M)


def get_mrt_relaxation_diag(omega):
    """Diagonal of S (lbm/collision/mrt.py:29-44)."""
    return [0, 1.4, 1.4, 0, 1.2, 0, 1.2, omega, omega]


def get_mrt_collision_operator(omega, dtype=np.float32):
    """M^-1 S M evaluated in ``dtype`` like JAX (lbm/collision/mrt.py:47-63)."""
    dt = np.dtype(dtype)
    S = np.diag(np.array(get_mrt_relaxation_diag(omega), dtype=dt))
    return (MRT_M_INV.astype(dt) @ S) @ MRT_M.astype(dt)


def get_mrt_forcing_operator(omega, dtype=np.float32):
    """M^-1 (I - S/2) M (lbm/forcing/guo.py:62-80)."""
    dt = np.dtype(dtype)
    S = np.diag(np.array(get_mrt_relaxation_diag(omega), dtype=dt))
    return (MRT_M_INV.astype(dt) @ (np.eye(9, dtype=dt) - 0.5 * S)) @ MRT_M.astype(dt)


def _matvec(op, v):
    op = op.astype(v.dtype)
    return np.stack([_seq([op[i, j] * v[j] for j in range(op.shape[1])]) for i in range(op.shape[0])])


def collision_mrt(f, feq, mrt_collision_matrix):
    """f + (M^-1 S M)(feq - f) (lbm/collision/mrt.py:66-88)."""
    return f + _matvec(mrt_collision_matrix, feq - f)


def collision_reg(f, feq, omega):
    """Regularised BGK via closed-form second-order moments (lbm/collision/reg.py:4-49)."""
    fneq = f - feq
    diag_sum = ((fneq[5] + fneq[6]) + fneq[7]) + fneq[8]
    pi_xx = (fneq[1] + fneq[3]) + diag_sum
    pi_yy = (fneq[2] + fneq[4]) + diag_sum
    pi_xy = ((fneq[5] - fneq[6]) + fneq[7]) - fneq[8]
    trace = (pi_xx + pi_yy) / 12.0
    axis_x = (2.0 * pi_xx - pi_yy) / 6.0
    axis_y = (2.0 * pi_yy - pi_xx) / 6.0
    diag_pos = trace + pi_xy / 4.0
    diag_neg = trace - pi_xy / 4.0
    reg = np.stack([-8.0 * trace, axis_x, axis_y, axis_x, axis_y,
                    diag_pos, diag_neg, diag_pos, diag_neg])
    return feq + (1 - omega) * reg


# -------------------------------------------------------------------- forcing

def get_guo_forcing_term(g, u):
    """Guo lattice force (lbm/forcing/guo.py:6-35)."""
    dt = np.result_type(g, u)
    ndim = u.ndim - 1
    c = Q9_C.astype(dt).reshape((9, 2) + (1,) * ndim)
    cx, cy = c[:, 0], c[:, 1]
    uc = u[None, 0] * cx + u[None, 1] * cy
    return _w(dt, ndim) * (
        g[None, 0] * (3 * (cx - u[None, 0]) + 9 * (uc * cx))
        + g[None, 1] * (3 * (cy - u[None, 1]) + 9 * (uc * cy)))


def forcing_edm(f, g, u):
    """f + Guo term (lbm/forcing/edm.py:4-31)."""
    return f + get_guo_forcing_term(g, u)


def forcing_guo_bgk(f, g, u, omega):
    """f + (1 - omega/2) Guo term (lbm/forcing/guo.py:38-59)."""
    return f + get_guo_forcing_term(g, u) * (1 - 0.5 * omega)


def forcing_guo_mrt(f, g, u, mrt_forcing_operator):
    """f + M^-1 (I - S/2) M Guo term (lbm/forcing/guo.py:83-107)."""
    return f + _matvec(mrt_forcing_operator, get_guo_forcing_term(g, u))


# ----------------------------------------------------------------- boundaries

def _face_len(f, loc):
    return f.shape[2] if Q9_FACES[loc].normal_axis == 0 else f.shape[1]


def broadcast_wall_values(f, loc, rho_wall=1, ux_wall=0, uy_wall=0):
    """Scalar wall data -> (N,) arrays (lbm/boundary/_helpers.py:50-76)."""
    n = _face_len(f, loc)
    dt = f.dtype

    def full(v):
        return np.full(n, v, dtype=dt) if np.isscalar(v) or np.ndim(v) == 0 else np.asarray(v, dtype=dt)

    return full(rho_wall), np.stack([full(ux_wall), full(uy_wall)])


def get_signed_wall_velocity(loc, ux_wall=0, uy_wall=0):
    """(lbm/boundary/_helpers.py:138-144)."""
    s = Q9_FACES[loc]
    normal = ux_wall if s.normal_axis == 0 else uy_wall
    tangential = uy_wall if s.normal_axis == 0 else ux_wall
    return s.normal_sign * normal, s.normal_sign * tangential


def _rho_wall_numerator(f, loc):
    """f0 + f_t0 + f_t1 + 2 (f_o0 + f_o1 + f_o2) at the wall (_helpers.py:124-135)."""
    s = Q9_FACES[loc]
    w = s.wall
    t0, t1 = s.tan_dirs
    o0, o1, o2 = s.out_dirs
    return ((f[(0,) + w] + f[(t0,) + w]) + f[(t1,) + w]) + 2 * ((f[(o0,) + w] + f[(o1,) + w]) + f[(o2,) + w])


def get_rho_wall_from_velocity(f, loc, ux_wall=0, uy_wall=0):
    """(_helpers.py:79-95)."""
    un, _ = get_signed_wall_velocity(loc, ux_wall, uy_wall)
    return _rho_wall_numerator(f, loc) / (1 - un)


def get_wall_velocity_from_pressure(f, loc, rho_wall=1):
    """Normal velocity from rho_wall, tangential copied from the neighbour (_helpers.py:98-121)."""
    s = Q9_FACES[loc]
    nb = s.neighbor
    ps0, ps1, ps2 = s.pos_side_dirs
    ns0, ns1, ns2 = s.neg_side_dirs
    rho_nb = _seq([f[(i,) + nb] for i in range(9)])
    nvs = 1 - _rho_wall_numerator(f, loc) / rho_wall
    normal = s.normal_sign * nvs
    tang = (((((f[(ps0,) + nb] - f[(ns0,) + nb]) + f[(ps1,) + nb]) - f[(ns1,) + nb])
             + f[(ps2,) + nb]) - f[(ns2,) + nb]) / rho_nb
    vel = [None, None]
    vel[s.normal_axis] = normal
    vel[1 - s.normal_axis] = tang
    return tuple(vel)


def get_corrected_wall_velocity(ux_wall, uy_wall, rho_wall=1, gx_wall=0, gy_wall=0):
    """Half-force wall velocity shift (_helpers.py:147-172)."""
    return (ux_wall - get_velocity_correction(gx_wall, rho_wall),
            uy_wall - get_velocity_correction(gy_wall, rho_wall))


def _set_wall(f, loc, vals):
    out = f.copy()
    out[(slice(None),) + Q9_FACES[loc].wall] = vals
    return out


def boundary_nee(f, loc, rho_wall=1, ux_wall=0, uy_wall=0):
    """Non-equilibrium extrapolation (lbm/boundary/nee.py:19-60)."""
    s = Q9_FACES[loc]
    rw, uw = broadcast_wall_values(f, loc, rho_wall, ux_wall, uy_wall)
    feq_wall = get_equilibrium(rw, uw)
    f_nb = f[(slice(None),) + s.neighbor]
    rho_nb, u_nb = get_macroscopic(f_nb)
    fneq_nb = f_nb - get_equilibrium(rho_nb, u_nb)
    return _set_wall(f, loc, feq_wall + fneq_nb)


def boundary_nebb(f, loc, rho_wall=1, ux_wall=0, uy_wall=0):
    """Zou/He non-equilibrium bounce-back (lbm/boundary/nebb.py:20-58)."""
    s = Q9_FACES[loc]
    un, ut = get_signed_wall_velocity(loc, ux_wall, uy_wall)
    wall = f[(slice(None),) + s.wall]
    shear = 0.5 * (wall[s.tan_dirs[0]] - wall[s.tan_dirs[1]]) * s.normal_sign
    normal_term = 1 / 6 * un * rho_wall
    tang_term = 0.5 * ut * rho_wall
    new = wall.copy()
    new[s.in_dirs[0]] = wall[s.out_dirs[0]] + 2 / 3 * un * rho_wall
    new[s.in_dirs[1]] = ((wall[s.out_dirs[1]] - shear) + normal_term) + tang_term
    new[s.in_dirs[2]] = ((wall[s.out_dirs[2]] + shear) + normal_term) - tang_term
    return _set_wall(f, loc, new)


def boundary_equilibrium(f, loc, rho_wall=1, ux_wall=0, uy_wall=0):
    """Wall set to feq(rho_wall, u_wall) (lbm/boundary/eq.py:25-56)."""
    rw, uw = broadcast_wall_values(f, loc, rho_wall, ux_wall, uy_wall)
    return _set_wall(f, loc, get_equilibrium(rw, uw))


def _wrap_velocity(fn):
    def wrapped(f, loc, ux_wall=0, uy_wall=0):
        rw = get_rho_wall_from_velocity(f, loc, ux_wall, uy_wall)
        return fn(f, loc, rho_wall=rw, ux_wall=ux_wall, uy_wall=uy_wall)
    return wrapped


def _wrap_pressure(fn):
    def wrapped(f, loc, rho_wall=1):
        ux, uy = get_wall_velocity_from_pressure(f, loc, rho_wall)
        return fn(f, loc, rho_wall=rho_wall, ux_wall=ux, uy_wall=uy)
    return wrapped


def _wrap_force_corrected(fn):
    def wrapped(f, loc, rho_wall=1, ux_wall=0, uy_wall=0, gx_wall=0, gy_wall=0):
        ux, uy = get_corrected_wall_velocity(ux_wall, uy_wall, rho_wall, gx_wall, gy_wall)
        return fn(f, loc, rho_wall=rho_wall, ux_wall=ux, uy_wall=uy)
    return wrapped


# lbm/boundary/{nee.py:63-65, nebb.py:60-62, eq.py:59-61}
boundary_velocity_nee = _wrap_velocity(boundary_nee)
boundary_pressure_nee = _wrap_pressure(boundary_nee)
boundary_force_corrected_nee = _wrap_force_corrected(boundary_nee)
boundary_velocity_nebb = _wrap_velocity(boundary_nebb)
boundary_pressure_nebb = _wrap_pressure(boundary_nebb)
boundary_force_corrected_nebb = _wrap_force_corrected(boundary_nebb)
boundary_velocity_equilibrium = _wrap_velocity(boundary_equilibrium)
boundary_pressure_equilibrium = _wrap_pressure(boundary_equilibrium)
boundary_force_corrected_equilibrium = _wrap_force_corrected(boundary_equilibrium)


def _bb_common(f_before_stream, f, loc, ux_wall, uy_wall, scatter):
    s = Q9_FACES[loc]
    un, ut = get_signed_wall_velocity(loc, ux_wall, uy_wall)
    pre = f_before_stream[(slice(None),) + s.wall]
    vals = [pre[s.out_dirs[0]] + 2 / 3 * un,
            pre[s.out_dirs[1]] + 1 / 6 * (un + ut),
            pre[s.out_dirs[2]] + 1 / 6 * (un - ut)]
    new = f[(slice(None),) + s.wall].copy()
    for d, v in zip(scatter, vals):
        new[d] = v
    return _set_wall(f, loc, new)


def boundary_bounce_back(f_before_stream, f, loc, ux_wall=0, uy_wall=0):
    """Half-way bounce-back with moving-wall term (lbm/boundary/bb.py:15-53)."""
    s = Q9_FACES[loc]
    return _bb_common(f_before_stream, f, loc, ux_wall, uy_wall, s.in_dirs)


def boundary_specular_reflection(f_before_stream, f, loc, ux_wall=0, uy_wall=0):
    """Mirror reflection: diagonal in_dirs swapped (lbm/boundary/bb.py:56-95)."""
    s = Q9_FACES[loc]
    return _bb_common(f_before_stream, f, loc, ux_wall, uy_wall,
                      (s.in_dirs[0], s.in_dirs[2], s.in_dirs[1]))


def obstacle_bounce_back(f, mask):
    """Masked nodes take their opposite populations (lbm/boundary/bb.py:98-110)."""
    out = f.copy()
    sel = f[:, mask]
    out[:, mask] = sel[list(Q9_OPP)]
    return out


def boundary_characteristic(rho, u, loc="right"):
    """Non-reflective characteristic update of (rho, u) on a face (lbm/boundary/cbc.py:14-53)."""
    if loc not in Q9_FACES:
        raise ValueError("loc must be one of: 'left', 'right', 'top', 'bottom'")
    s = Q9_FACES[loc]
    na = s.normal_axis
    ta = 1 - na
    sg = s.normal_sign
    cs = (1 / np.sqrt(np.asarray(3, dtype=rho.dtype))).astype(rho.dtype)
    idx = [0, 1, 2] if sg > 0 else [-1, -2, -3]
    rb = [np.take(rho, i, axis=na) for i in idx]
    ub = [np.take(u[na], i, axis=na) for i in idx]
    ut = np.take(u[ta], 0 if sg > 0 else -1, axis=na)
    dc = -0.5 * sg
    drho = dc * ((3 * rb[0] - 4 * rb[1]) + rb[2])
    dun = dc * ((3 * ub[0] - 4 * ub[1]) + ub[2])
    char_out = dun - ((sg * cs) / rb[0]) * drho
    l_out = (ub[0] - sg * cs) * char_out
    rho_next = rb[0] - ((0.5 * rb[0]) / cs) * l_out
    un_next = ub[0] - 0.5 * l_out
    vel = [None, None]
    vel[na] = un_next
    vel[ta] = ut
    return rho_next, np.stack(vel)
