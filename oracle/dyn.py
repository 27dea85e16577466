"""Rigid-body dynamics — NumPy restatement of vivsim/dyn.py (test infrastructure only)."""

import numpy as np


def newmark(a, v, d, h, m, k, c, dt=1, gamma=0.5, beta=0.25):
    """Newmark-beta predictor/corrector, scalar or matrix mass (vivsim/dyn.py:5-51)."""
    c1, c2 = gamma * dt, beta * dt ** 2
    v1 = v + dt * (1 - gamma) * a
    v2 = d + dt * v + dt ** 2 * (0.5 - beta) * a
    if np.ndim(m) > 0:
        a_next = np.linalg.solve(m + c1 * c + c2 * k, h - np.dot(c, v1) - np.dot(k, v2))
    else:
        a_next = (h - c * v1 - k * v2) / (m + c1 * c + c2 * k)
    return a_next, c1 * a_next + v1, c2 * a_next + v2


def get_markers_coords_2dof(x_markers_init, y_markers_init, d):
    """(vivsim/dyn.py:68-81)."""
    return x_markers_init + d[0], y_markers_init + d[1]


def get_markers_coords_3dof(x_markers_init, y_markers_init, x_center_init, y_center_init, d):
    """(vivsim/dyn.py:84-99)."""
    xr = x_markers_init - x_center_init
    yr = y_markers_init - y_center_init
    cs, sn = np.cos(d[2]), np.sin(d[2])
    return (((x_center_init + d[0]) + xr * cs) - yr * sn,
            ((y_center_init + d[1]) + xr * sn) + yr * cs)


def get_markers_velocity_3dof(x_markers, y_markers, x_center_init, y_center_init, d, v):
    """(vivsim/dyn.py:102-120)."""
    xr = (x_markers - x_center_init) - d[0]
    yr = (y_markers - y_center_init) - d[1]
    return np.stack([v[0] - v[2] * yr, v[1] + v[2] * xr], axis=-1)


def get_force_to_obj(h_markers):
    """(vivsim/dyn.py:126-136)."""
    out = h_markers[0].copy()
    for i in range(1, h_markers.shape[0]):
        out = out + h_markers[i]
    return out


def get_torque_to_obj(x_markers, y_markers, x_center_init, y_center_init, d, h_markers):
    """(vivsim/dyn.py:139-154)."""
    xr = x_markers - (x_center_init + d[0])
    yr = y_markers - (y_center_init + d[1])
    t = xr * h_markers[:, 1] - yr * h_markers[:, 0]
    out = t[0]
    for i in range(1, t.shape[0]):
        out = out + t[i]
    return out
