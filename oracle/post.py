"""Flow diagnostics — NumPy restatement of vivsim/post.py (test infrastructure only).

np.gradient has jnp.gradient's definition (unit spacing, edge_order 1): central
differences inside, one-sided differences at both ends of each axis.
"""

import numpy as np


def velocity_magnitude(u):
    """post.py:6-14"""
    return np.linalg.norm(u, axis=0)


def velocity_gradient(u):
    """post.py:17-29: G[i, j] = d u_i / d x_j"""
    d = u.shape[0]
    grads = np.gradient(u, axis=tuple(range(1, d + 1)))
    return np.stack(grads, axis=1)


def vorticity(u):
    """post.py:32-54"""
    if u.shape[0] == 2:
        return np.gradient(u[1], axis=0) - np.gradient(u[0], axis=1)
    dudy, dudz = np.gradient(u[0], axis=1), np.gradient(u[0], axis=2)
    dvdx, dvdz = np.gradient(u[1], axis=0), np.gradient(u[1], axis=2)
    dwdx, dwdy = np.gradient(u[2], axis=0), np.gradient(u[2], axis=1)
    return np.stack([dwdy - dvdz, dudz - dwdx, dvdx - dudy])


def vorticity_magnitude(u):
    """post.py:57-68"""
    w = vorticity(u)
    return np.abs(w) if u.shape[0] == 2 else np.linalg.norm(w, axis=0)


def divergence(u):
    """post.py:72-83"""
    return sum(np.gradient(u[i], axis=i) for i in range(u.shape[0]))


def strain_rate(u):
    """post.py:86-95"""
    G = velocity_gradient(u)
    return 0.5 * (G + np.swapaxes(G, 0, 1))


def strain_rate_magnitude(u):
    """post.py:98-107"""
    S = strain_rate(u)
    return np.sqrt(np.einsum("ij...,ij...->...", S, S))


def kinetic_energy(u):
    """post.py:110-118"""
    return 0.5 * np.sum(u ** 2, axis=0)


def mean_kinetic_energy(u):
    """post.py:121-129"""
    return np.mean(kinetic_energy(u))


def pressure(rho, cs2=1.0 / 3.0):
    """post.py:132-141"""
    return rho * cs2


def enstrophy(u):
    """post.py:144-155"""
    w = vorticity(u)
    return 0.5 * w ** 2 if u.shape[0] == 2 else 0.5 * np.sum(w ** 2, axis=0)


def mean_enstrophy(u):
    """post.py:158-167"""
    return np.mean(enstrophy(u))


def q_criterion(u):
    """post.py:172-186: -0.5 trace(G G)"""
    G = velocity_gradient(u)
    return -0.5 * np.einsum("ij...,ji...->...", G, G)
