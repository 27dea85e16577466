"""Flow diagnostics with the reference's names (vivsim/post.py), computed on the GPU.

Each field function takes a velocity tensor u of shape (2, NX, NY) or (3, NX, NY, NZ)
(CUDA) and runs one kernel of the C ABI (vs_post).  ``*_from_populations`` variants take
the populations f instead and compute u on the fly.
"""

import torch

from . import _lib as V

VELOCITY_MAGNITUDE, VELOCITY_GRADIENT, VORTICITY, VORTICITY_MAGNITUDE, DIVERGENCE = 0, 1, 2, 3, 4
STRAIN_RATE, STRAIN_RATE_MAGNITUDE, KINETIC_ENERGY, ENSTROPHY, Q_CRITERION = 5, 6, 7, 8, 9
MEAN_KINETIC_ENERGY, MEAN_ENSTROPHY = 10, 11


def _field(what, u=None, f=None):
    src = u if u is not None else f
    V.require_cuda(src)
    src = V.cont(src)
    if u is not None:
        d = int(src.shape[0])
        if d not in (2, 3) or src.dim() != d + 1:
            raise ValueError("u must have shape (2, NX, NY) or (3, NX, NY, NZ)")
        q = 9 if d == 2 else 19
    else:
        q = int(src.shape[0])
        if q not in (9, 19) or src.dim() != (3 if q == 9 else 4):
            raise ValueError("f must have shape (9, NX, NY) or (19, NX, NY, NZ)")
        d = 2 if q == 9 else 3
    dims = [int(x) for x in src.shape[1:]] + [1]
    nx, ny, nz = dims[0], dims[1], dims[2]
    code = V.dtype_code(src)
    up, fp = (V.ptr(src), None) if u is not None else (None, V.ptr(src))
    if what in (MEAN_KINETIC_ENERGY, MEAN_ENSTROPHY):
        acc = torch.zeros(1, dtype=torch.float64, device=src.device)
        V.call("vs_post", q, code, what, up, fp, nx, ny, nz, None, V.ptr(acc), V.stream())
        return (acc[0] / float(nx * ny * nz)).to(src.dtype)
    nc = V.lib().vs_post_components(q, what)
    shape = tuple(src.shape[1:])
    if what in (VELOCITY_GRADIENT, STRAIN_RATE):
        oshape = (d, d) + shape
    elif what == VORTICITY and d == 3:
        oshape = (3,) + shape
    else:
        oshape = shape
    out = torch.empty((nc,) + shape if nc > 1 else shape, dtype=src.dtype, device=src.device)
    V.call("vs_post", q, code, what, up, fp, nx, ny, nz, V.ptr(out), None, V.stream())
    return out.reshape(oshape)


def velocity_magnitude(u):
    return _field(VELOCITY_MAGNITUDE, u)


def velocity_gradient(u):
    return _field(VELOCITY_GRADIENT, u)


def vorticity(u):
    return _field(VORTICITY, u)


def vorticity_magnitude(u):
    return _field(VORTICITY_MAGNITUDE, u)


def divergence(u):
    return _field(DIVERGENCE, u)


def strain_rate(u):
    return _field(STRAIN_RATE, u)


def strain_rate_magnitude(u):
    return _field(STRAIN_RATE_MAGNITUDE, u)


def kinetic_energy(u):
    return _field(KINETIC_ENERGY, u)


def mean_kinetic_energy(u):
    return _field(MEAN_KINETIC_ENERGY, u)


def enstrophy(u):
    return _field(ENSTROPHY, u)


def mean_enstrophy(u):
    return _field(MEAN_ENSTROPHY, u)


def q_criterion(u):
    return _field(Q_CRITERION, u)


def pressure(rho, cs2=1.0 / 3.0):
    V.require_cuda(rho)
    r = V.cont(rho)
    out = torch.empty_like(r)
    V.call("vs_post_pressure", V.dtype_code(r), V.ptr(r), int(r.numel()), float(cs2), V.ptr(out), V.stream())
    return out


def vorticity_from_populations(f):
    """vorticity(get_macroscopic(f)[1]) in one pass over the populations."""
    return _field(VORTICITY, f=f)


def q_criterion_from_populations(f):
    return _field(Q_CRITERION, f=f)


# deprecated aliases of the reference (post.py:194-212)
calculate_curl = vorticity
calculate_vorticity = vorticity
calculate_velocity_magnitude = velocity_magnitude


def calculate_vorticity_dimensionless(u, l, u0):
    return vorticity(u) * l / u0
