"""Concrete, seeded inputs of the benchmark cases (all synthetic; numpy default_rng draws).

Each builder returns a dict with the lattice-step arguments, the initial populations
(numpy, float32) and, where the case has one, the immersed body, so that the fused
kernels, the benchmark and the tests set a case up identically.

Cases:
  cavity        lid-driven cavity 256 x 256, D2Q9 BGK, NEE walls, lid ux = 0.1 (Re 1000)
                (examples/2d/lid_driven_cavity.py:55-63; wall order top, left, right, bottom)
  viv2d         cylinder VIV 1024 x 512, D2Q9 KBC (or MRT), D = 40 at (256, 256), 126 markers,
                Peskin 4-point, MDF 3, Re 100, transverse spring (mass ratio 10, U_r 5, no
                damping), equilibrium inflow ux = 0.05, pressure-NEE outflow rho = 1, periodic
                y; u_y perturbation N(0, 1e-4) from seed 0
                (examples/2d/vortex_induced_vibration.py:96-148)
  sphere3d      fixed sphere 256 x 128 x 128, D3Q19 regularised (or BGK), D = 24 at
                (64, 64, 64), 1810 Fibonacci markers, Peskin 4-point, MDF 3, Re 300,
                equilibrium inflow, pressure-NEE outflow, periodic y/z; u perturbation
                N(0, 1e-4) from seed 1 (examples/3d/flow_past_sphere.py:139-180)
  periodic2d    D2Q9 KBC on a periodic 8192 x 8192 grid (an HBM-bound size), no body
"""

import math

import numpy as np


def omega_of(nu):
    return 1 / (3 * nu + 0.5)


def equilibrium_d2q9(rho, u):
    """Host equilibrium for initial conditions (vivsim/lbm/basic.py:114-135), float32."""
    w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4, dtype=np.float32)
    c = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]], np.float32)
    uc = u[None, 0] * c[:, 0, None, None] + u[None, 1] * c[:, 1, None, None]
    usq = u[0] * u[0] + u[1] * u[1]
    return ((rho * w[:, None, None]) * (((1 + 3 * uc) + 4.5 * (uc * uc)) - 1.5 * usq)).astype(np.float32)


def equilibrium_d3q19(rho, u):
    """Host equilibrium for initial conditions (vivsim/lbm3d/basic.py:109-130), float32."""
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, dtype=np.float32)
    c = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                  [1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1],
                  [-1, 0, -1], [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1]], np.float32)
    out = np.empty((19,) + rho.shape, np.float32)
    usq = (u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]
    cs2 = np.float32(1 / 3)
    for q in range(19):
        uc = c[q, 0] * u[0] + c[q, 1] * u[1] + c[q, 2] * u[2]
        out[q] = (rho * w[q]) * (((1 + uc / cs2) + (0.5 * (uc * uc)) / np.float32(1 / 9)) - (0.5 * usq) / cs2)
    return out


def fibonacci_sphere(n, radius, center):
    """Markers on a sphere, equal area each: golden-angle spiral."""
    k = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * k / n)
    theta = math.pi * (1 + 5 ** 0.5) * k
    return np.stack([center[0] + radius * np.cos(theta) * np.sin(phi),
                     center[1] + radius * np.sin(theta) * np.sin(phi),
                     center[2] + radius * np.cos(phi)], axis=1)


def cavity(n=256, u_lid=0.1, nu=0.0256):
    rho = np.ones((n, n), np.float32)
    u = np.zeros((2, n, n), np.float32)
    return dict(
        name=f"lid_driven_cavity_d2q9_bgk_{n}x{n}", q=9, shape=(n, n), collision="bgk", omega=omega_of(nu),
        forcing="none",
        boundaries=[("nee", "top", "given", dict(ux_wall=u_lid)), ("nee", "left", "given", {}),
                    ("nee", "right", "given", {}), ("nee", "bottom", "given", {})],
        f0=equilibrium_d2q9(rho, u), body=None)


def viv2d(nx=1024, ny=512, collision="kbc", D=40.0, center=(256.0, 256.0), n_markers=126, U0=0.05, Re=100.0,
          mass_ratio=10.0, U_r=5.0, seed=0, n_iter=3):
    nu = U0 * D / Re
    rng = np.random.default_rng(seed)
    rho = np.ones((nx, ny), np.float32)
    u = np.zeros((2, nx, ny), np.float32)
    u[0] = U0
    u[1] = rng.normal(0.0, 1e-4, (nx, ny)).astype(np.float32)
    th = 2 * np.pi * np.arange(n_markers) / n_markers
    X = np.stack([center[0] + 0.5 * D * np.cos(th), center[1] + 0.5 * D * np.sin(th)], axis=1)
    area = math.pi * (D / 2) ** 2
    mass = area * mass_ratio
    fn = U0 / (U_r * D)
    K = (2 * math.pi * fn) ** 2 * mass * (1 + 1 / mass_ratio)
    body = dict(markers=X.astype(np.float32).astype(np.float64), ds=math.pi * D / n_markers, kernel="peskin4",
                radius=2, n_iter=n_iter, moving=True, free_dof=(False, True, False), mass=mass, stiffness=K,
                damping=0.0, added_mass_area=area)
    return dict(
        name=f"viv_cylinder_d2q9_{collision}_{nx}x{ny}_m{n_markers}_mdf{n_iter}", q=9, shape=(nx, ny),
        collision=collision, omega=omega_of(nu), forcing="edm",
        boundaries=[("equilibrium", "left", "given", dict(ux_wall=U0)),
                    ("nee", "right", "pressure", dict(rho_wall=1.0))],
        f0=equilibrium_d2q9(rho, u), body=body)


def sphere3d(nx=256, ny=128, nz=128, collision="reg", D=24.0, center=(64.0, 64.0, 64.0), n_markers=1810, U0=0.05,
             Re=300.0, seed=1, n_iter=3):
    nu = U0 * D / Re
    rng = np.random.default_rng(seed)
    rho = np.ones((nx, ny, nz), np.float32)
    u = rng.normal(0.0, 1e-4, (3, nx, ny, nz)).astype(np.float32)
    u[0] += np.float32(U0)
    X = fibonacci_sphere(n_markers, D / 2, center)
    body = dict(markers=X.astype(np.float32).astype(np.float64), ds=4 * math.pi * (D / 2) ** 2 / n_markers,
                kernel="peskin4", radius=2, n_iter=n_iter, moving=False)
    return dict(
        name=f"sphere_d3q19_{collision}_{nx}x{ny}x{nz}_m{n_markers}_mdf{n_iter}", q=19, shape=(nx, ny, nz),
        collision=collision, omega=omega_of(nu), forcing="edm",
        boundaries=[("equilibrium", "left", "given", dict(ux_wall=U0)),
                    ("nee", "right", "pressure", dict(rho_wall=1.0))],
        f0=equilibrium_d3q19(rho, u), body=body)


def periodic2d(n=8192, collision="kbc", U0=0.05, nu=0.01, seed=4):
    rng = np.random.default_rng(seed)
    rho = np.ones((n, n), np.float32)
    u = np.zeros((2, n, n), np.float32)
    u[0] = U0
    u[1] = rng.normal(0.0, 1e-3, (n, n)).astype(np.float32)
    return dict(name=f"periodic_d2q9_{collision}_{n}x{n}", q=9, shape=(n, n), collision=collision,
                omega=omega_of(nu), forcing="none", boundaries=[], f0=equilibrium_d2q9(rho, u), body=None)


def viv_sweep(n_cases=64, seed=3, heights=(64, 128, 256, 512), collision="kbc"):
    """Independent cylinder VIV cases of uneven size: H uniform in `heights`, grid 2H x H,
    D = H/12 at (H/2, H/2) (W/4, H/2 with W = 2H), round(pi D) markers, U_r ~ U[3, 8],
    Re ~ U[50, 200], U0 = 0.05, mass ratio 10, KBC; boundaries as viv2d.  Draw order per
    case from default_rng(seed): H, U_r, Re, then the case's perturbation seed."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_cases):
        H = int(heights[int(rng.integers(len(heights)))])
        U_r = float(rng.uniform(3.0, 8.0))
        Re = float(rng.uniform(50.0, 200.0))
        s = int(rng.integers(1 << 31))
        D = H / 12.0
        out.append(viv2d(nx=2 * H, ny=H, collision=collision, D=D, center=(H / 2.0, H / 2.0),
                         n_markers=int(round(math.pi * D)), Re=Re, U_r=U_r, seed=s))
    return out


CASES = {"cavity": cavity, "viv2d": viv2d, "sphere3d": sphere3d, "periodic2d": periodic2d}


def build_solver(case, device="cuda", variant="auto", dtype=None):
    """LatticeStep, RigidBody (or None) and Simulation for a case dict (float32 unless
    dtype says otherwise)."""
    import torch

    from . import solver as S
    bcs = [S.boundary(k, loc, mode=m, **kw) for (k, loc, m, kw) in case["boundaries"]]
    step = S.LatticeStep(case["q"], case["shape"], case["collision"], case["omega"], forcing=case["forcing"],
                         boundaries=bcs, variant=variant, dtype=dtype or torch.float32)
    body = None
    if case["body"] is not None:
        b = case["body"]
        body = S.RigidBody(step, b["markers"], b["ds"], kernel=b["kernel"], radius=b["radius"], n_iter=b["n_iter"],
                           moving=b["moving"], free_dof=b.get("free_dof", (False, False, False)),
                           mass=b.get("mass", 1.0), stiffness=b.get("stiffness", 0.0),
                           damping=b.get("damping", 0.0), added_mass_area=b.get("added_mass_area", 0.0))
    sim = S.Simulation(step, torch.from_numpy(case["f0"]).to(device), body)
    return step, body, sim
