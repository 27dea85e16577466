"""The oracle's time step spread over the host's cores, for the timed CPU baseline.

Test infrastructure only, like the rest of ``oracle/``: it times the CPU restatement; the
product never calls it.  The stages of recipes.ib_lbm_step_2d / lbm_step_2d /
lbm_step_3d that act node by node are run on x slabs in a thread pool:

* moments, equilibrium, collision;
* EDM forcing.

NumPy releases the interpreter lock inside its array loops.  Streaming runs one thread
per population.  The immersed boundary and the Newmark update run on one thread.  The
face boundaries also run on one thread, on the planes next to each face only.  Every
value comes from the same NumPy operation on the same operands as in the serial recipe,
so the state is bit-identical to it (tests/test_oracle_golden.py).
"""

import concurrent.futures as cf
import os

import numpy as np

from . import lbm2d as L2
from . import lbm3d as L3
from . import recipes
from .lattice import Q9_C, Q19_C


def _shift_into(out, src, shift):
    """out = np.roll(src, shift) along every axis, by slice copies (no temporary)."""
    def spans(n, s):
        s %= n
        return [(slice(s, n), slice(0, n - s)), (slice(0, s), slice(n - s, n))] if s else [(slice(0, n), slice(0, n))]
    dims = [spans(n, s) for n, s in zip(src.shape, shift)]
    idx = [()]
    for d in dims:
        idx = [i + (p,) for i in idx for p in d]
    for parts in idx:
        dst = tuple(p[0] for p in parts)
        srcs = tuple(p[1] for p in parts)
        out[dst] = src[srcs]


_FACE = {"left": (0, 0), "right": (0, -1), "bottom": (1, 0), "top": (1, -1), "back": (2, 0), "front": (2, -1)}


def _faces_in_place(L, table, f_post, f, bcs, moments):
    """recipes._apply_bcs on the three planes next to each face instead of the whole
    array.  A face boundary reads the wall and at most the next two planes (the
    characteristic condition's three) and writes only the wall, so the values are the
    serial recipe's.  The whole-array copies are avoided."""
    for name, loc, kw in bcs:
        ax, side = _FACE[loc]
        n = f.shape[1 + ax]
        w = min(3, n)
        idx = (slice(None),) * (1 + ax) + ((slice(0, w) if side == 0 else slice(n - w, n)),)
        mom = None
        if moments is not None:
            rho, u = moments
            mom = (rho[idx[1:]], u[(slice(None),) + idx[1:]])
        f[idx] = recipes._apply_bcs(L, table, f_post[idx], f[idx].copy(), [(name, loc, kw)], mom)
    return f


def host_threads():
    """Cores this process may run on (at most 16: the slab loops stop scaling there)."""
    try:
        n = len(os.sched_getaffinity(0))
    except AttributeError:
        n = os.cpu_count() or 1
    return max(1, min(16, n))


class ThreadedStep:
    """One time step of a benchmark case (the dict of vivsim_gb300.configs) per call.

    ``dtype`` (float32 by default, as the benchmark) sets the precision of the populations,
    the markers and the MRT operator; float64 gives the double-precision oracle of the
    same case from the same (float32) initial populations."""

    def __init__(self, case, threads=None, dtype=np.float32):
        self.q = case["q"]
        self.L = L2 if self.q == 9 else L3
        self.C = Q9_C if self.q == 9 else Q19_C
        self.table = recipes._BC2 if self.q == 9 else recipes._BC3
        names = {("nee", "given"): "nee", ("nebb", "given"): "nebb", ("equilibrium", "given"): "eq",
                 ("nee", "pressure"): "pnee", ("nee", "velocity"): "vnee", ("nebb", "force_corrected"): "fcnebb"}
        self.bcs = [(names[(k, m)], loc, kw) for (k, loc, m, kw) in case["boundaries"]]
        self.coll, self.om = case["collision"], case["omega"]
        dt = np.dtype(dtype)
        self.op = L2.get_mrt_collision_operator(self.om, dt) if (self.coll == "mrt" and self.q == 9) else None
        self.f = case["f0"].astype(dt)
        self.body = None
        self.body3 = None
        b = case["body"]
        if b is not None and self.q == 9:
            X = b["markers"].astype(dt)
            self.body = recipes.Body2D(X[:, 0], X[:, 1], b["ds"], b["mass"], b["stiffness"], b["damping"],
                                       b["added_mass_area"], free=b["free_dof"][:2], kernel=b["kernel"],
                                       n_iter=b["n_iter"])
        elif b is not None:  # a fixed 3-D body: static stencil (recipes.ib_lbm_step_3d)
            from . import ib as OIB
            X = b["markers"].astype(dt)
            W, I = OIB.get_ib_stencil_3d(X, case["shape"])
            self.body3 = (W, I, np.zeros((X.shape[0], 3), dt), b["ds"], b["n_iter"])
        self.threads = threads or host_threads()
        nx = self.f.shape[1]
        k = min(self.threads * 2, nx)
        cuts = [nx * i // k for i in range(k + 1)]
        self.slabs = [(cuts[i], cuts[i + 1]) for i in range(k) if cuts[i + 1] > cuts[i]]
        self.pool = cf.ThreadPoolExecutor(self.threads)

    def close(self):
        self.pool.shutdown()

    def _map(self, fn, items):
        for _ in self.pool.map(fn, items):
            pass

    def __call__(self):
        """Advance self.f (and the body) by one step; self.h is the step's body force."""
        L, f = self.L, self.f
        grid = f.shape[1:]
        rho = np.empty(grid, f.dtype)
        u = np.empty((len(grid),) + grid, f.dtype)
        fp = np.empty_like(f)

        def collide(sl):
            lo, hi = sl
            r, uu = L.get_macroscopic(f[:, lo:hi])
            rho[lo:hi] = r
            u[:, lo:hi] = uu
            fp[:, lo:hi] = recipes._collide(L, f[:, lo:hi], L.get_equilibrium(r, uu), self.coll, self.om, self.op)

        self._map(collide, self.slabs)
        g = None
        self.h = None
        if self.body is not None:
            g, self.h = recipes.body_forces_2d(u, self.body, grid[1])
        elif self.body3 is not None:
            from . import ib as OIB
            W, I, mu, ds, n_iter = self.body3
            g, mh = OIB.multi_direct_forcing(u, W, I, mu, ds, n_iter)
            h = mh[0].copy()  # total force, summed in marker order as recipes.ib_lbm_step_3d does
            for i in range(1, mh.shape[0]):
                h = h + mh[i]
            self.h = h
        if g is not None:
            def force(sl):
                lo, hi = sl
                fp[:, lo:hi] = L.forcing_edm(fp[:, lo:hi], g[:, lo:hi], u[:, lo:hi])

            self._map(force, self.slabs)
        out = np.empty_like(fp)
        self._map(lambda i: _shift_into(out[i], fp[i], tuple(int(c) for c in self.C[i][:len(grid)])), range(self.q))
        self.f = _faces_in_place(L, self.table, fp, out, self.bcs, (rho, u))
