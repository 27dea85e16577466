"""Fused IB-LBM time stepping: one plan per lattice, one per immersed body.

The reference has no driver; its examples compose the per-operator functions into an
``update_step`` run under ``jax.jit`` + ``lax.scan`` (e.g.
examples/2d/vortex_induced_vibration.py:96-157).  ``Simulation`` is that loop, executed by
the fused kernels of ``vs_step``/``vs_run``/``vs_run_graph`` with the body state kept on
the device, so a multi-step run never synchronises with the host.
"""

import ctypes as C

import numpy as np
import torch

from . import _lib as V
from ._ops import mrt_collision_operator, mrt_forcing_operator

COLLISIONS = {"bgk": V.VS_COLLIDE_BGK, "kbc": V.VS_COLLIDE_KBC, "mrt": V.VS_COLLIDE_MRT, "reg": V.VS_COLLIDE_REG}
FORCINGS = {"none": V.VS_FORCE_NONE, "edm": V.VS_FORCE_EDM, "guo_bgk": V.VS_FORCE_GUO_BGK,
            "guo_mrt": V.VS_FORCE_GUO_MRT}
BC_KINDS = {"nee": V.VS_BC_NEE, "nebb": V.VS_BC_NEBB, "equilibrium": V.VS_BC_EQ, "eq": V.VS_BC_EQ,
            "bounce_back": V.VS_BC_BB, "specular_reflection": V.VS_BC_SPECULAR}
WALL_MODES = {"given": V.VS_WALL_GIVEN, "velocity": V.VS_WALL_VELOCITY, "pressure": V.VS_WALL_PRESSURE,
              "force_corrected": V.VS_WALL_FORCE_CORRECTED, "characteristic": V.VS_WALL_CHARACTERISTIC}
KERNELS = {"peskin3": V.VS_KERNEL_PESKIN3, "peskin4": V.VS_KERNEL_PESKIN4, "cosine4": V.VS_KERNEL_COSINE4}


def boundary(kind, loc, mode="given", rho_wall=1.0, ux_wall=0.0, uy_wall=0.0, uz_wall=0.0, gx_wall=0.0,
             gy_wall=0.0, gz_wall=0.0):
    """One face boundary of the step, e.g. ``boundary("nee", "right", mode="pressure")``.

    ``kind`` names the reference scheme (boundary_nee / _nebb / _equilibrium /
    _bounce_back / _specular_reflection) and ``mode`` its wrapper (velocity / pressure /
    force_corrected, lbm/boundary/_helpers.py:175-239).  ``mode="characteristic"`` takes
    the wall density and velocity of every face node from boundary_characteristic
    (lbm/boundary/cbc.py:14-53) of the step's input moments: a non-reflective outflow,
    imposed by the nee, nebb or equilibrium scheme.
    """
    return dict(kind=kind, loc=loc, mode=mode, rho=rho_wall, ux=ux_wall, uy=uy_wall, uz=uz_wall, gx=gx_wall,
                gy=gy_wall, gz=gz_wall)


def check_finite(f):
    """True when every value of the CUDA tensor f is finite (one scan kernel; synchronises)."""
    V.require_cuda(f)
    f = V.cont(f)
    status = torch.zeros(1, dtype=torch.int32, device=f.device)
    V.call("vs_check_finite", V.dtype_code(f), V.ptr(f), f.numel(), V.ptr(status), V.stream())
    return int(status.item()) == 0


def _tdtype(dtype):
    return torch.float64 if dtype in (torch.float64, "float64", np.float64) else torch.float32


class LatticeStep:
    """Plan of the fused collide-force-stream-boundary step on one grid."""

    def __init__(self, q, shape, collision="bgk", omega=1.0, dtype=torch.float32, mrt_op=None, forcing="none",
                 g=None, boundaries=(), variant="auto", obstacle_mask=None, watchdog_every=0):
        if q not in (9, 19):
            raise ValueError("q must be 9 (D2Q9) or 19 (D3Q19)")
        self.q = q
        self.dim = 2 if q == 9 else 3
        self.shape = tuple(int(s) for s in shape)
        if len(self.shape) != self.dim:
            raise ValueError(f"shape must have {self.dim} entries")
        self.dtype = _tdtype(dtype)
        if collision not in COLLISIONS:
            raise ValueError(f"collision must be one of {', '.join(repr(x) for x in COLLISIONS)}")
        if forcing not in FORCINGS:
            raise ValueError(f"forcing must be one of {', '.join(repr(x) for x in FORCINGS)}")
        self.collision = collision
        self.omega = float(omega)
        cfg = V.vs_lattice_cfg()
        cfg.q = q
        cfg.dtype = V.VS_F64 if self.dtype == torch.float64 else V.VS_F32
        cfg.nx, cfg.ny = self.shape[0], self.shape[1]
        cfg.nz = self.shape[2] if self.dim == 3 else 1
        cfg.collision = COLLISIONS[collision]
        cfg.omega = self.omega
        if collision == "mrt":
            op = mrt_collision_operator(q, omega, self.dtype) if mrt_op is None else mrt_op
            a = np.asarray(op.cpu().double() if isinstance(op, torch.Tensor) else op, dtype=np.float64).reshape(-1)
            for i, v in enumerate(a):
                cfg.mrt_op[i] = float(v)
        cfg.forcing = FORCINGS[forcing]
        if forcing == "guo_mrt":
            a = mrt_forcing_operator(q, omega, self.dtype).double().numpy().reshape(-1)
            for i, v in enumerate(a):
                cfg.mrt_fop[i] = float(v)
        if g is not None:
            for i, v in enumerate(g):
                cfg.g_uniform[i] = float(v)
        if len(boundaries) > V.VS_MAX_BC:
            raise ValueError(f"at most {V.VS_MAX_BC} boundaries")
        cfg.n_bc = len(boundaries)
        for k, b in enumerate(boundaries):
            s = cfg.bc[k]
            for key, table in (("kind", BC_KINDS), ("mode", WALL_MODES), ("loc", V.LOCS)):
                if b.get(key) not in table:
                    raise ValueError(f"boundary {k}: {key} must be one of {', '.join(repr(x) for x in table)}")
            s.kind = BC_KINDS[b["kind"]]
            s.mode = WALL_MODES[b["mode"]]
            s.loc = V.LOCS[b["loc"]]
            for name in ("rho", "ux", "uy", "uz", "gx", "gy", "gz"):
                setattr(s, name, float(b.get(name, 1.0 if name == "rho" else 0.0)))
        variants = {"auto": V.VS_GRID_AUTO, "plain": V.VS_GRID_PLAIN, "tma": V.VS_GRID_TMA}
        if variant not in variants:
            raise ValueError(f"variant must be one of {', '.join(repr(x) for x in variants)}")
        cfg.variant = variants[variant]
        self._mask = None
        if obstacle_mask is not None:  # obstacle_bounce_back after the face boundaries, every step
            m = obstacle_mask if isinstance(obstacle_mask, torch.Tensor) else torch.as_tensor(obstacle_mask)
            if tuple(m.shape) != self.shape:
                raise ValueError(f"obstacle_mask must have shape {self.shape}")
            V.require_cuda(m)
            self._mask = m.to(torch.uint8).contiguous()
            cfg.obstacle_mask = V.ptr(self._mask)
        cfg.watchdog_every = int(watchdog_every)  # NaN/Inf scan every K steps of a run (check() reports it)
        self.cfg = cfg
        handle = C.c_void_p()
        V.call("vs_lattice_plan_create", C.byref(cfg), C.byref(handle))
        self.handle = handle

    @property
    def n_nodes(self):
        return int(np.prod(self.shape))

    def set_run_form(self, form):
        """'steps' (launches per time step, the default) or 'persistent' (one cooperative
        launch per run where it applies): vs_lattice_set_run_form.  Same bits either way."""
        codes = {"steps": V.VS_RUN_STEPS, "persistent": V.VS_RUN_PERSISTENT}
        if form not in codes:
            raise ValueError("form must be 'steps' or 'persistent'")
        V.call("vs_lattice_set_run_form", self.handle, codes[form])
        self.run_form = form

    def check(self, reset=True):
        """Raise if a grid kernel of this plan reported a device-side error, or the watchdog
        found a NaN/Inf population (synchronises)."""
        V.call("vs_lattice_status", self.handle, 1 if reset else 0, V.stream())

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            V.lib().vs_lattice_plan_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RigidBody:
    """Immersed rigid body: markers, IB stencil, MDF and a Newmark spring-mass update.

    ``free_dof`` names the Newmark-integrated DOFs: x, y, z in 3-D; x, y and the rotation
    angle about ``center`` in 2-D (get_markers_coords_3dof / get_markers_velocity_3dof /
    get_torque_to_obj, vivsim/dyn.py:84-154), the latter with ``inertia``,
    ``rot_stiffness``, ``rot_damping`` and h[2] = torque + a[2] * ``added_inertia``.
    ``fsi_iter`` (moving 2-D bodies) repeats markers, stencil, MDF, force and Newmark that
    many times per step, each pass from the latest state with Newmark restarting from the
    step's saved one: the FSI_ITER loop of examples/2d/vortex_induced_vibration.py:111-139.
    """

    def __init__(self, step, markers, ds, kernel="peskin4", radius=2, n_iter=3, moving=False,
                 free_dof=(False, False, False), mass=1.0, stiffness=0.0, damping=0.0, added_mass_area=0.0,
                 d0=(0, 0, 0), v0=(0, 0, 0), a0=(0, 0, 0), center=None, inertia=0.0, rot_stiffness=0.0,
                 rot_damping=0.0, added_inertia=0.0, fsi_iter=1):
        X = np.asarray(markers.cpu() if isinstance(markers, torch.Tensor) else markers, dtype=np.float64)
        if X.ndim != 2 or X.shape[1] != step.dim:
            raise ValueError(f"markers must have shape (n_markers, {step.dim})")
        self.step = step
        self.M = X.shape[0]
        self._cols = [np.ascontiguousarray(X[:, d]) for d in range(step.dim)]
        cfg = V.vs_body_cfg()
        cfg.dim = step.dim
        cfg.dtype = step.cfg.dtype
        cfg.n_markers = self.M
        P = C.POINTER(C.c_double)
        cfg.x0_host = self._cols[0].ctypes.data_as(P)
        cfg.y0_host = self._cols[1].ctypes.data_as(P)
        cfg.z0_host = self._cols[2].ctypes.data_as(P) if step.dim == 3 else None
        if np.ndim(ds) == 0:
            cfg.ds_scalar = float(ds)
            cfg.ds_host = None
        else:
            self._ds = np.ascontiguousarray(np.asarray(ds, dtype=np.float64).reshape(-1))
            cfg.ds_host = self._ds.ctypes.data_as(P)
        cfg.kernel = KERNELS[kernel]
        cfg.radius = int(radius)
        cfg.n_iter = int(n_iter)
        cfg.moving = 1 if moving else 0
        for i in range(3):
            cfg.free_dof[i] = 1 if (i < len(free_dof) and free_dof[i]) else 0
        cfg.mass, cfg.stiffness, cfg.damping = float(mass), float(stiffness), float(damping)
        cfg.added_mass_area = float(added_mass_area)
        if center is None:
            center = (float(np.mean(X[:, 0])), float(np.mean(X[:, 1])))
        cfg.center_x, cfg.center_y = float(center[0]), float(center[1])
        cfg.inertia, cfg.rot_stiffness = float(inertia), float(rot_stiffness)
        cfg.rot_damping, cfg.added_inertia = float(rot_damping), float(added_inertia)
        cfg.fsi_iter = int(fsi_iter)
        for name, val in (("d0", d0), ("v0", v0), ("a0", a0)):
            arr = getattr(cfg, name)
            for i in range(3):
                arr[i] = float(val[i]) if i < len(val) else 0.0
        self.cfg = cfg
        handle = C.c_void_p()
        V.call("vs_body_plan_create", C.byref(cfg), step.handle, C.byref(handle))
        self.handle = handle

    def state(self):
        """Body state as float64 numpy arrays a, v, d, h (3 each); synchronises."""
        buf = (C.c_double * 12)()
        V.call("vs_body_get_state", self.handle, buf, V.stream())
        a = np.frombuffer(buf, dtype=np.float64).copy()
        return dict(a=a[0:3], v=a[3:6], d=a[6:9], h=a[9:12])

    def set_state(self, a=(0, 0, 0), v=(0, 0, 0), d=(0, 0, 0)):
        buf = (C.c_double * 12)(*([float(x) for x in a] + [float(x) for x in v] + [float(x) for x in d] + [0.0] * 3))
        V.call("vs_body_set_state", self.handle, buf, V.stream())

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            V.lib().vs_body_plan_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Simulation:
    """Populations in two ping-pong device buffers advanced by the fused step."""

    def __init__(self, step, f0, body=None):
        V.require_cuda(f0)
        if tuple(f0.shape) != (step.q,) + step.shape:
            raise ValueError(f"f0 must have shape {(step.q,) + step.shape}")
        self.step = step
        self.body = body
        self._a = f0.to(step.dtype).contiguous().clone()
        self._b = torch.empty_like(self._a)
        self._cur_is_a = True

    @property
    def f(self):
        """Current populations (reference convention: after streaming and boundaries)."""
        return self._a if self._cur_is_a else self._b

    def save(self, path):
        """Checkpoint to an .npz file: the populations and the body state (a, v, d)."""
        data = {"f": self.f.detach().cpu().numpy()}
        if self.body is not None:
            st = self.body.state()
            data.update(a=st["a"], v=st["v"], d=st["d"])
        np.savez(path, **data)

    def load(self, path):
        """Resume from a checkpoint written by save(): the run continues bit for bit."""
        z = np.load(path)
        f = torch.from_numpy(z["f"])
        if tuple(f.shape) != tuple(self.f.shape):
            raise ValueError(f"checkpoint populations have shape {tuple(f.shape)}, expected {tuple(self.f.shape)}")
        self.f.copy_(f.to(device=self.f.device, dtype=self.f.dtype))
        if self.body is not None:
            if "d" not in z:
                raise ValueError("checkpoint holds no body state")
            self.body.set_state(a=z["a"], v=z["v"], d=z["d"])

    def run(self, n_steps, graph=False, force_history=False):
        """Advance n_steps; returns the (n_steps, 3) body-force history when asked."""
        if n_steps <= 0:
            return None
        src, dst = (self._a, self._b) if self._cur_is_a else (self._b, self._a)
        hist = None
        if force_history:
            hist = torch.empty((n_steps, 3), dtype=self.step.dtype, device=self._a.device)
        body = self.body.handle if self.body is not None else None
        fn = "vs_run_graph" if graph else "vs_run"
        V.call(fn, self.step.handle, body, V.ptr(src), V.ptr(dst), int(n_steps), V.ptr(hist), V.stream())
        if n_steps % 2 == 1:
            self._cur_is_a = not self._cur_is_a
        return hist

    def persistent(self, n_steps):
        """True when run(n_steps) advances all steps in one persistent launch (vs_run_persistent)."""
        body = self.body.handle if self.body is not None else None
        return bool(V.lib().vs_run_persistent(self.step.handle, body, int(n_steps)))

    def tune(self, trial_steps=200):
        """Choose the faster run form of this plan (LatticeStep.set_run_form): each form that
        applies runs trial_steps twice from a CUDA graph on a side stream, the second time
        timed with CUDA events; the faster stays set.  Advances the simulation by
        4 * trial_steps steps or fewer.  Returns {form: ms per step}."""
        old = getattr(self.step, "run_form", "steps")
        forms = ["steps"]
        self.step.set_run_form("persistent")
        if self.persistent(trial_steps):
            forms.append("persistent")
        cur = torch.cuda.current_stream()
        side = torch.cuda.Stream()
        side.wait_stream(cur)
        times = {}
        try:
            with torch.cuda.stream(side):
                for form in forms:
                    self.step.set_run_form(form)
                    self.run(trial_steps, graph=True)
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    self.run(trial_steps, graph=True)
                    e1.record()
                    e1.synchronize()
                    times[form] = e0.elapsed_time(e1) / trial_steps
        except Exception:
            self.step.set_run_form(old)
            raise
        cur.wait_stream(side)
        self.step.set_run_form(min(times, key=times.get))
        return times


class Batch:
    """Many independent simulations advanced together: per time step one body launch, one
    grid launch over all cases and one launch over all body boxes (vs_batch_run)."""

    def __init__(self, sims, threads_per_block=128, steps_per_graph=64, nodes_per_thread=1):
        self.sims = list(sims)
        n = len(self.sims)
        if n == 0:
            raise ValueError("a batch needs at least one simulation")
        lat = (C.c_void_p * n)(*[s.step.handle.value for s in self.sims])
        bod = (C.c_void_p * n)(*[(s.body.handle.value if s.body is not None else None) for s in self.sims])
        h = C.c_void_p()
        V.call("vs_batch_plan_create", lat, bod, n, C.byref(h))
        self.handle = h
        self.set_launch(threads_per_block, steps_per_graph, nodes_per_thread)

    def set_launch(self, threads_per_block=128, steps_per_graph=64, nodes_per_thread=1):
        V.call("vs_batch_set_launch", self.handle, int(threads_per_block), int(steps_per_graph))
        V.call("vs_batch_set_nodes_per_thread", self.handle, int(nodes_per_thread))
        self.threads_per_block, self.steps_per_graph = int(threads_per_block), int(steps_per_graph)
        self.nodes_per_thread = int(nodes_per_thread)

    def tune(self, trial_steps=64, candidates=None):
        """Pick the launch shape (threads per block, steps per graph, nodes per thread of the
        main launch) with the shortest time for `trial_steps` steps; each candidate runs
        twice (the first run builds its tables and graph) and the second is timed with CUDA
        events.  Advances the simulations by 2 * trial_steps * len(candidates) steps.
        Returns {(tb, spg, npt): ms per step}."""
        if candidates is None:
            candidates = [(tb, spg, npt) for npt in (1, 2) for tb in (64, 128, 256) for spg in (16, 64)]
        times = {}
        for cand in candidates:
            tb, spg, npt = (tuple(cand) + (1,))[:3]
            self.set_launch(tb, spg, npt)
            self.run(trial_steps)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            self.run(trial_steps)
            e1.record()
            torch.cuda.synchronize()
            times[(tb, spg, npt)] = e0.elapsed_time(e1) / trial_steps
        best = min(times, key=times.get)
        self.set_launch(*best)
        return times

    def run(self, n_steps):
        if n_steps <= 0:
            return
        n = len(self.sims)
        cur = [(s._a if s._cur_is_a else s._b) for s in self.sims]
        oth = [(s._b if s._cur_is_a else s._a) for s in self.sims]
        fa = (C.c_void_p * n)(*[V.ptr(t) for t in cur])
        fb = (C.c_void_p * n)(*[V.ptr(t) for t in oth])
        V.call("vs_batch_run", self.handle, fa, fb, int(n_steps), V.stream())
        if n_steps % 2 == 1:
            for s in self.sims:
                s._cur_is_a = not s._cur_is_a

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            V.lib().vs_batch_plan_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Refined:
    """Blocks of several refinement levels (vivsim/multigrid.py) advanced together.

    ``blocks`` are Simulations, one per block, each with its own LatticeStep (omega from
    ``multigrid.get_omega(nu, level)``, the block's own face boundaries); ``levels`` their
    refinement levels; ``links`` (coarse, fine, side) pairs of block indices whose levels
    differ by one, ``side`` being where the fine block lies relative to the coarse one
    ('left', 'right', 'up', 'down').  The coarse block carries the buffer line on that side.

    One cycle advances the coarsest level by one step, and level L by 2**(L - L_min) steps,
    recursively: the blocks of a level step (collide, stream, their boundaries); the
    coarse_to_fine transfer into each of them from its coarser neighbour's new state;
    then the next finer level runs two cycles and fine_to_coarse refills this level's
    buffer lines.  With ``graph=True`` two cycles (which bring every ping-pong
    buffer back to where it started) are captured once into a CUDA graph and replayed.
    """

    _F2C = {"right": "left", "left": "right", "up": "down", "down": "up"}

    def __init__(self, blocks, levels, links):
        from . import multigrid as _mg
        self._mg = _mg
        self.blocks = list(blocks)
        self.levels = [int(x) for x in levels]
        if len(self.levels) != len(self.blocks) or not self.blocks:
            raise ValueError("one level per block, at least one block")
        for b in self.blocks:
            if b.step.q != 9 or b.body is not None:
                raise ValueError("refined blocks are D2Q9 lattices without bodies (vivsim/multigrid.py)")
        self.links = []
        for c, f, side in links:
            if side not in self._F2C:
                raise ValueError("side must be one of 'left', 'right', 'up', 'down'")
            if self.levels[f] != self.levels[c] + 1:
                raise ValueError("a link joins a block to a block exactly one level finer")
            self.links.append((int(c), int(f), side))
        self.lmin, self.lmax = min(self.levels), max(self.levels)
        self._graph = None
        self._graph_parity = None

    def f(self, i):
        return self.blocks[i].f

    def _step(self, i):
        b = self.blocks[i]
        src, dst = (b._a, b._b) if b._cur_is_a else (b._b, b._a)
        V.call("vs_step", b.step.handle, None, V.ptr(src), V.ptr(dst), None, V.stream())
        b._cur_is_a = not b._cur_is_a

    def _cycle(self, level):
        for i, lv in enumerate(self.levels):
            if lv == level:
                self._step(i)
        for c, f, side in self.links:
            if self.levels[f] == level:
                self._mg.transfer_("coarse_to_fine", self.f(c), self.f(f), side)
        if level < self.lmax:
            self._cycle(level + 1)
            self._cycle(level + 1)
            for c, f, side in self.links:
                if self.levels[c] == level:
                    self._mg.transfer_("fine_to_coarse", self.f(f), self.f(c), self._F2C[side])

    def _parity(self):
        return tuple(b._cur_is_a for b in self.blocks)

    def run(self, n_cycles, graph=False):
        """Advance n_cycles steps of the coarsest level."""
        n = int(n_cycles)
        if not graph:
            for _ in range(n):
                self._cycle(self.lmin)
            return
        while n > 0:
            if self._graph is None and n >= 3:
                self._cycle(self.lmin)  # first launches (lazy attributes) outside the capture
                n -= 1
                g = torch.cuda.CUDAGraph()
                s = torch.cuda.Stream()
                s.wait_stream(torch.cuda.current_stream())
                with torch.cuda.stream(s):
                    saved = self._parity()
                    g.capture_begin()
                    self._cycle(self.lmin)
                    self._cycle(self.lmin)
                    g.capture_end()
                    for b, p in zip(self.blocks, saved):  # capture launched nothing
                        b._cur_is_a = p
                torch.cuda.current_stream().wait_stream(s)
                self._graph, self._graph_parity = g, saved
            if self._graph is not None and n >= 2 and self._parity() == self._graph_parity:
                self._graph.replay()
                n -= 2
            else:
                self._cycle(self.lmin)
                n -= 1
