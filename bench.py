#!/usr/bin/env python
"""Benchmark of the fused IB-LBM time step (MLUPS) on one GB300, plus HBM-roofline cases.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Headline workload (default): the 2-D cylinder VIV case, D2Q9 KBC on 1024 x 512 with a
126-marker spring-mounted cylinder, MDF 3 iterations (vivsim_gb300.configs.viv2d).  One
bench step = `--chunk` time steps replayed from a CUDA graph; L2 is flushed (a 512 MiB
write) before every bench step, so each bench step starts from HBM.  MLUPS = nodes x
time steps / seconds / 1e6.

Extra measurements on the same line: the grid kernel's HBM roofline on this case and on
two HBM-bound cases (D3Q19 regularised sphere 256 x 128 x 128, D2Q9 KBC 8192 x 8192),
the end-to-end rate through the public API with host buffers, and a CPU baseline (the
NumPy oracle on the host).  ``--impl reference`` times the CPU implementation alone.

Multi-GPU (torchrun): every rank advances its own replica (no exchange): weak scaling.
"""

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

BYTES_PER_UPDATE = {9: 72, 19: 152}  # f32: each population read once and written once


def parse():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["viv2d", "cavity", "sphere3d", "periodic2d"], default="viv2d")
    ap.add_argument("--chunk", type=int, default=500, help="time steps per bench step")
    ap.add_argument("--no-extras", action="store_true", help="skip the HBM-bound roofline cases")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU-baseline sample budget")
    ap.add_argument("--batch-steps", type=int, default=5000, help="time steps of the batched-sweep comparison")
    ap.add_argument("--adjoint-steps", type=int, default=4000, help="time steps of the adjoint timing")
    return ap.parse_args()


# ------------------------------------------------------------------------ utilities

def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profiles(workload):
    """Per-launch DRAM bytes of the grid kernel from the committed ncu summary, if any."""
    path = os.path.join(HERE, "profiles", "dram_traffic.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == workload:
                return float(parts[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        import threading
        self.lines = []
        self._first = threading.Event()
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "50",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return self

        def reader():
            for ln in self.proc.stdout:
                if ln.strip():
                    self.lines.append(ln)
                    self._first.set()
            self._first.set()

        self._thread = threading.Thread(target=reader, daemon=True)
        self._thread.start()
        self._first.wait(timeout=5.0)  # sampling is running before the timed region starts
        self._start = len(self.lines)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self._stop = len(self.lines)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.proc.wait()
            self._thread.join(timeout=5)
            # samples taken while the timed region ran (plus the one just before it)
            self.lines = self.lines[max(0, self._start - 1):max(self._stop, self._start)]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for name, val in zip(names, p[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------- GPU timing

def build_case(name, chunk_hint=None):
    from vivsim_gb300 import configs
    return configs.CASES[name]()


def time_chunks(torch, run, K, W, flush):
    """W untimed + K timed bench steps; L2 flushed before each; device time per step."""
    for _ in range(W):
        flush()
        run()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    for k in range(K):
        flush()
        ev[k][0].record()
        run()
        ev[k][1].record()
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / 1e3


def grid_kernel_time(torch, step, body, sim, launches, flush):
    """Average duration of the grid kernel alone (vs_step_grid_only), L2 flushed once.  The
    kernel is timed over the whole grid without the body: the bulk launch of a step, which
    in a step leaves only the body's small box to another launch."""
    from vivsim_gb300 import _lib as V
    a = sim.f
    b = torch.empty_like(a)
    bh = None
    flush()
    V.call("vs_step_grid_only", step.handle, bh, V.ptr(a), V.ptr(b), V.stream())
    torch.cuda.synchronize()
    flush()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    src, dst = a, b
    for _ in range(launches):
        V.call("vs_step_grid_only", step.handle, bh, V.ptr(src), V.ptr(dst), V.stream())
        src, dst = dst, src
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3 / launches


def roofline(torch, case, step, body, sim, flush, peak, peak_kind, launches):
    t = grid_kernel_time(torch, step, body, sim, launches, flush)
    n = int(math.prod(case["shape"]))
    bytes_per_launch = BYTES_PER_UPDATE[case["q"]] * n
    achieved = bytes_per_launch / t / 1e9
    return {"kernel": "k_step_fast (grid: collide + push-stream, bulk launch)", "workload": case["name"], "bound": "hbm",
            "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
            "peak_source": f"{peak_kind} hbm_gbs", "bytes_per_launch": bytes_per_launch,
            "traffic": traffic_from_profiles(case["name"]), "kernel_us": round(t * 1e6, 3),
            "kernel_mlups": round(n / t / 1e6, 1)}


def batched_vs_sequential(torch, steps, n_cases=64, seed=3):
    """The uneven VIV sweep (vivsim_gb300.configs.viv_sweep): every case's loop run one
    after the other with plain launches (vs_run), against all cases advanced together
    (vs_batch_run, launch shape from the autotuner, graph replay).  Aggregate MLUPS."""
    from vivsim_gb300 import configs, solver
    cases = configs.viv_sweep(n_cases, seed)
    nodes = sum(int(math.prod(c["shape"])) for c in cases)
    seq = [configs.build_solver(c)[2] for c in cases]
    for sim in seq:
        sim.run(2)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for sim in seq:
        sim.run(steps)
    e1.record()
    torch.cuda.synchronize()
    t_seq = e0.elapsed_time(e1) / 1e3
    del seq
    bat = [configs.build_solver(c)[2] for c in cases]
    batch = solver.Batch(bat)
    tuned = batch.tune(trial_steps=32)
    batch.run(steps)  # tables and graph for this buffer parity (untimed)
    torch.cuda.synchronize()
    e0.record()
    batch.run(steps)
    e1.record()
    torch.cuda.synchronize()
    t_bat = e0.elapsed_time(e1) / 1e3
    m_seq, m_bat = nodes * steps / t_seq / 1e6, nodes * steps / t_bat / 1e6
    return {"workload": f"viv_sweep_{n_cases}_cases_seed{seed}_d2q9_kbc", "cases": n_cases, "nodes": nodes,
            "time_steps": steps, "sequential_plain_mlups": round(m_seq, 1), "batched_mlups": round(m_bat, 1),
            "batched_over_sequential": round(m_bat / m_seq, 2),
            "launch_shape": {"threads_per_block": batch.threads_per_block,
                             "steps_per_graph": batch.steps_per_graph, "nodes_per_thread": batch.nodes_per_thread},
            "tuning_ms_per_step": {f"{k[0]}x{k[1]}x{k[2]}": round(v, 4) for k, v in tuned.items()}}


def adjoint_over_forward(torch, steps):
    """Differentiable cylinder (D2Q9 BGK 512 x 256, D = 20, 64 markers, 1-DOF spring,
    checkpoint every 100 steps, objective = mean drag over the second half): time of the
    forward run alone vs the forward run with checkpoints plus the reverse sweep."""
    import numpy as np
    from vivsim_gb300 import adjoint
    off = np.random.default_rng(2).normal(0.0, 0.1, 64)
    plan = adjoint.CylinderDrag(nx=512, ny=256, D=20.0, Re=100.0, n_markers=64, offsets=off, n_steps=steps,
                                checkpoint_every=100, obj_start=steps // 2)
    plan.forward(keep_checkpoints=True)
    plan.backward()  # captures the graphs (untimed)
    torch.cuda.synchronize()

    def timed(fn):  # CUDA events on the stream the plan launches on (each call ends with a sync)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize()
        return out, e0.elapsed_time(e1) / 1e3

    J, t_fwd = timed(lambda: plan.forward(keep_checkpoints=False))
    _, t_fck = timed(lambda: plan.forward(keep_checkpoints=True))
    (gU0, gK, goff), t_bwd = timed(plan.backward)
    plan.close()
    return {"workload": f"diff_cylinder_d2q9_bgk_512x256_m64_{steps}steps_ckpt100", "objective": J,
            "forward_s": round(t_fwd, 4), "forward_with_checkpoints_s": round(t_fck, 4),
            "reverse_s": round(t_bwd, 4), "adjoint_over_forward": round(t_bwd / t_fwd, 3),
            "gradient_over_forward": round((t_fck + t_bwd) / t_fwd, 3),
            "grad_U0": gU0, "grad_stiffness": gK, "grad_offsets_norm": float(np.linalg.norm(goff)),
            "timing": "CUDA events on the launching stream around each call (each call ends with a stream sync)"}


def job_seconds(torch, dist, secs, device):
    """The job's time: the maximum over ranks of each rank's timed-region seconds."""
    if dist is None:
        return secs
    t = torch.tensor([secs], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def aggregate_rate(units_per_rank, world, secs):
    """Whole-job rate in millions of units per second: every rank (replica) processed
    units_per_rank within the job's time."""
    return units_per_rank * world / secs / 1e6


def gb300_arm(args, world, rank, local):
    import numpy as np
    import torch
    import __graft_entry__ as g
    g.build()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    peak, peak_kind = peaks()
    stream = torch.cuda.Stream()
    flush_buf = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush():
        flush_buf.fill_(1.0)

    from vivsim_gb300 import configs
    case = build_case(args.workload)
    n = int(math.prod(case["shape"]))
    with torch.cuda.stream(stream):
        step, body, sim = configs.build_solver(case)
        run = lambda: sim.run(args.chunk, graph=True)  # noqa: E731
        run()  # capture the graph once (untimed)
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        try:
            gpu_id = "GPU-" + str(torch.cuda.get_device_properties(local).uuid)
        except Exception:
            gpu_id = str(local)
        with ClockSampler(gpu_id) as clk:
            secs = time_chunks(torch, run, args.steps, args.warmup, flush)
        torch.cuda.synchronize()
        secs = job_seconds(torch, dist, secs, "cuda")
        mlups = aggregate_rate(n * args.chunk * args.steps, world, secs)
        # with a body: body kernel, grid launch outside its box, box launch; the x-face
        # boundaries of these cases run on the next step's load and once at the end of a chunk.
        # The persistent form: one launch per chunk plus the chunk's closing face launch.
        persistent = sim.persistent(args.chunk)
        if persistent:
            launches_per_chunk = 1 + step_groups(case)
        else:
            launches_per_step = 3 if body is not None else 1 + step_groups(case)
            launches_per_chunk = launches_per_step * args.chunk + (step_groups(case) if body is not None else 0)
        rl = roofline(torch, case, step, body, sim, flush, peak, peak_kind, 2 * args.chunk)

        # end to end through the public API with host buffers: H2D f, chunk, D2H f
        f_host = torch.from_numpy(case["f0"]).pin_memory()
        out_host = torch.empty_like(f_host).pin_memory()
        e2e_sim = configs.build_solver(case)[2]

        def e2e_run():
            e2e_sim.f.copy_(f_host, non_blocking=True)
            e2e_sim.run(args.chunk, graph=True)
            out_host.copy_(e2e_sim.f, non_blocking=True)

        e2e_run()
        torch.cuda.synchronize()
        e2e_secs = time_chunks(torch, e2e_run, max(3, args.steps // 2), 2, flush)
        e2e_mlups = n * args.chunk * max(3, args.steps // 2) / e2e_secs / 1e6
        fbytes = int(f_host.numel() * f_host.element_size())

        extras = {}
        extras_batch = None
        extras_adj = None
        if not args.no_extras and rank == 0:
            del e2e_sim
            for name in ("sphere3d", "periodic2d"):
                if name == args.workload:
                    continue
                c2 = build_case(name)
                st2, bd2, sm2 = configs.build_solver(c2)
                r2 = lambda: sm2.run(50, graph=True)  # noqa: E731
                r2()
                torch.cuda.synchronize()
                s2 = time_chunks(torch, r2, 5, 2, flush)
                extras[name] = {
                    "workload": c2["name"], "time_steps": 50 * 5,
                    "mlups": round(int(math.prod(c2["shape"])) * 50 * 5 / s2 / 1e6, 1),
                    "roofline": roofline(torch, c2, st2, bd2, sm2, flush, peak, peak_kind, 10)}
                del st2, bd2, sm2, c2
                torch.cuda.empty_cache()
            extras_batch = batched_vs_sequential(torch, args.batch_steps)
            torch.cuda.empty_cache()
            extras_adj = adjoint_over_forward(torch, args.adjoint_steps)
            torch.cuda.empty_cache()
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    cpu = cpu_baseline(case, args.cpu_seconds)
    clocks = clk.summary()
    line = {
        "metric": "MLUPS (fused IB-LBM step; HBM roofline per fused step)",
        "value": round(mlups, 1),
        "unit": "MLUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(secs / args.steps * 1e3, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded numpy draws of the named configuration)",
        "config": arm_config(case, world),
        "time_steps_per_bench_step": args.chunk,
        "l2": "flushed (512 MiB write) before every bench step; the two population buffers "
              f"({2 * n * BYTES_PER_UPDATE[case['q']] // 2 / 1e6:.1f} MB) stay L2-resident within one",
        "roofline": rl,
        "roofline_hbm_bound": extras,
        "batched_vs_sequential": extras_batch,
        "adjoint": extras_adj,
        "e2e": {"value": round(e2e_mlups, 1), "unit": "MLUPS", "h2d_bytes_per_step": fbytes,
                "d2h_bytes_per_step": fbytes,
                "path": "vivsim_gb300.solver.Simulation.run from pinned host populations"},
        "gpu_launches": launches_per_chunk * args.steps,
        "step_form": "persistent (one cooperative launch per bench step)" if persistent else "one launch group per step",
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def arm_config(case, world):
    """The workload as both arms name it (the same dict on the GPU arm and the reference arm)."""
    return {"workload": case["name"], "nodes": int(math.prod(case["shape"])),
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


def step_groups(case):
    """Face-kernel launches per step (opposite faces of one axis share a launch)."""
    groups, size, prev = 0, 0, None
    axis = {"left": 0, "right": 0, "bottom": 1, "top": 1, "back": 2, "front": 2}
    for (_, loc, _, _) in case["boundaries"]:
        if prev is not None and size == 1 and axis[prev] == axis[loc] and prev != loc:
            size = 2
        else:
            groups += 1
            size = 1
        prev = loc
    return groups


# -------------------------------------------------------------------- CPU side

def oracle_stepper(case):
    """A closure running one time step of `case` with the NumPy oracle."""
    import numpy as np

    from oracle import ib as OIB
    from oracle import lbm2d as L2
    from oracle import recipes
    names = {("nee", "given"): "nee", ("nebb", "given"): "nebb", ("equilibrium", "given"): "eq",
             ("nee", "pressure"): "pnee", ("nee", "velocity"): "vnee", ("nebb", "force_corrected"): "fcnebb"}
    bcs = [(names[(k, m)], loc, kw) for (k, loc, m, kw) in case["boundaries"]]
    state = {"f": case["f0"].copy()}
    q, coll, om = case["q"], case["collision"], case["omega"]
    b = case["body"]
    if q == 9 and b is not None:
        X = b["markers"].astype(np.float32)
        body = recipes.Body2D(X[:, 0], X[:, 1], b["ds"], b["mass"], b["stiffness"], b["damping"],
                              b["added_mass_area"], free=b["free_dof"][:2], kernel=b["kernel"], n_iter=b["n_iter"])
        op = L2.get_mrt_collision_operator(om, np.float32) if coll == "mrt" else None

        def one():
            state["f"], _ = recipes.ib_lbm_step_2d(state["f"], body, coll, om, op, bcs)
    elif q == 19 and b is not None:
        X = b["markers"].astype(np.float32)
        W, I = OIB.get_ib_stencil_3d(X, case["shape"])
        zero = np.zeros((X.shape[0], 3), np.float32)

        def one():
            state["f"], _ = recipes.ib_lbm_step_3d(state["f"], W, I, zero, b["ds"], coll, om, None, bcs, b["n_iter"])
    elif q == 9 and coll == "bgk" and len(bcs) == 4:
        def one():
            state["f"] = recipes.cavity_step(state["f"], om, case["boundaries"][0][3].get("ux_wall", 0.0))
    else:
        def one():
            state["f"] = recipes.lbm_step_2d(state["f"], coll, om, None, bcs) if q == 9 else \
                recipes.lbm_step_3d(state["f"], coll, om, None, bcs)
    return one


def cpu_stepper(case):
    """(step closure, threads, description): the oracle's step over all host cores
    (oracle/threaded.py, bit-equal to the serial restatement), or the serial one where
    the threaded step does not apply (3-D bodies)."""
    from oracle.threaded import ThreadedStep
    try:
        t = ThreadedStep(case)
    except NotImplementedError:
        return oracle_stepper(case), 1, "NumPy restatement of the reference, single thread"
    return t, t.threads, f"NumPy restatement of the reference, node stages split over {t.threads} threads"


def cpu_baseline(case, budget_s):
    """The oracle on the host's cores on a bounded sample of the same workload: full grid,
    few steps."""
    one, cores, what = cpu_stepper(case)
    n = int(math.prod(case["shape"]))
    t0 = time.perf_counter()
    one()  # first step (allocation warm-up) is timed too, it is a full step
    steps = 1
    while time.perf_counter() - t0 < budget_s and steps < 200:
        one()
        steps += 1
    secs = time.perf_counter() - t0
    return {"value": round(n * steps / secs / 1e6, 3), "unit": "MLUPS", "cores": cores, "kind": "port",
            "sample": f"{steps} time steps of {case['name']} on the full grid ({what})"}


REF_DIR = os.path.join(HERE, "baseline", "_ref")


def reference_probe():
    """Can the reference itself run here?  vivsim is installed without its dependencies
    under baseline/_ref; its JAX path needs JAX.  Returns (True, detail) or (False, why)."""
    if not os.path.isdir(os.path.join(REF_DIR, "vivsim")):
        return False, "the reference is not installed under baseline/_ref"
    try:
        import jax  # noqa: F401
    except Exception as e:  # ImportError, or a broken install
        return False, f"vivsim is installed under baseline/_ref but import jax failed ({type(e).__name__}: {e})"
    return True, f"jax {jax.__version__}"


def reference_jax_stepper(case, chunk):
    """The reference's own time step for `case`: vivsim's functions (from baseline/_ref)
    composed as its examples compose them (examples/2d/lid_driven_cavity.py:55-63,
    examples/2d/vortex_induced_vibration.py:96-148 with a full-grid stencil,
    examples/3d/flow_past_sphere.py:139-180 with a static stencil), jitted over a
    lax.scan of `chunk` steps on the host CPU in float32.  Returns (run, threads, what):
    run() advances `chunk` steps and blocks until they are done."""
    os.environ.setdefault("JAX_PLATFORMS", "cpu")
    if REF_DIR not in sys.path:
        sys.path.insert(0, REF_DIR)
    import jax
    import jax.numpy as jnp
    from vivsim import dyn, ib, ib3d, lbm, lbm3d

    q, coll, om = case["q"], case["collision"], case["omega"]
    L = lbm if q == 9 else lbm3d
    names = {("nee", "given"): "boundary_nee", ("nebb", "given"): "boundary_nebb",
             ("equilibrium", "given"): "boundary_equilibrium", ("nee", "pressure"): "boundary_pressure_nee",
             ("nee", "velocity"): "boundary_velocity_nee", ("nebb", "force_corrected"): "boundary_force_corrected_nebb"}
    bcs = [(getattr(L, names[(k, m)]), loc, kw) for (k, loc, m, kw) in case["boundaries"]]
    if coll == "mrt":
        mrt_op = L.get_mrt_collision_operator(om)
        collide = lambda f, feq: L.collision_mrt(f, feq, mrt_op)  # noqa: E731
    else:
        fn = {"bgk": L.collision_bgk, "kbc": L.collision_kbc, "reg": L.collision_reg}[coll]
        collide = lambda f, feq: fn(f, feq, om)  # noqa: E731
    b = case["body"]
    kern = {"peskin3": ib.kernel_peskin_3pt, "peskin4": ib.kernel_peskin_4pt, "cosine4": ib.kernel_cosine_4pt}
    if b is not None and q == 19:
        X = jnp.asarray(b["markers"], jnp.float32)
        W3, I3 = ib3d.get_ib_stencil(X, tuple(case["shape"]), kernel=kern[b["kernel"]], stencil_radius=b["radius"])
        mu0 = jnp.zeros((X.shape[0], 3), jnp.float32)
    if b is not None and q == 9:
        X0 = jnp.asarray(b["markers"][:, 0], jnp.float32)
        Y0 = jnp.asarray(b["markers"][:, 1], jnp.float32)
        ny = case["shape"][1]
        free = b["free_dof"][:2]

    def step(carry, _):
        f, a, v, d = carry
        rho, u = L.get_macroscopic(f)
        f = collide(f, L.get_equilibrium(rho, u))
        if b is not None and q == 9:
            mx, my = dyn.get_markers_coords_2dof(X0, Y0, d)
            W, I = ib.get_ib_stencil(mx, my, ny, kernel=kern[b["kernel"]], stencil_radius=b["radius"])
            mv = jnp.repeat(v[None, :], X0.shape[0], axis=0)
            g, mh = ib.multi_direct_forcing(u, W, I, mv, b["ds"], n_iter=b["n_iter"])
            h = dyn.get_force_to_obj(mh) + a * b["added_mass_area"]
            an, vn, dn = dyn.newmark(a, v, d, h, b["mass"], b["stiffness"], b["damping"])
            keep = jnp.asarray([0.0 if fr else 1.0 for fr in free], jnp.float32)
            a, v, d = (keep * a + (1 - keep) * an, keep * v + (1 - keep) * vn, keep * d + (1 - keep) * dn)
            f = L.forcing_edm(f, g, u)
        elif b is not None:
            g, _mh = ib.multi_direct_forcing(u, W3, I3, mu0, b["ds"], n_iter=b["n_iter"])
            f = L.forcing_edm(f, g, u)
        f = L.streaming(f)
        for fn, loc, kw in bcs:
            f = fn(f, loc=loc, **kw)
        return (f, a, v, d), None

    run_chunk = jax.jit(lambda carry: jax.lax.scan(step, carry, None, length=chunk)[0])
    z = jnp.zeros(2, jnp.float32)
    state = {"c": (jnp.asarray(case["f0"]), z, z, z)}

    def run():
        state["c"] = jax.block_until_ready(run_chunk(state["c"]))

    threads = os.cpu_count() or 1
    return run, threads, f"the reference's own JAX path (jit + lax.scan of {chunk} steps, XLA CPU)"


def reference_arm(args, world, rank):
    if rank != 0:
        return
    from vivsim_gb300 import configs
    case = configs.CASES[args.workload]()
    n = int(math.prod(case["shape"]))
    ok, probe = reference_probe()
    if ok:  # the reference's own JAX CPU path: a bench step is one scanned chunk of steps
        chunk = 10
        one, cores, what = reference_jax_stepper(case, chunk)
        kind = "reference"
    else:  # the oracle's restatement of the reference over the host cores
        chunk = 1
        one, cores, what = cpu_stepper(case)
        kind = "port"
    for _ in range(args.warmup):
        one()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one()
    secs = time.perf_counter() - t0
    v = n * chunk * args.steps / secs / 1e6
    line = {
        "impl": "reference", "metric": "MLUPS (fused IB-LBM step; HBM roofline per fused step)", "value": round(v, 3),
        "unit": "MLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(secs / args.steps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded numpy draws of the named configuration)",
        "config": arm_config(case, world),
        "time_steps_per_bench_step": chunk,
        "reference_probe": probe,
        "cpu_baseline": {"value": round(v, 3), "unit": "MLUPS", "cores": cores, "kind": kind,
                         "sample": f"{args.steps * chunk} timed time steps of {case['name']} on the full grid "
                                   f"({what})"},
        "e2e": {"value": round(v, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_info()
    if args.impl == "reference":
        reference_arm(args, world, rank)
    else:
        gb300_arm(args, world, rank, local)


if __name__ == "__main__":
    main()
