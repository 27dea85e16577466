"""Run a few fused steps of a benchmark case, for profilers (ncu) and quick timing.

    python -m vivsim_gb300.profile_case --case periodic2d --n 4096 --steps 3
    python -m vivsim_gb300.profile_case --case sphere3d --steps 3
    python -m vivsim_gb300.profile_case --case viv2d --steps 20 --graph
    python -m vivsim_gb300.profile_case --batch 64 --steps 8 [--npt 2]
    python -m vivsim_gb300.profile_case --adjoint --steps 400

Each step launches the body kernel (cases with a body), the grid kernel ``k_step`` and
the face kernel(s); ``--grid-only`` launches only the grid kernel (with ``--no-body`` the
whole grid's bulk launch ``k_step_fast``, as bench.py's roofline times it).  ``--batch N`` runs the
N-case VIV sweep as one batch (seed 3, as bench.py), ``--adjoint`` the differentiable
cylinder's forward and reverse sweep over ``--steps`` steps.  Prints the mean step time.
"""

import argparse
import math

import torch

from . import _lib as V
from . import configs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", choices=sorted(configs.CASES), default="viv2d")
    ap.add_argument("--n", type=int, default=None, help="periodic2d / cavity edge length")
    ap.add_argument("--collision", default=None)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--graph", action="store_true")
    ap.add_argument("--grid-only", action="store_true")
    ap.add_argument("--no-body", action="store_true",
                    help="with --grid-only: the whole grid without the body (the bulk launch bench.py times)")
    ap.add_argument("--npt", type=int, default=1, help="--batch: nodes per thread of the main launch")
    ap.add_argument("--variant", choices=["auto", "plain", "tma"], default="auto")
    ap.add_argument("--batch", type=int, default=0, help="run the N-case VIV sweep as one batch")
    ap.add_argument("--adjoint", action="store_true", help="forward + reverse sweep of the adjoint cylinder")
    a = ap.parse_args()
    if a.batch:
        return batch(a.batch, a.steps, a.npt)
    if a.adjoint:
        return adjoint(a.steps)
    kw = {}
    if a.n is not None and a.case in ("periodic2d", "cavity"):
        kw["n"] = a.n
    if a.collision:
        kw["collision"] = a.collision
    case = configs.CASES[a.case](**kw)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        step, body, sim = configs.build_solver(case, variant=a.variant)
        if a.graph and not a.grid_only:
            sim.run(a.steps, graph=True)  # capture (untimed)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        if a.grid_only:
            src, dst = sim.f, torch.empty_like(sim.f)
            bh = body.handle if body is not None and not a.no_body else None
            for _ in range(a.steps):
                V.call("vs_step_grid_only", step.handle, bh, V.ptr(src), V.ptr(dst), V.stream())
                src, dst = dst, src
        else:
            sim.run(a.steps, graph=a.graph)
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.steps
    n = math.prod(case["shape"])
    print(f"{case['name']}: {ms * 1e3:.1f} us/step, {n / ms / 1e3:.1f} MLUPS")


def _timed(fn):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def batch(n_cases, steps, npt=1):
    from . import solver
    cases = configs.viv_sweep(n_cases, 3)
    nodes = sum(math.prod(c["shape"]) for c in cases)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        b = solver.Batch([configs.build_solver(c)[2] for c in cases], threads_per_block=64, steps_per_graph=0,
                         nodes_per_thread=npt)
        b.run(2)
        torch.cuda.synchronize()
        ms = _timed(lambda: b.run(steps)) / steps
    print(f"batch of {n_cases} VIV cases ({nodes} nodes): {ms * 1e3:.1f} us/step, {nodes / ms / 1e3:.1f} MLUPS")


def adjoint(steps):
    import numpy as np
    from . import adjoint as A
    off = np.random.default_rng(2).normal(0.0, 0.1, 64)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        plan = A.CylinderDrag(nx=512, ny=256, D=20.0, Re=100.0, n_markers=64, offsets=off, n_steps=steps,
                              checkpoint_every=100, obj_start=steps // 2)
        plan.forward()
        ms_f = _timed(plan.forward)
        ms_b = _timed(plan.backward)
        plan.close()
    print(f"adjoint cylinder, {steps} steps: forward {ms_f:.2f} ms, reverse sweep {ms_b:.2f} ms")


if __name__ == "__main__":
    main()
