"""Run a few fused steps of a benchmark case, for profilers (ncu) and quick timing.

    python -m vivsim_gb300.profile_case --case periodic2d --n 4096 --steps 3
    python -m vivsim_gb300.profile_case --case sphere3d --steps 3
    python -m vivsim_gb300.profile_case --case viv2d --steps 20 --graph

Each step launches the body kernel (cases with a body), the grid kernel ``k_step`` and
the face kernel(s); ``--grid-only`` launches only ``k_step``.  Prints the mean step time.
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
    ap.add_argument("--variant", choices=["auto", "plain", "tma"], default="auto")
    a = ap.parse_args()
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
            bh = body.handle if body is not None else None
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


if __name__ == "__main__":
    main()
