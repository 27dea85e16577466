"""Float32 drift of the oracle itself: the oracle run in float32 and in float64 from the same
float32 initial state, compared at checkpoints.

    python -m oracle.drift --case viv2d --steps 20000 --at 1000 2000 5000 20000

Test infrastructure, like the rest of ``oracle/``: it measures how far a float32 run of the
reference's arithmetic drifts from float64 on a benchmark configuration, which is the yard
stick for the fused float32 step's own drift (the product never runs it).  Each line is
JSON: the step count and the norm-relative errors max|a - b| / max|b| of rho and u (moments
taken in float64), and with ``--perturb`` also the distance between the float64 run and a
float64 run whose initial state differs by one float32 ulp in population 0 at every 97th
node (how much the flow itself amplifies a rounding-sized change over the same steps).
"""

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import lbm2d as L2  # noqa: E402
from oracle import lbm3d as L3  # noqa: E402
from oracle.threaded import ThreadedStep  # noqa: E402


def moments(f):
    f = np.asarray(f, np.float64)
    return (L2 if f.shape[0] == 9 else L3).get_macroscopic(f)


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def perturbed(f0):
    """One float32 ulp added to population 0 at every 97th node (memory order)."""
    fp = np.array(f0, copy=True)
    flat = fp.reshape(fp.shape[0], -1)
    flat[0, ::97] = np.nextafter(flat[0, ::97], np.float32(2.0))
    return fp


def main():
    from vivsim_gb300 import configs  # the benchmark configurations (plain NumPy)

    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="viv2d", choices=sorted(configs.CASES))
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--at", type=int, nargs="*", default=None, help="checkpoints (default: the last step)")
    ap.add_argument("--perturb", action="store_true")
    a = ap.parse_args()
    at = sorted(set(a.at or []) | {a.steps})
    case = configs.CASES[a.case]()
    runs = {"o32": ThreadedStep(case), "o64": ThreadedStep(case, dtype=np.float64)}
    if a.perturb:
        cp = dict(case, f0=perturbed(case["f0"]))
        runs["o64p"] = ThreadedStep(cp, dtype=np.float64)
    t0 = time.time()
    for n in range(1, a.steps + 1):
        for r in runs.values():
            r()
        if n in at:
            r32, u32 = moments(runs["o32"].f)
            r64, u64 = moments(runs["o64"].f)
            out = dict(case=case["name"], steps=n, oracle32_vs_64_rho=rel(r32, r64), oracle32_vs_64_u=rel(u32, u64),
                       seconds=round(time.time() - t0, 1))
            if a.perturb:
                rp, up = moments(runs["o64p"].f)
                out.update(perturbed64_vs_64_rho=rel(rp, r64), perturbed64_vs_64_u=rel(up, u64))
            print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
