"""Error of the float32 fused step against float64 over whole runs of the benchmark cases.

    python -m vivsim_gb300.accuracy [--cases cavity viv2d sphere3d] [--out FILE]

Each case runs its full step count in float32 and in float64 (the float64 fused step
matches the float64 oracle to ~1e-12 per step) from the same float32 initial state, and
the norm-relative differences max|a - b| / max|b| of rho and u (and of the body
displacement) are printed as one JSON line per case.
"""

import argparse
import json

import torch

from . import configs

FULL_STEPS = {"cavity": 1000, "viv2d": 20000, "sphere3d": 5000}


def _velocities(q, dtype, device):
    if q == 9:
        c = [[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]]
    else:
        c = [[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [1, 1, 0], [-1, 1, 0],
             [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1], [0, 1, 1], [0, -1, 1],
             [0, 1, -1], [0, -1, -1]]
    return torch.tensor(c, dtype=dtype, device=device)


def rho_u(f):
    f = f.double()
    c = _velocities(f.shape[0], f.dtype, f.device)
    rho = f.sum(0)
    u = torch.einsum("qd,q...->d...", c, f) / rho
    return rho, u


def run(name, steps, dtype, chunk=500):
    case = configs.CASES[name]()
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        step, body, sim = configs.build_solver(case, dtype=dtype)
        done = 0
        while done < steps:
            k = min(chunk, steps - done)
            sim.run(k, graph=True)
            done += k
        torch.cuda.synchronize()
        step.check()
        d = body.state()["d"] if body is not None else None
        return sim.f.clone(), d


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


def compare(name, steps):
    f32, d32 = run(name, steps, torch.float32)
    f64, d64 = run(name, steps, torch.float64)
    r32, u32 = rho_u(f32)
    r64, u64 = rho_u(f64)
    out = {"case": configs.CASES[name]()["name"], "steps": steps, "rho_rel_err": rel(r32, r64),
           "u_rel_err": rel(u32, u64)}
    if d32 is not None:
        out["body_d"] = {"f32": [float(x) for x in d32[:2]], "f64": [float(x) for x in d64[:2]]}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cases", nargs="*", default=list(FULL_STEPS))
    ap.add_argument("--steps", type=int, default=None, help="override the full step count")
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    lines = []
    for name in a.cases:
        res = compare(name, a.steps or FULL_STEPS[name])
        print(json.dumps(res), flush=True)
        lines.append(res)
    if a.out:
        with open(a.out, "w") as fh:
            for r in lines:
                fh.write(json.dumps(r) + "\n")


if __name__ == "__main__":
    main()
