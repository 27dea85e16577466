"""Error of the float32 fused step against float64 over whole runs of the benchmark cases.

    python -m vivsim_gb300.accuracy [--cases cavity viv2d sphere3d adjoint sweep] [--out FILE]

Each case runs its full step count in float32 and in float64 (the float64 fused step
matches the float64 oracle to ~1e-12 per step) from the same float32 initial state, and
the norm-relative differences max|a - b| / max|b| of rho and u (and of the body
displacement) are printed as one JSON line per case.  ``adjoint`` is the differentiable
cylinder (512 x 256, 4000 steps): the objective and its gradients in float32 against
float64.  ``sweep`` is the 64-case VIV sweep advanced as one batch: the largest rho and u
error over the cases.
"""

import argparse
import json

import torch

from . import configs

FULL_STEPS = {"cavity": 1000, "viv2d": 20000, "sphere3d": 5000, "adjoint": 4000, "sweep": 2000}


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


def compare_adjoint(steps):
    from .adjoint import CylinderDrag
    res = {}
    for dt in (torch.float32, torch.float64):
        plan = CylinderDrag(n_steps=steps, dtype=dt)
        J = plan.forward(keep_checkpoints=True)
        gU0, gK, goff = plan.backward()
        plan.close()
        res[dt] = (J, gU0, gK, goff)
    (J32, u32, k32, o32), (J64, u64, k64, o64) = res[torch.float32], res[torch.float64]
    return {"case": "adjoint cylinder D2Q9 BGK 512 x 256, 64 markers", "steps": steps,
            "J_rel_err": abs(J32 - J64) / abs(J64), "dU0_rel_err": abs(u32 - u64) / abs(u64),
            "dK_rel_err": abs(k32 - k64) / abs(k64),
            "doffsets_rel_err": float(abs(o32 - o64).max() / abs(o64).max()),
            "values_f32": {"J": float(J32), "dU0": float(u32), "dK": float(k32)},
            "values_f64": {"J": float(J64), "dU0": float(u64), "dK": float(k64)}}


def compare_sweep(steps, n_cases=64):
    from . import solver
    out = {}
    for dt in (torch.float32, torch.float64):
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            sims = [configs.build_solver(c, dtype=dt)[2] for c in configs.viv_sweep(n_cases)]
            batch = solver.Batch(sims)
            batch.run(steps)
            torch.cuda.synchronize()
        out[dt] = [s.f.clone() for s in sims]
        batch.close()
    er = eu = 0.0
    for a, b in zip(out[torch.float32], out[torch.float64]):
        ra, ua = rho_u(a)
        rb, ub = rho_u(b)
        er, eu = max(er, rel(ra, rb)), max(eu, rel(ua, ub))
    return {"case": f"VIV sweep, {n_cases} cases batched", "steps": steps, "rho_rel_err": er, "u_rel_err": eu}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cases", nargs="*", default=list(FULL_STEPS))
    ap.add_argument("--steps", type=int, default=None, help="override the full step count")
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    lines = []
    for name in a.cases:
        steps = a.steps or FULL_STEPS[name]
        if name == "adjoint":
            res = compare_adjoint(steps)
        elif name == "sweep":
            res = compare_sweep(steps)
        else:
            res = compare(name, steps)
        print(json.dumps(res), flush=True)
        lines.append(res)
    if a.out:
        with open(a.out, "w") as fh:
            for r in lines:
                fh.write(json.dumps(r) + "\n")


if __name__ == "__main__":
    main()
