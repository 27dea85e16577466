"""Size-independent properties at the benchmark sizes, where the oracle is too slow to
compare node by node.

* Periodic D2Q9 KBC 8192^2 (the HBM-bound roofline case): with periodic walls and no
  force, every collision keeps mass and momentum, and streaming only moves them, so both
  totals stay put over a run.  The test sums 604 M float32 populations in float64.
* VIV cylinder 1024 x 512 (the headline workload): a float32 run and a float64 run of the
  same 2000 steps agree to 5e-4 of the largest population (measured 1.1e-4).  The
  float64 run's own error is about 1e-12 per step, so the difference is the float32
  rounding of the whole pipeline.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def C():
    import vivsim_gb300
    vivsim_gb300.build()
    from vivsim_gb300 import configs
    return configs


def _totals(f):
    c = torch.tensor([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]],
                     dtype=torch.float64, device=f.device)
    per_q = f.double().sum(dim=(1, 2))  # (9,)
    return float(per_q.sum()), (per_q[:, None] * c).sum(dim=0).cpu().numpy()


def test_periodic_8192_conserves_mass_and_momentum(C):
    case = C.periodic2d(n=8192)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        step, _, sim = C.build_solver(case)
        m0, p0 = _totals(sim.f)
        sim.run(20, graph=True)
        torch.cuda.synchronize()
        m1, p1 = _totals(sim.f)
    step.check()
    assert abs(m1 - m0) / m0 < 1e-6, (m0, m1)
    assert np.max(np.abs(p1 - p0)) / m0 < 1e-6, (p0, p1)


def test_viv_float32_against_float64(C):
    case = C.viv2d()
    s = torch.cuda.Stream()
    out = {}
    with torch.cuda.stream(s):
        for dt in (torch.float32, torch.float64):
            c = dict(case)
            c["f0"] = case["f0"].astype(np.float64 if dt == torch.float64 else np.float32)
            step, body, sim = C.build_solver(c, dtype=dt)
            sim.run(2000, graph=True)
            torch.cuda.synchronize()
            step.check()
            out[dt] = (sim.f.double().cpu().numpy(), body.state())
    (f32, s32), (f64, s64) = out[torch.float32], out[torch.float64]
    err = np.max(np.abs(f32 - f64)) / np.max(np.abs(f64))
    assert err < 5e-4, err  # measured 1.1e-4 (largest next to the body)
    assert np.all(np.isfinite(s32["d"])) and np.all(np.isfinite(s64["d"]))
