"""Grid-refinement transfers (vs_fine_to_coarse / vs_coarse_to_fine) and the block stepper
(solver.Refined) against the golden vectors of vivsim/multigrid.py.

The transfers copy populations and take one 4-term average in the reference's order, so
they must match bit for bit.  The two-level channel goes through the fused step (its own
rounding of the collision), so it is held to the composed-recipe tolerance: float32 2e-5,
float64 1e-11 (norm-relative).
"""

import numpy as np
import pytest
import torch

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu
TOL_RECIPE = {"f32": 2e-5, "f64": 1e-11}
DIRS = ("left", "right", "up", "down")


@pytest.fixture(scope="module")
def mg():
    import vivsim_gb300
    vivsim_gb300.build()
    from vivsim_gb300 import multigrid
    return multigrid


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_transfers_bit_exact(mg, mode):
    G = golden(mode)
    for d in DIRS:
        ff, fc = _t(G[f"mg.{d}.ff"]), _t(G[f"mg.{d}.fc"])
        ff0, fc0 = ff.clone(), fc.clone()
        got = mg.fine_to_coarse(ff, fc, d).cpu().numpy()
        assert np.array_equal(got, G[f"mg.{d}.f2c"]), d
        got = mg.coarse_to_fine(fc, ff, d).cpu().numpy()
        assert np.array_equal(got, G[f"mg.{d}.c2f"]), d
        assert torch.equal(ff, ff0) and torch.equal(fc, fc0), "arguments must stay untouched"
    got = mg.coarse_to_fine(_t(G["mg.bc.fc"]), _t(G["mg.bc.ff"]), "right").cpu().numpy()
    assert np.array_equal(got, G["mg.bc.c2f"])


def test_transfer_errors_and_host_helpers(mg, mode):
    G = golden(mode)
    ff, fc = _t(G["mg.left.ff"]), _t(G["mg.left.fc"])
    assert mg.fine_to_coarse(ff, fc, "sideways") is fc  # the reference ignores an unknown dir
    with pytest.raises(ValueError):
        mg.fine_to_coarse(ff, fc[:, :, :5].contiguous(), "left")  # 12 fine nodes onto 5 coarse
    with pytest.raises(ValueError):
        mg.coarse_to_fine(fc[:, :, :4].contiguous(), ff, "left")
    om = [mg.get_omega(nu, lv) for nu in (0.004, 0.02, 0.1) for lv in (-2, -1, 0, 1, 2, 3)]
    assert np.array_equal(np.array(om), G["mg.omega"])
    shapes = [tuple(mg.init_grid(w, h, lv, bx, by)[0].shape[1:]) for w, h, lv, bx, by in
              ((16, 8, 0, 1, 0), (16, 8, 1, 0, 0), (16, 8, -1, 0, 2), (10, 6, 2, 1, 1))]
    assert np.array_equal(np.array(shapes), G["mg.init"])


@pytest.mark.parametrize("graph", [False, True])
def test_refined_channel_matches_reference(mg, mode, graph):
    from vivsim_gb300 import solver as S
    G = golden(mode)
    dt = torch.float64 if mode == "f64" else torch.float32
    om_c, om_f, u0 = (float(x) for x in G["rc.omega"])
    coarse = S.LatticeStep(9, (17, 16), "bgk", om_c, dtype=dt,
                           boundaries=[S.boundary("equilibrium", "left", ux_wall=u0)])
    fine = S.LatticeStep(9, (16, 32), "bgk", om_f, dtype=dt,
                         boundaries=[S.boundary("nee", "right", mode="pressure", rho_wall=1.0)])
    blocks = [S.Simulation(coarse, _t(G["rc.fc0"])), S.Simulation(fine, _t(G["rc.ff0"]))]
    R = S.Refined(blocks, levels=[0, 1], links=[(0, 1, "right")])
    R.run(1)
    assert rel_err(R.f(0).cpu().numpy(), G["rc.fc1"]) <= TOL_RECIPE[mode]
    assert rel_err(R.f(1).cpu().numpy(), G["rc.ff1"]) <= TOL_RECIPE[mode]
    R.run(5, graph=graph)
    torch.cuda.synchronize()
    assert rel_err(R.f(0).cpu().numpy(), G["rc.fc6"]) <= TOL_RECIPE[mode]
    assert rel_err(R.f(1).cpu().numpy(), G["rc.ff6"]) <= TOL_RECIPE[mode]
    coarse.check()
    fine.check()
