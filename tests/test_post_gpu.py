"""Flow diagnostics (vs_post) against the golden vectors of vivsim/post.py.

Tolerance (norm-relative): float32 2e-6, float64 1e-12; means 1e-6 / 1e-12 (the kernel
sums in double, the reference in the working precision).
"""

import numpy as np
import pytest
import torch

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu
TOL = {"f32": 2e-6, "f64": 1e-12}
FIELDS = ("velocity_magnitude", "velocity_gradient", "vorticity", "vorticity_magnitude", "divergence",
          "strain_rate", "strain_rate_magnitude", "kinetic_energy", "mean_kinetic_energy", "enstrophy",
          "mean_enstrophy", "q_criterion")


@pytest.fixture(scope="module")
def post():
    import vivsim_gb300
    vivsim_gb300.build()
    from vivsim_gb300 import post
    return post


def test_fields_match_reference(post, mode):
    G = golden(mode)
    for tag in ("p2", "p3"):
        u = torch.from_numpy(np.ascontiguousarray(G[f"{tag}.u"])).cuda()
        for name in FIELDS:
            got = getattr(post, name)(u)
            ref = G[f"{tag}.{name}"]
            assert tuple(got.shape) == ref.shape, (tag, name, got.shape, ref.shape)
            tol = (1e-6 if mode == "f32" else 1e-12) if name.startswith("mean") else TOL[mode]
            err = rel_err(got.cpu().numpy(), ref)
            assert err <= tol, f"{tag}.{name}: {err:.3e}"
    rho = torch.from_numpy(np.ascontiguousarray(G["p.rho"])).cuda()
    assert rel_err(post.pressure(rho).cpu().numpy(), G["p.pressure"]) <= TOL[mode]


def test_from_populations_equals_two_passes(post, mode):
    import vivsim_gb300
    from vivsim_gb300 import lbm, lbm3d
    G = golden(mode)
    f2 = torch.from_numpy(np.ascontiguousarray(G["d2.f"])).cuda()
    _, u2 = lbm.get_macroscopic(f2)
    assert torch.equal(post.vorticity_from_populations(f2), post.vorticity(u2))
    assert torch.equal(post.q_criterion_from_populations(f2), post.q_criterion(u2))
    f3 = torch.from_numpy(np.ascontiguousarray(G["d3.f"])).cuda()
    _, u3 = lbm3d.get_macroscopic(f3)
    assert torch.equal(post.vorticity_from_populations(f3), post.vorticity(u3))
