"""``torch.ops.vivsim.*``: registration and shapes on CPU (fake tensors), values on the GPU."""

import numpy as np
import pytest
import torch
from torch._subclasses.fake_tensor import FakeTensorMode

import vivsim_gb300.torch_ops  # noqa: F401  (registers the operators)
from conftest import golden, rel_err


def test_registered_with_fake_shapes():
    with FakeTensorMode():
        f = torch.empty(9, 16, 8)
        assert torch.ops.vivsim.streaming(f).shape == f.shape
        rho, u = torch.ops.vivsim.get_macroscopic(f)
        assert rho.shape == (16, 8) and u.shape == (2, 16, 8)
        assert torch.ops.vivsim.get_equilibrium(rho, u).shape == f.shape
        assert torch.ops.vivsim.collision_kbc(f, f, 1.7).shape == f.shape
        f3 = torch.empty(19, 8, 8, 8)
        r3, u3 = torch.ops.vivsim.get_macroscopic(f3)
        assert u3.shape == (3, 8, 8, 8)
        W, I = torch.empty(5, 16), torch.empty(5, 16, dtype=torch.int32)
        assert torch.ops.vivsim.interpolate(u, W, I).shape == (5, 2)
        g, h = torch.ops.vivsim.multi_direct_forcing(u, W, I, torch.empty(5, 2), 1.0, 3)
        assert g.shape == u.shape and h.shape == (5, 2)
        fc = torch.empty(9, 9, 4)
        assert torch.ops.vivsim.fine_to_coarse(f, fc, "left").shape == fc.shape
        assert torch.ops.vivsim.coarse_to_fine(fc, f, "right").shape == f.shape


@pytest.mark.gpu
def test_values_match_the_shims(mode):
    import vivsim_gb300
    vivsim_gb300.build()
    from vivsim_gb300 import lbm
    G = golden(mode)
    f = torch.from_numpy(np.ascontiguousarray(G["d2.f"])).cuda()
    rho, u = torch.ops.vivsim.get_macroscopic(f)
    feq = torch.ops.vivsim.get_equilibrium(rho, u)
    assert rel_err(torch.ops.vivsim.collision_kbc(f, feq, 1.7).cpu().numpy(),
                   lbm.collision_kbc(f, feq, 1.7).cpu().numpy()) == 0.0
    assert rel_err(torch.ops.vivsim.streaming(f).cpu().numpy(), G["d2.streaming"]) <= 1e-12
    ff, fc = (torch.from_numpy(np.ascontiguousarray(G[k])).cuda() for k in ("mg.left.ff", "mg.left.fc"))
    assert np.array_equal(torch.ops.vivsim.fine_to_coarse(ff, fc, "left").cpu().numpy(), G["mg.left.f2c"])
    assert np.array_equal(torch.ops.vivsim.coarse_to_fine(fc, ff, "left").cpu().numpy(), G["mg.left.c2f"])
