"""vs_ib_spread_noalloc (fixed device scratch, no allocation) against vs_ib_spread.

Collected last so that it also runs after the other GPU tests have loaded the library and
used the workspace entry points.  Two calls in a row on one stream: the second reuses the
scratch the first left behind, so stale scratch would show up as a mismatch.
"""

import ctypes as C

import numpy as np
import pytest
import torch

from oracle import ib as oib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def V():
    import vivsim_gb300
    vivsim_gb300.build()
    from vivsim_gb300 import _lib
    return _lib


def _stencil(m, nx, ny, seed, dtype):
    rng = np.random.default_rng(seed)
    th = 2 * np.pi * np.arange(m) / m + rng.uniform(0, 0.1)
    r = 0.3 * min(nx, ny) * (1 + 0.05 * rng.standard_normal(m))
    x = (0.5 * nx + r * np.cos(th)).astype(dtype)
    y = (0.5 * ny + r * np.sin(th)).astype(dtype)
    W, I = oib.get_ib_stencil(x, y, ny, oib.kernel_peskin_4pt, 2)
    return np.ascontiguousarray(W, dtype), np.ascontiguousarray(I, np.int32)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_noalloc_matches_workspace_spread(V, dtype):
    nx, ny, m, c = 96, 80, 200, 2
    W, I = _stencil(m, nx, ny, 11, dtype)
    s = W.shape[1]
    dev = torch.device("cuda")
    Wd, Id = torch.from_numpy(W).to(dev), torch.from_numpy(I).to(dev)
    code = V.dtype_code(Wd)
    rng = np.random.default_rng(12)
    stream = V.stream()
    ws = torch.empty(V.lib().vs_ib_workspace_bytes(m, s), dtype=torch.uint8, device=dev)
    for call in range(2):
        vals = torch.from_numpy(rng.standard_normal((m, c)).astype(dtype)).to(dev)
        grid = torch.from_numpy(rng.standard_normal((c, nx * ny)).astype(dtype)).to(dev)
        ref = torch.empty_like(grid)
        out = torch.empty_like(grid)
        V.call("vs_ib_spread", code, V.ptr(vals), V.ptr(grid), V.ptr(ref), c, nx * ny, V.ptr(Wd), V.ptr(Id), m, s,
               V.ptr(ws), ws.numel(), stream)
        V.call("vs_ib_spread_noalloc", code, V.ptr(vals), V.ptr(grid), V.ptr(out), c, nx * ny, V.ptr(Wd),
               V.ptr(Id), m, s, stream)
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        tol = 1e-6 if dtype == np.float32 else 1e-14
        err = np.max(np.abs(a - b)) / np.max(np.abs(b))
        assert err <= tol, f"call {call}: rel err {err:.3e}"
        # same pairs, same summation order: the two entry points agree bit for bit
        assert np.array_equal(a, b), f"call {call}: results differ"


def test_noalloc_rejects_oversize(V):
    dev = torch.device("cuda")
    m, s, c, n_grid = 4097, 16, 1, 1 << 16
    vals = torch.zeros((m, c), device=dev)
    grid = torch.zeros((c, n_grid), device=dev)
    W = torch.zeros((m, s), device=dev)
    I = torch.zeros((m, s), dtype=torch.int32, device=dev)
    rc = V.lib().vs_ib_spread_noalloc(V.VS_F32, V.ptr(vals), V.ptr(grid), V.ptr(grid), c, n_grid, V.ptr(W),
                                      V.ptr(I), m, s, V.stream())
    assert rc == 1  # VS_ERR_INVALID_ARG
    assert b"fixed scratch limit" in V.lib().vs_last_error()
