import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        have_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        have_gpu = False
    if have_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


_GOLDEN = {}


def golden(mode):
    """Golden vectors produced by the reference's own functions (see tests/golden/make_golden.py)."""
    if mode not in _GOLDEN:
        _GOLDEN[mode] = dict(np.load(os.path.join(GOLDEN_DIR, f"golden_{mode}.npz")))
    return _GOLDEN[mode]


def rel_err(a, b):
    """Norm-relative error max|a - b| / max|b| (the parity metric used in every test)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    den = np.max(np.abs(b)) if b.size else 0.0
    if den == 0.0:
        return float(np.max(np.abs(a))) if a.size else 0.0
    return float(np.max(np.abs(a - b)) / den)


@pytest.fixture(params=["f32", "f64"])
def mode(request):
    return request.param
