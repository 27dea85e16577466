"""The bounds-checked build (nvcc -DVIVSIM_BOUNDS_CHECK) on small cases of every grid path.

The checked library tests every gather and scatter index of the grid kernels against its
array and reports VS_ERR_RANGE through the plan's status word instead of touching memory
outside it.  Each case runs in a child process that loads the checked library
(VIVSIM_GB300_LIBRARY), must report no range error, and must give the default library's
populations (1e-6 norm-relative: the checks change no arithmetic, only the code around it).
"""

import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from conftest import ROOT, rel_err

pytestmark = pytest.mark.gpu

CHILD = r"""
import sys, numpy as np, torch
sys.path.insert(0, {root!r})
from vivsim_gb300 import configs
out = {{}}
cases = dict(
    viv=configs.viv2d(nx=256, ny=256, D=24.0, center=(64.0, 128.0), n_markers=75),
    sphere=configs.sphere3d(nx=48, ny=32, nz=32, D=8.0, center=(16.0, 16.0, 16.0), n_markers=200),
    periodic=configs.periodic2d(n=512),
    cavity=configs.cavity(n=64),
)
stream = torch.cuda.Stream()
with torch.cuda.stream(stream):
    for name, case in cases.items():
        step, body, sim = configs.build_solver(case)
        sim.run(3)
        sim.run(6, graph=True)
        torch.cuda.synchronize()
        step.check()
        out[name] = sim.f.cpu().numpy()
np.savez({path!r}, **out)
"""


def run_child(path, library=None):
    env = dict(os.environ)
    if library:
        env["VIVSIM_GB300_LIBRARY"] = library
    code = CHILD.format(root=ROOT, path=path)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    return dict(np.load(path))


def test_bounds_checked_build_matches_default(tmp_path):
    import vivsim_gb300
    from vivsim_gb300 import _build
    vivsim_gb300.build()
    checked = _build.build(checked=True)
    assert torch.cuda.is_available()
    ref = run_child(str(tmp_path / "default.npz"))
    chk = run_child(str(tmp_path / "checked.npz"), checked)
    for name in ref:
        assert rel_err(chk[name], ref[name]) <= 1e-6, name
