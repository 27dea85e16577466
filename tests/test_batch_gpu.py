"""Batched cases (vs_batch_run) against each case run on its own (vs_run).

The batch runs the same per-node and per-body code as the single-case step, only with
the launches of all cases merged, so the populations and body states must agree bit for
bit, over several calls, with and without graph replay.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import vivsim_gb300
    vivsim_gb300.build()
    from vivsim_gb300 import solver
    return solver


def _cases():
    from vivsim_gb300 import configs
    cases = configs.viv_sweep(n_cases=4, seed=7, heights=(64, 128))
    # a body in the general form (markers in random order), and a case without a body
    shuffled = configs.viv2d(nx=128, ny=64, D=64 / 12.0, center=(32.0, 32.0), n_markers=17 * 3, seed=9)
    perm = np.random.default_rng(1).permutation(shuffled["body"]["markers"].shape[0])
    shuffled["body"]["markers"] = shuffled["body"]["markers"][perm]
    cases.append(shuffled)
    cases.append(configs.periodic2d(n=64))
    return cases


def _build(S, cases):
    from vivsim_gb300 import configs
    return [configs.build_solver(c)[2] for c in cases]


def _state(sims):
    out = []
    for s in sims:
        st = s.body.state() if s.body is not None else None
        out.append((s.f.cpu().numpy(), st))
    return out


@pytest.mark.parametrize("tb,spg", [(128, 4), (64, 0), (256, 6)])
def test_batch_equals_single_runs(S, tb, spg):
    cases = _cases()
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        ref = _build(S, cases)
        for sim in ref:
            sim.run(23)
        bat = _build(S, cases)
        batch = S.Batch(bat, threads_per_block=tb, steps_per_graph=spg)
        batch.run(10)
        batch.run(13)
        torch.cuda.synchronize()
    for k, ((fa, sa), (fb, sb)) in enumerate(zip(_state(ref), _state(bat))):
        assert np.array_equal(fa, fb), f"case {k}: populations differ"
        if sa is not None:
            for key in ("a", "v", "d", "h"):
                assert np.array_equal(sa[key], sb[key]), f"case {k}: body {key} differs"
    for sim in ref + bat:
        sim.step.check()


def test_batch_rejects_mixed_collisions(S):
    from vivsim_gb300 import configs
    a = configs.build_solver(configs.periodic2d(n=64))[2]
    b = configs.build_solver(configs.periodic2d(n=64, collision="bgk"))[2]
    with pytest.raises(RuntimeError, match="differs"):
        S.Batch([a, b])


def test_batch_and_single_runs_interleave(S):
    """Odd-length batch runs, single-case runs of the same simulations in between (the body
    kernels hand the window prediction over in alternating slots), then the batch again."""
    cases = _cases()
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        ref = _build(S, cases)
        for sim in ref:
            sim.run(35)
        bat = _build(S, cases)
        batch = S.Batch(bat, threads_per_block=128, steps_per_graph=4)
        batch.run(9)
        batch.run(13)
        for sim in bat:
            sim.run(5)
        batch.run(1)
        batch.run(7)
        torch.cuda.synchronize()
    for k, ((fa, sa), (fb, sb)) in enumerate(zip(_state(ref), _state(bat))):
        assert np.array_equal(fa, fb), f"case {k}: populations differ"
        if sa is not None:
            for key in ("a", "v", "d", "h"):
                assert np.array_equal(sa[key], sb[key]), f"case {k}: body {key} differs"
    for sim in ref + bat:
        sim.step.check()
