"""Order of operations of solver.Refined (host logic, no GPU): the recursive sub-cycling
of vivsim/multigrid.py's block layouts, recorded through stand-ins for the kernels."""

from types import SimpleNamespace

import pytest

from vivsim_gb300 import solver as S


def _layout(levels, links):
    blocks = [SimpleNamespace(step=SimpleNamespace(q=9), body=None, f=f"f{i}") for i in range(len(levels))]
    R = S.Refined(blocks, levels, links)
    log = []
    R._step = lambda i: log.append(("step", i))
    R.f = lambda i: i
    R._mg = SimpleNamespace(transfer_=lambda kind, src, dst, d: log.append((kind, src, dst, d)))
    return R, log


def test_two_levels_match_the_channel_recipe():
    R, log = _layout([0, 1], [(0, 1, "right")])
    R.run(1)
    assert log == [("step", 0), ("step", 1), ("coarse_to_fine", 0, 1, "right"), ("step", 1),
                   ("coarse_to_fine", 0, 1, "right"), ("fine_to_coarse", 1, 0, "left")]


def test_three_levels_subcycle_recursively():
    R, log = _layout([0, 1, 2, 1], [(0, 1, "up"), (1, 2, "left"), (0, 3, "down")])
    R.run(1)
    steps = [e[1] for e in log if e[0] == "step"]
    assert steps.count(0) == 1 and steps.count(1) == 2 and steps.count(3) == 2 and steps.count(2) == 4
    # level-2 block: two steps, each followed by its transfer from block 1, then back into block 1
    i = log.index(("step", 1))
    assert log[i:i + 4] == [("step", 1), ("step", 3), ("coarse_to_fine", 0, 1, "up"), ("coarse_to_fine", 0, 3, "down")]
    assert log[i + 4:i + 9] == [("step", 2), ("coarse_to_fine", 1, 2, "left"), ("step", 2),
                                ("coarse_to_fine", 1, 2, "left"), ("fine_to_coarse", 2, 1, "right")]
    assert log[-2:] == [("fine_to_coarse", 1, 0, "down"), ("fine_to_coarse", 3, 0, "up")]


def test_links_must_join_neighbouring_levels():
    blocks = [SimpleNamespace(step=SimpleNamespace(q=9), body=None) for _ in range(2)]
    with pytest.raises(ValueError):
        S.Refined(blocks, [0, 2], [(0, 1, "right")])
    with pytest.raises(ValueError):
        S.Refined(blocks, [0, 1], [(0, 1, "north")])


def test_subcycling_counts_for_random_layouts():
    """Level L takes 2**(L - L_min) steps per cycle; each link's coarse_to_fine runs once per
    fine step and its fine_to_coarse once per coarse step."""
    import random
    rnd = random.Random(5)
    for _ in range(30):
        n_levels = rnd.randint(1, 4)
        levels = sorted(rnd.randint(0, n_levels - 1) for _ in range(rnd.randint(1, 6)))
        levels = [lv - levels[0] for lv in levels]
        links = []
        for f, lf in enumerate(levels):
            coarse = [c for c, lc in enumerate(levels) if lc == lf - 1]
            if coarse:
                links.append((rnd.choice(coarse), f, rnd.choice(["left", "right", "up", "down"])))
        R, log = _layout(levels, links)
        R.run(2)
        for i, lv in enumerate(levels):
            assert sum(1 for e in log if e == ("step", i)) == 2 * 2 ** lv
        for c, f, side in links:
            assert sum(1 for e in log if e[0] == "coarse_to_fine" and e[1:3] == (c, f)) == 2 * 2 ** levels[f]
            assert sum(1 for e in log if e[0] == "fine_to_coarse" and e[1:3] == (f, c)) == 2 * 2 ** levels[c]
