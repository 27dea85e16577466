"""The N > 1 path of bench.py on CPU: world-size-2 gloo ranks (replicas, no data exchange).

Each rank times its own replica; the job's time is the maximum over ranks and the
whole-job rate counts every rank's units (weak scaling).  This exercises the same
functions the torchrun launch uses, with the gloo backend instead of NCCL.
"""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_info() == (world, rank, rank)
        secs = bench.job_seconds(torch, dist, 1.0 + 0.5 * rank, "cpu")
        out[rank] = (secs, bench.aggregate_rate(1_000_000, world, secs))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_take_the_max_time():
    world = 2
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    # both ranks see the slowest rank's time; the rate counts both replicas
    for r in range(world):
        assert res[r][0] == 1.5
        assert abs(res[r][1] - 2 * 1_000_000 / 1.5 / 1e6) < 1e-12


def test_single_rank_is_unchanged():
    assert bench.job_seconds(torch, None, 2.0, "cpu") == 2.0
    assert bench.aggregate_rate(4_000_000, 1, 2.0) == 2.0
