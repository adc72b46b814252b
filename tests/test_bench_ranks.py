"""The benchmark's multi-rank bookkeeping on two CPU processes (gloo,
127.0.0.1): every rank runs its own replica of the workload, the reported
time of each leg is the slowest rank's (all-reduce MAX, no other data moves
between ranks), and the whole-job rate counts one mesh per rank per step."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took (100 + 10 r) ms for BF16, (400 - r) for FP32, 130 + r for e2e
        got = bench.max_over_ranks([100 + 10 * rank, 400 - rank, 130 + rank], "cpu", world)
        out[rank] = (got, bench.job_rate(got[0], world))
    finally:
        dist.destroy_process_group()


def test_two_ranks_report_the_slowest_rank():
    world = 2
    out = mp.Manager().dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    for rank in range(world):
        times, rate = out[rank]
        assert times == [110.0, 400.0, 131.0]
        assert rate == pytest.approx(2 * 1000.0 / 110.0)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks([1.5, 2.5], "cpu", 1) == [1.5, 2.5]
    assert bench.job_rate(125.0, 1) == 8.0
