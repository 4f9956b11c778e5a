"""The benchmark's multi-rank logic on CPU (two gloo ranks on 127.0.0.1):
every rank recovers its own signals (distinct seeds, no collective on the
data path), the job's time is the slowest rank's, and the job's rate counts
every rank's signals. bench.py runs the same functions over NCCL on GPUs."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 + 50.0 * rank          # the ranks' own times differ
        job_ms = bench.max_over_ranks(ms, dist, "cpu")
        seeds = bench.rank_seeds(rank, 4)
        gathered = [None] * world
        dist.all_gather_object(gathered, seeds)
        out.put((rank, job_ms, gathered))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_distinct_signals():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    results = sorted(q.get() for _ in range(world))
    for rank, job_ms, gathered in results:
        assert job_ms == 150.0                      # max over ranks, on every rank
        assert not set(gathered[0]) & set(gathered[1])  # replicas: own signals
    # 2 ranks x 4 signals x 3 steps in the slowest rank's 150 ms
    assert bench.job_rate(2, 4, 3, 150.0) == pytest.approx(160.0)


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.rank_seeds(0, 3) == [10_000, 10_001, 10_002]
