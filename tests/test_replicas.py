"""bench.py --gpus N runs N independent replicas (the step does not shard: one world per
GPU, no exchange) and reports the job's throughput from its slowest rank.  The rank
combination is host logic: checked here with two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, queue) -> None:
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        env = bench.dist_env()
        got = bench.max_over_ranks([1.0 + rank, 5.0 - 2.0 * rank, 0.25], world)
        queue.put((rank, env, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict()
    for _ in procs:
        rank, env, got = queue.get(timeout=120)
        results[rank] = (env, got)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in range(2):
        env, got = results[rank]
        assert env == (rank, 2, rank)
        assert got == [2.0, 5.0, 0.25]  # element-wise max over the ranks, on every rank


def test_max_over_ranks_one_rank_is_identity():
    import bench

    assert bench.max_over_ranks([3.0, 1.5], 1) == [3.0, 1.5]
