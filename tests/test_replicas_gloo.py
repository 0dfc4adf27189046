"""The N > 1 host logic of bench.py (replicas: barrier, max-over-ranks timing,
whole-job aggregation) on two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    elapsed = [2.0, 3.0][rank]  # rank 1 is the slow one
    bench.barrier(world)
    slowest = bench.max_over_ranks(elapsed, world, device="cpu")
    value = bench.aggregate(world, 5, 1e12, slowest)
    out.put((rank, slowest, value))
    dist.destroy_process_group()


def test_two_rank_replicas_aggregate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [3.0, 3.0]
    # 2 replicas x 5 steps x 1e12 relaxations in the slowest rank's 3 s
    assert res[0][2] == pytest.approx(2 * 5 * 1e12 / 3.0)
