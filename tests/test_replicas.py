"""Replica/shard bookkeeping for several GPUs, as world-size-2 gloo process
groups on the CPU (the data path itself has no collective)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from lqt1_gb300 import replicas  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # throughput: work summed, time of the slowest rank
        value, ms, work = replicas.aggregate_throughput(1e9 * (rank + 1), 100.0 + 50.0 * rank)
        # a sharded batch of 10 instances with uneven work, per-instance rows gathered
        weights = np.array([5, 1, 1, 1, 1, 1, 1, 1, 1, 5], float)
        lo, hi = replicas.shard_bounds(10, rank, world, weights)
        local = np.arange(lo, hi, dtype=float)[:, None] * np.array([[1.0, 10.0]])
        rows = replicas.gather_rows(local, 10, lo)
        q.put((rank, value, ms, work, lo, hi, rows))
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregation_and_shards():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in procs])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms, work, lo, hi, rows in res:
        assert ms == 150.0 and work == 3e9
        assert value == pytest.approx(3e9 / 0.150)
        np.testing.assert_array_equal(rows, np.arange(10)[:, None] * np.array([[1.0, 10.0]]))
    (_, _, _, _, lo0, hi0, _), (_, _, _, _, lo1, hi1, _) = res
    assert lo0 == 0 and hi0 == lo1 and hi1 == 10 and 0 < hi0 < 10


def test_shard_bounds_cover_and_balance():
    w = np.random.default_rng(0).uniform(1, 10, 1000)
    for world in (1, 2, 3, 8):
        b = [replicas.shard_bounds(1000, r, world, w) for r in range(world)]
        assert b[0][0] == 0 and b[-1][1] == 1000
        assert all(b[i][1] == b[i + 1][0] for i in range(world - 1))
        loads = [w[lo:hi].sum() for lo, hi in b]
        assert max(loads) - min(loads) <= 2 * w.max()
