"""Multi-rank (replica) bookkeeping on CPU: world size 2 over gloo, as bench.py
runs it under torchrun (one replica per rank, maximum of the timed region over
ranks, aggregate throughput over the slowest rank)."""

from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from jaxdem_gb300 import replicas  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        # rank r "took" 10 + 5 r ms for its replica of N * K units
        t = replicas.max_over_ranks(dist, 10.0 + 5.0 * rank)
        units = [1000 * 50] * world
        value = replicas.aggregate_throughput(units, t * 1e-3)
        mine = list(replicas.shard(4096, rank, world))
        q.put((rank, t, value, mine[0], len(mine)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_timing_and_shard():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's time and the same aggregate
    assert [g[1] for g in got] == [15.0, 15.0]
    assert got[0][2] == got[1][2] == pytest.approx(2 * 1000 * 50 / 15e-3)
    # the two shards tile the 4096 systems without overlap
    assert got[0][3] == 0 and got[1][3] == got[0][4] and got[0][4] + got[1][4] == 4096


def test_shard_partitions_evenly():
    for n in (0, 1, 7, 4096, 12_000_001):
        for world in (1, 2, 3, 8):
            parts = [replicas.shard(n, r, world) for r in range(world)]
            assert sum(len(p) for p in parts) == n
            assert all(parts[r].stop == parts[r + 1].start for r in range(world - 1))
            assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)


def test_replica_workloads_are_independent_draws():
    """bench.py seeds each rank's replica differently, with the same size and box."""
    import bench

    a, b = bench.make_workload("c1", 512, 0), bench.make_workload("c1", 512, 1)
    assert a.N == b.N and (a.box_size == b.box_size).all()
    assert not (a.pos == b.pos).all()
