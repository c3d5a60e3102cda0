"""Multi-rank host logic on CPU (gloo, world size 2): the scene sharding and
the benchmark's barrier + max-over-ranks timing reduction.  No GPU."""
import os
import socket

import pytest

import shard
import workloads as W


def test_shards_cover_and_balance():
    reqs = W.batched_requests(256)
    for world in (1, 2, 4, 8):
        parts = [shard.shard_requests(reqs, world, r) for r in range(world)]
        seeds = sorted(r["seed"] for p in parts for r in p)
        assert seeds == sorted(r["seed"] for r in reqs)  # disjoint and complete
        loads = shard.shard_loads(reqs, world)
        biggest = max(shard.request_cost(r) for r in reqs)
        assert max(loads) - min(loads) <= biggest  # within one request of even
    with pytest.raises(ValueError):
        shard.shard_requests(reqs, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    reqs = W.batched_requests(64)
    mine = shard.shard_requests(reqs, world, rank)
    # each rank's "time" differs; the job's time is the slowest rank's
    t = bench.barrier_max(1.0 + rank, world)
    total = [None] * world
    dist.all_gather_object(total, sum(r["particles"] for r in mine))
    q.put((rank, t, sum(total), len(mine)))
    dist.destroy_process_group()


def test_two_rank_reduction_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    reqs = W.batched_requests(64)
    for rank, t, total, n in out:
        assert t == 2.0
        assert total == sum(r["particles"] for r in reqs)
    assert sum(n for _, _, _, n in out) == len(reqs)
