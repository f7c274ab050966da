"""CPU tests of the multi-rank path: the batch shards into disjoint,
balanced pieces, and a world-size-2 gloo run reproduces the bench's
max-over-ranks timing reduction and the sum of solved instances."""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from odil_gb300.batch import shard_instances


def test_shards_partition_and_balance():
    rng = np.random.default_rng(0)
    sides = rng.integers(64, 513, 512)
    costs = [int(n) * int(n) for n in sides]
    for world in (1, 2, 3, 4, 8):
        parts = [shard_instances(costs, r, world) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(512))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= min(loads) + max(costs)
    with pytest.raises(ValueError):
        shard_instances(costs, 2, 2)
    # more ranks than instances: the extra ranks own nothing
    parts = [shard_instances([5, 9, 7], r, 8) for r in range(8)]
    assert sorted(i for p in parts for i in p) == [0, 1, 2]
    assert sum(1 for p in parts if not p) == 5


def _worker(rank, world, port, costs, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard_instances(costs, rank, world)
    # Stand-in for a rank's timed solve: time proportional to its load.
    t = torch.tensor([float(sum(costs[i] for i in mine))])
    n = torch.tensor([float(len(mine))])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    dist.barrier()
    q.put((rank, t.item(), n.item(), mine))
    dist.destroy_process_group()


def test_gloo_world2_sharded_batch():
    costs = [int(c) for c in np.random.default_rng(1).integers(10, 100, 37)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, costs, q))
             for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert res[0][1] == res[1][1]  # same max time on every rank
    assert res[0][2] == res[1][2] == 37.0
    assert sorted(res[0][3] + res[1][3]) == list(range(37))


def _failing_worker(rank, world, port, q):
    """Rank 1 fails on the host before the step's collective; rank 0 must
    learn of it through an error of its collective (short process-group
    timeout), not hang."""
    import datetime
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=10))
    if rank == 1:
        q.put((rank, "raised"))
        raise SystemExit(3)
    t = torch.ones(1)
    try:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        q.put((rank, "completed"))
    except Exception as e:  # the peer is gone
        q.put((rank, "error: " + type(e).__name__))


def test_gloo_rank_failure_is_reported():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 30500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_failing_worker, args=(r, 2, port, q))
             for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert res[1] == "raised" and procs[1].exitcode == 3
    assert res[0].startswith("error"), res[0]
