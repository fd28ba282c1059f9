"""Multi-rank host logic on CPU: world_size-2 gloo process groups (no GPU).
Instance sharding covers every instance once with balanced cost, results
gather in instance order on rank 0, and the timed region is the maximum
over ranks -- the same helpers bench.py and batch drivers use over NCCL."""
import os
import socket

import pytest

from adscf_gb300 import parallel


def test_shard_covers_every_instance_once():
    costs = [24**3 * 100, 64**3 * 200, 32**3 * 150, 48**3 * 120, 40**3 * 180] * 7
    for world in (1, 2, 3, 4, 8):
        ranges = [parallel.shard(costs, r, world) for r in range(world)]
        seen = [i for rg in ranges for i in rg]
        assert seen == list(range(len(costs)))
        if world <= len(costs):
            loads = [sum(costs[i] for i in rg) for rg in ranges]
            assert max(loads) <= sum(costs) / world + max(costs)


def test_shard_more_ranks_than_instances():
    ranges = [parallel.shard([1.0, 1.0], r, 4) for r in range(4)]
    assert sorted(i for rg in ranges for i in rg) == [0, 1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        costs = [float(10 + (i * 7) % 13) for i in range(11)]
        rg = parallel.shard(costs, rank, world)
        # a stand-in for each instance's SCF result: (index, free energy)
        local = [(i, 0.5 * i + rank * 0.0) for i in rg]
        out = parallel.gather_instances(local, rg, len(costs))
        tmax = parallel.max_over_ranks(1.0 + rank)
        q.put((rank, out, tmax))
    finally:
        dist.destroy_process_group()


def _stand_in_runner(instances, fields, n_iter, tol):
    # per-instance result computed from the instance itself (no GPU)
    return [dict(grid=k["grid"][0], total=float(sum(f.sum() for f in fl)), n_iter=n_iter)
            for k, fl in ((k, [f]) for k, f in zip(instances, fields))]


def _sharded_worker(rank, world, port, q):
    import numpy as np
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        inst = [dict(grid=(g, g, g), ds=0.01, block_length=(0.4, 0.6)) for g in (24, 64, 32, 48, 40, 64, 24)]
        fields = [np.full((2, 3), float(i)) for i in range(len(inst))]
        out = parallel.run_batch_sharded(inst, fields, 5, runner=_stand_in_runner)
        rg = parallel.shard([parallel.instance_cost(k) for k in inst], rank, world)
        q.put((rank, out, list(rg)))
    finally:
        dist.destroy_process_group()


def test_run_batch_sharded_over_two_gloo_ranks():
    """The sharded batch driver: each rank runs its own instance range
    through the runner, rank 0 gets all results in instance order."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_sharded_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {r: (out, rg) for r, out, rg in (q.get(timeout=120) for _ in procs)}
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out0, rg0 = res[0]
    out1, rg1 = res[1]
    assert out1 is None
    assert rg0 and rg1 and rg0 + rg1 == list(range(7))   # both ranks own work
    assert [o["grid"] for o in out0] == [24, 64, 32, 48, 40, 64, 24]
    assert [o["total"] for o in out0] == [6.0 * i for i in range(7)]
    assert all(o["n_iter"] == 5 for o in out0)


def test_gather_and_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    by_rank = dict((r, (out, t)) for r, out, t in res)
    out0, t0 = by_rank[0]
    assert out0 == [(i, 0.5 * i) for i in range(11)]
    assert by_rank[1][0] is None
    assert t0 == by_rank[1][1] == 2.0
