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
