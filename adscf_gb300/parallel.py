"""Multi-rank helpers (one process per GPU, torch.distributed).

A single bulk instance does not shard: its 3D FFTs would need two
all-to-alls per contour step.  Multi-GPU runs are therefore either
independent replicas (the benchmark) or a batch split by instance: every
rank owns a contiguous set of instances, runs them with no data-path
collective, and the per-instance results are gathered on the host.  These
helpers hold that host logic; they work on any process group (NCCL on GPUs,
gloo on CPUs for tests).
"""
from __future__ import annotations

from typing import Sequence


def shard(costs: Sequence[float], rank: int, world: int) -> range:
    """Contiguous instance range [lo, hi) of `rank` balancing the summed cost
    (for example grid points x contour steps per instance).  Every instance
    belongs to exactly one rank; a rank may own none when world > len(costs)."""
    n = len(costs)
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world")
    total = float(sum(costs))
    bounds = [0]
    acc, k = 0.0, 0
    for r in range(1, world):
        target = total * r / world
        while k < n and acc + 0.5 * costs[k] <= target:
            acc += costs[k]
            k += 1
        bounds.append(k)
    bounds.append(n)
    return range(bounds[rank], bounds[rank + 1])


def gather_instances(local: list, rng: range, n: int, group=None) -> list | None:
    """Gather per-instance results (any picklable objects) of every rank's
    range onto rank 0, in instance order; other ranks get None."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    payload = (rng.start, rng.stop, list(local))
    parts = [None] * world if rank == 0 else None
    dist.gather_object(payload, parts, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * n
    for lo, hi, items in parts:
        if hi - lo != len(items):
            raise RuntimeError("a rank returned the wrong number of instance results")
        out[lo:hi] = items
    if any(v is None for v in out):
        raise RuntimeError("instances missing after the gather")
    return out


def instance_cost(kw) -> float:
    """Work of one batch instance: grid points x contour steps."""
    gx, gy, gz = kw.get("grid", (32, 32, 32))
    planes = gz if kw.get("geometry", 0) == 0 else gz + 1
    if kw.get("dss") is not None:
        steps = len(kw["dss"]) - 1
    else:
        f = kw.get("block_length", (0.5, 0.5))
        ds = kw.get("ds", 0.01)
        steps = round(f[0] / ds) + round(f[1] / ds)
    return float(gx * gy * planes) * float(steps)


def run_batch(instances, fields, n_iter, tol=-1.0):
    """One rank's share: a Batch (adscf_batch_*) over `instances`, n_iter SCF
    iterations; per-instance (free energy, accuracy, log Q, status, iter)."""
    from .scf import Batch
    if not instances:
        return []
    with Batch(instances) as b:
        b.set_fields(fields)
        res = b.scf_run(n_iter, tol)
    return [dict(free_energy=r.free_energy, accuracy=r.accuracy, logQ=r.logQ,
                 status=r.status, iter=r.iter) for r in res]


def run_batch_sharded(instances, fields, n_iter, tol=-1.0, runner=None, group=None):
    """Run a batch split across the ranks of `group`: rank r takes the
    contiguous, cost-balanced range shard(costs, r, world), runs it with
    `runner(instances, fields, n_iter, tol)` (default: run_batch on this
    rank's GPU) with no collective on the data path, and rank 0 receives
    every instance's result in instance order (other ranks: None)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    rg = shard([instance_cost(k) for k in instances], rank, world)
    run = runner or run_batch
    local = run([instances[i] for i in rg], [fields[i] for i in rg], n_iter, tol)
    return gather_instances(local, rg, len(instances), group=group)


def max_over_ranks(value: float, group=None, device=None) -> float:
    """Maximum of a per-rank scalar (the benchmark's timed region)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
