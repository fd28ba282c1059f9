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


def max_over_ranks(value: float, group=None, device=None) -> float:
    """Maximum of a per-rank scalar (the benchmark's timed region)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
