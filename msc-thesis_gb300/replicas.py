"""Work split and timing across ranks, one process per GPU.

A single run does not shard (its deposit and field solve are global), so
several GPUs run independent replicas; an ensemble shards by run.  Neither
exchanges data: the only collectives are a barrier around the timed region
and a MAX of the ranks' times, so that whole-job throughput is
units of all ranks / slowest rank's time.  Works with any torch.distributed
backend (NCCL between GPUs; gloo in the CPU tests).
"""
from __future__ import annotations

import heapq


def shard_runs(weights, world):
    """Split runs over `world` ranks, balancing the summed weight (particle
    counts): largest run first to the least-loaded rank.  Returns one sorted
    list of run indices per rank; every run appears exactly once."""
    if world < 1:
        raise ValueError("world must be >= 1")
    heap = [(0, r) for r in range(world)]
    shards = [[] for _ in range(world)]
    for i in sorted(range(len(weights)), key=lambda k: (-weights[k], k)):
        load, r = heapq.heappop(heap)
        shards[r].append(i)
        heapq.heappush(heap, (load + weights[i], r))
    return [sorted(s) for s in shards]


def max_over_ranks(value, dist=None, device=None):
    """MAX of a float over all ranks (the value itself without a process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, dist=None, device=None):
    """SUM of a float over all ranks."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(units_all_ranks, seconds_max):
    """Throughput of the whole job: every rank's units over the slowest time."""
    return units_all_ranks / seconds_max
