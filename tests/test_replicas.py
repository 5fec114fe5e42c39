"""Multi-rank host logic (replicas and ensemble sharding) with gloo, world size 2, on CPU."""
import os
import socket

import pytest

import replicas as R


def test_shard_runs_covers_every_run_once_and_balances():
    weights = [64 * 64 * 16, 512 * 512 * 256, 128 * 128 * 32, 256 * 256 * 64, 64 * 64 * 256,
               512 * 512 * 16, 128 * 128 * 128, 256 * 256 * 16]
    for world in (1, 2, 3, 8):
        shards = R.shard_runs(weights, world)
        assert len(shards) == world
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(weights)))
        loads = [sum(weights[i] for i in s) for s in shards]
        # greedy largest-first: no rank exceeds the ideal share by more than the largest run
        assert max(loads) <= sum(weights) / world + max(weights)
    assert R.shard_runs([], 2) == [[], []]
    with pytest.raises(ValueError):
        R.shard_runs([1], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank timed its own replica; the job's time is the slowest rank's
        ms = [12.5, 20.0][rank]
        ms_max = R.max_over_ranks(ms, dist)
        units = R.sum_over_ranks(1000.0 * (rank + 1), dist)
        weights = [5, 9, 2, 7, 7, 1]
        mine = R.shard_runs(weights, world)[rank]
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        dist.barrier()
        q.put((rank, ms_max, units, R.whole_job_rate(units, ms_max / 1000.0), gathered))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_max_time_and_shards():
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
    for rank, ms_max, units, rate, gathered in out:
        assert ms_max == 20.0          # MAX, not the rank's own time
        assert units == 3000.0
        assert rate == pytest.approx(3000.0 / 0.020)
        flat = sorted(i for s in gathered for i in s)
        assert flat == list(range(6))  # the ranks' shards partition the runs
