"""Several ranks on CPU (gloo, world size 2): the host side of bench.py's N > 1 path.

Each rank runs in its own process (spawned); they share no GPU. Checked: the scene
partition of the batched workload covers every scene exactly once and balances particles,
the max/sum reductions and the barrier, and the whole-job throughput formula (every rank's
particles over the slowest rank's time).
"""
from __future__ import annotations

import multiprocessing as mp
import os
import socket
import traceback

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    try:
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                          WORLD_SIZE=str(world))
        import torch.distributed as dist

        from fluid_gb300 import scenes
        from fluid_gb300.shard import barrier, max_over_ranks, shard_scenes, sum_over_ranks

        dist.init_process_group("gloo", rank=rank, world_size=world)
        counts = scenes.batched_counts()
        parts = shard_scenes(counts, world)
        mine = parts[rank]
        everyone = [None] * world
        dist.all_gather_object(everyone, mine)
        assert everyone == parts  # every rank computes the same partition
        flat = sorted(i for p in everyone for i in p)
        assert flat == list(range(len(counts)))
        loads = [sum(counts[i] for i in p) for p in everyone]
        assert max(loads) - min(loads) <= max(counts)
        # per-rank timing: the job is as slow as its slowest rank
        my_ms = 10.0 + 5.0 * rank
        assert max_over_ranks(my_ms, world) == 10.0 + 5.0 * (world - 1)
        my_particles = sum(counts[i] for i in mine)
        assert sum_over_ranks(my_particles, world) == sum(counts)
        barrier(world)
        steps = 4
        value = sum_over_ranks(my_particles, world) * steps / (max_over_ranks(my_ms, world) / 1e3)
        q.put((rank, "ok", value, loads))
        dist.destroy_process_group()
    except Exception:
        q.put((rank, traceback.format_exc(), None, None))


def test_two_ranks_partition_and_reduce():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
    for rank, status, value, loads in out:
        assert status == "ok", status
    values = {round(v, 6) for _, _, v, _ in out}
    assert len(values) == 1  # both ranks report the same whole-job number
    loads = out[0][3]
    print(f"2 ranks: particles per rank {loads}, whole-job value {values.pop():.4g}")
    assert all(p.exitcode == 0 for p in procs)


def test_partition_single_rank_and_many():
    from fluid_gb300 import scenes
    from fluid_gb300.shard import shard_scenes

    counts = scenes.batched_counts()
    assert shard_scenes(counts, 1) == [list(range(len(counts)))]
    parts = shard_scenes(counts, 8)
    assert sorted(i for p in parts for i in p) == list(range(len(counts)))
    loads = [sum(counts[i] for i in p) for p in parts]
    assert (max(loads) - min(loads)) / (sum(loads) / 8) < 0.05
    with pytest.raises(ValueError):
        shard_scenes(counts, 0)
