"""Several GPUs: scene-parallel sharding and the timing reductions of bench.py.

A single scene does not shard without a halo exchange before every neighbour pass;
batches of independent scenes partition by scene with no data-path collective. Each rank
steps its own scenes on its own GPU; the ranks exchange only timings (max over ranks)
and counts. These helpers take the torch.distributed process group as initialised by
the caller (NCCL on GPUs, gloo on CPU in the tests).
"""
from __future__ import annotations


def shard_scenes(counts, world: int) -> list:
    """Partition scene indices over `world` ranks, balanced by particle count: scenes in
    descending count (ties by index) each go to the rank with the fewest particles so far
    (ties by rank). Deterministic; every scene lands on exactly one rank; each rank's
    scenes are listed in ascending index."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(counts)), key=lambda k: (-int(counts[k]), k)):
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += int(counts[i])
    return [sorted(p) for p in parts]


def _device():
    import torch
    import torch.distributed as dist

    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def max_over_ranks(x: float, world: int) -> float:
    """The largest of every rank's `x` (timings: the job takes as long as its slowest rank)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
