"""Multi-GPU layout of the render path: replicas only.

Pixels and frames are independent (no exchange step), so N processes, one per
GPU, each hold a full replica of the sky, blackbody table and gas grid and
render a disjoint share of the frames (or row bands); the host gathers the
results.  The only collective is the timing reduction of the benchmark.
"""
from __future__ import annotations


def shard(n_units: int, rank: int, world: int) -> range:
    """Contiguous block of [0, n_units) owned by `rank` of `world`; the blocks
    partition the range and differ in size by at most one."""
    if world <= 0 or not 0 <= rank < world or n_units < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(n_units, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(values, device=None):
    """All-reduce MAX of a list of floats over the default process group
    (gloo or NCCL); identity when torch.distributed is not initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]
