"""Multi-GPU = independent replicas (no data-path collective).

The solver path has no exchange step between systems: a stream of requests
(or an atlas of charts) is split across GPUs by request, each rank runs its
own server on its own GPU, and the only cross-rank operations are a barrier
before and after the timed region and a max-reduction of the timings (the
job is as slow as its slowest rank).  ``torch.distributed`` is plumbing here.
"""
from __future__ import annotations


def max_over_ranks(values, dist=None, device="cpu"):
    """Element-wise max of a list of floats over all ranks (identity when
    dist is None or the world has one rank)."""
    vals = [float(v) for v in values]
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return vals
    import torch
    t = torch.tensor(vals, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def shard(items, rank: int, world: int):
    """Requests of this rank: round-robin by index (deterministic)."""
    return [it for i, it in enumerate(items) if i % world == rank]
