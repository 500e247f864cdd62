"""Replicas-only multi-GPU execution: cells are independent, so ranks take disjoint
contiguous shards of the batch and never exchange data while stepping.  The only
collectives are host-side bookkeeping after a run (max of per-rank times, gather of
per-cell results), done with ``torch.distributed`` (NCCL on GPUs, gloo on CPU)."""

from __future__ import annotations

import numpy as np

__all__ = ["shard_range", "balanced_shards", "reduce_max", "gather_objects"]


def shard_range(n_items: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous ``[lo, hi)`` share of ``n_items`` for ``rank`` of ``world``."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError(f"bad rank/world {rank}/{world}")
    base, extra = divmod(int(n_items), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def balanced_shards(weights, world: int) -> list[np.ndarray]:
    """Split item indices into ``world`` groups of near-equal total weight (greedy LPT)."""
    w = np.asarray(weights, dtype=np.float64)
    order = np.argsort(-w, kind="stable")
    loads = np.zeros(world)
    groups: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = int(np.argmin(loads))
        groups[r].append(int(i))
        loads[r] += w[i]
    return [np.sort(np.asarray(g, dtype=np.int64)) for g in groups]


def reduce_max(value: float) -> float:
    """Max of ``value`` over ranks (identity when not distributed)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_objects(obj) -> list:
    """All ranks' ``obj`` in rank order (``[obj]`` when not distributed)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return [obj]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out
