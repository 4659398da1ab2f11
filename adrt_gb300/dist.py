"""Batch sharding across ranks (replicas; no collective on the data path).

Images are independent, so a batch is split into contiguous per-rank shards,
each rank transforms its shard, and results are only gathered when the caller
wants them on one rank.  ``shard_bounds`` is the split rule; ``gather_shards``
collects per-rank results (any backend: gloo on CPU, NCCL on GPUs);
``max_over_ranks`` is the timing reduction the benchmark uses.
"""

from __future__ import annotations

import torch
import torch.distributed as dist

__all__ = ["shard_bounds", "shard", "gather_shards", "max_over_ranks"]


def shard_bounds(batch: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [lo, hi) of `batch` items for `rank`; sizes differ by at most one."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(batch, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard(x: torch.Tensor, rank: int, world: int) -> torch.Tensor:
    lo, hi = shard_bounds(x.shape[0], rank, world)
    return x[lo:hi]


def gather_shards(local: torch.Tensor, batch: int, group=None) -> torch.Tensor:
    """All ranks receive the full (batch, ...) result assembled from the shards."""
    world = dist.get_world_size(group)
    sizes = [shard_bounds(batch, r, world) for r in range(world)]
    maxn = max(hi - lo for lo, hi in sizes)
    pad = torch.zeros((maxn, *local.shape[1:]), dtype=local.dtype, device=local.device)
    pad[: local.shape[0]] = local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([p[: hi - lo] for p, (lo, hi) in zip(parts, sizes)])


def max_over_ranks(value: float, device=None, group=None) -> float:
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
