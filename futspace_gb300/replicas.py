"""Multi-GPU form of the renderer: replicas, no data-path collective.

Views are independent (each frame depends only on its camera and the shared
maps), so N GPUs each hold a copy of the maps and render their own views. Two
ways to split work:

* weak scaling: every rank renders a full batch of its own (per-GPU work fixed);
* strong scaling: one global view list is split into contiguous rank shards.

The only cross-rank step is the report: pixels are summed and the slowest
rank's time is the job's time. That reduction runs after the timed region on
the host side of torch.distributed (gloo or nccl); the frames never move.
"""
from __future__ import annotations

from typing import Sequence, TypeVar

T = TypeVar("T")


def shard(items: Sequence[T], rank: int, world: int) -> list[T]:
    """Contiguous shard `rank` of `world` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    n = len(items)
    lo = (n * rank) // world
    hi = (n * (rank + 1)) // world
    return list(items[lo:hi])


def aggregate(pixels: int, ms: float, dist=None, device=None) -> dict:
    """Whole-job rate: total pixels over all ranks / slowest rank's time."""
    total, worst = float(pixels), float(ms)
    world = 1
    if dist is not None and dist.is_initialized():
        import torch

        t = torch.tensor([float(pixels), float(ms)], dtype=torch.float64, device=device)
        p = t[:1].clone()
        m = t[1:].clone()
        dist.all_reduce(p, op=dist.ReduceOp.SUM)
        dist.all_reduce(m, op=dist.ReduceOp.MAX)
        total, worst = float(p.item()), float(m.item())
        world = dist.get_world_size()
    return {"pixels": total, "ms": worst, "gpix_s": total / worst / 1e6 if worst > 0 else 0.0,
            "world": world}
