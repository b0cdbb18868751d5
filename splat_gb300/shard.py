"""Sharding one frame's rays over ranks.

Rays are independent and the scene is read-only, so a frame shards into
contiguous ray ranges of the light grid, one per rank (every rank holds the
whole scene).  The only exchange is the elementwise sum of the ranks' light
maps; with int32 fixed-point accumulation that sum is exact and independent
of the order, so a sharded frame equals the single-GPU frame bit for bit.
The benchmark itself runs replicas (one frame per rank, no exchange); this
module is the path for a frame larger than one GPU's time budget.
"""
from __future__ import annotations

from typing import List, Tuple


def ray_ranges(n_rays: int, world: int) -> List[Tuple[int, int]]:
    """Balanced contiguous ranges [begin, end) covering 0..n_rays."""
    if world < 1:
        raise ValueError("world must be >= 1")
    base, extra = divmod(n_rays, world)
    out, lo = [], 0
    for r in range(world):
        hi = lo + base + (1 if r < extra else 0)
        out.append((lo, hi))
        lo = hi
    return out


def trace_shard(wl, rank: int, world: int, scene=None):
    """This rank's part of the frame: its ray range traced on its GPU.
    Returns the partial light map tensor (planes, h, w)."""
    from . import tracer

    lo, hi = ray_ranges(wl.n_rays, world)[rank]
    if hi <= lo:
        return tracer.new_light_map(wl.map_w, wl.map_h, wl.n_planes, wl.accum)
    return tracer.trace_forward(wl, scene=scene, ray_begin=lo, ray_end=hi).tex


def reduce_maps(tex, group=None):
    """Sum the ranks' partial light maps in place (all_reduce SUM)."""
    import torch.distributed as dist

    dist.all_reduce(tex, op=dist.ReduceOp.SUM, group=group)
    return tex
