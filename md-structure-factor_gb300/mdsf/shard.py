"""Frame sharding across ranks (one process per GPU).

Frames are independent and ``sf`` is an additive FP64 sum (dens.py:318), so
N ranks each take a contiguous slice of the trajectory, accumulate their own
``sf`` with no exchange on the data path, and one SUM all-reduce of the FP64
accumulator (n0*n1*(n2/2+1)*8 bytes) combines them at the end.
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def shard_range(n_frames, rank, world):
    """Contiguous [start, stop) of the frames owned by `rank` (sizes differ by at most 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(int(n_frames), world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def reduce_sf(sf, group=None):
    """Sum the per-rank FP64 accumulators in place (no-op without a process group)."""
    if sf.dtype != torch.float64:
        raise TypeError("sf must be float64")
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(sf, op=dist.ReduceOp.SUM, group=group)
    return sf


def structure_factor_sharded(positions, box, weights, grid_dims, rank=None, world=None, **kw):
    """Each rank runs :func:`mdsf.structure_factor` on its frames, then one all-reduce."""
    from .api import structure_factor
    if rank is None:
        rank = dist.get_rank() if dist.is_initialized() else 0
    if world is None:
        world = dist.get_world_size() if dist.is_initialized() else 1
    a, b = shard_range(positions.shape[0], rank, world)
    bx = box[a:b] if getattr(box, "ndim", 1) == 2 else box
    sf = structure_factor(positions[a:b], bx, weights, grid_dims, **kw)
    return reduce_sf(sf)
