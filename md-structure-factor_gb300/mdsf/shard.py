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


def shard_inputs(n_frames, box, rank, world):
    """(start, stop, scale, L) of `rank`'s frames.

    With per-frame boxes (T, 3) the reference rescales every frame to the
    mean box of the WHOLE trajectory and bins in that box (dens.py:50-58), so
    the factors avg/box_t and the mean box are computed over all T frames
    first and each rank takes its rows of the factors: every rank then builds
    the same grid and bins exactly as one process would.  ``scale`` is None
    for a single (3,) box."""
    from .api import frame_scale
    a, b = shard_range(n_frames, rank, world)
    scale, L = frame_scale(box)
    if scale is not None and scale.shape[0] != n_frames:
        raise ValueError("per-frame boxes must have one row per frame")
    return a, b, (None if scale is None else scale[a:b]), L


def structure_factor_sharded(positions, box, weights, grid_dims, rank=None, world=None, **kw):
    """Each rank runs :func:`mdsf.structure_factor` on its frames, then one all-reduce."""
    from .api import structure_factor
    if rank is None:
        rank = dist.get_rank() if dist.is_initialized() else 0
    if world is None:
        world = dist.get_world_size() if dist.is_initialized() else 1
    a, b, scale, L = shard_inputs(positions.shape[0], box, rank, world)
    sf = structure_factor(positions[a:b], L, weights, grid_dims, scale=scale, **kw)
    return reduce_sf(sf)
