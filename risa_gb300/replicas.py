"""Multi-GPU by replicas.

Slices are independent, so the reconstruction shards with no exchange step:
one process per GPU, each reconstructing its own frames, and no collective on
the data path. The reference hands frames to devices round robin
(H2D.cu:92-93); here the unit of distribution is a group of n_planes
consecutive frames (one frame of every plane), so every rank's frames stay
plane-interleaved and can go through the engine with PLANES_INTERLEAVED.

The collectives below are host-side bookkeeping only (collecting images for
writing, the slowest rank's time); they run on any torch.distributed backend,
gloo included.
"""
from __future__ import annotations

import numpy as np


def shard_indices(n_frames: int, rank: int, world: int, n_planes: int = 1) -> np.ndarray:
    """Frame indices of `rank`: groups of n_planes frames dealt round robin."""
    if world < 1 or not 0 <= rank < world or n_planes < 1:
        raise ValueError("bad rank / world / n_planes")
    if n_frames % n_planes:
        raise ValueError("n_frames must be a multiple of n_planes")
    groups = np.arange(n_frames // n_planes)
    mine = groups[groups % world == rank]
    return (mine[:, None] * n_planes + np.arange(n_planes)[None, :]).reshape(-1)


def reassemble(parts, n_frames: int, world: int, n_planes: int = 1) -> np.ndarray:
    """Images of all ranks (parts[r] in rank r's frame order) back in frame order."""
    first = next(p for p in parts if len(p))
    out = np.empty((n_frames,) + tuple(first.shape[1:]), dtype=first.dtype)
    for r, p in enumerate(parts):
        idx = shard_indices(n_frames, r, world, n_planes)
        if len(idx) != len(p):
            raise ValueError(f"rank {r} holds {len(p)} images, expected {len(idx)}")
        out[idx] = p
    return out


def gather_images(local: np.ndarray, n_frames: int, n_planes: int = 1, dst: int = 0):
    """Collects every rank's images on rank `dst` (host memory) in frame order;
    returns them there and None elsewhere."""
    import torch.distributed as dist

    world, rank = dist.get_world_size(), dist.get_rank()
    parts = [None] * world if rank == dst else None
    dist.gather_object(np.ascontiguousarray(local), parts, dst=dst)
    return reassemble(parts, n_frames, world, n_planes) if rank == dst else None


def run_sharded(n_frames: int, n_planes: int, reconstruct, dst: int = 0):
    """One rank's part of a job split over the ranks (strong scaling): this
    rank's frame indices (shard_indices), reconstructed by
    `reconstruct(indices) -> images` -- the engine on this rank's GPU, or any
    other worker -- then every rank's images collected on rank `dst` in frame
    order. Returns the images there and None elsewhere."""
    import torch.distributed as dist

    idx = shard_indices(n_frames, dist.get_rank(), dist.get_world_size(), n_planes)
    return gather_images(np.asarray(reconstruct(idx)), n_frames, n_planes, dst)


def max_over_ranks(value: float) -> float:
    """The largest value over all ranks (e.g. the slowest rank's step time)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
