"""Multi-rank helpers (one process per GPU).

The render path shards in two ways:

* additive frames (a_eq_e=true) by particles: each rank renders a contiguous
  share of the particle array into a full image and the pre-exp images are
  summed -- the reference's composite_images (splotch/splotchutils.cc:217-224,
  an MPI_Allreduce over the image) with the same shares as calcShareGeneral
  (cxxsupport/share_utils.h:41-49);
* batches of frames by frame: frames are independent, rank r renders frames
  r, r+world, ... with no data-path collective.

Ordered (a_eq_e=false) frames are not particle-sharded: compositing is not a
sum, so each rank renders whole frames.
"""
from __future__ import annotations

import numpy as np


def share(n: int, rank: int, world: int) -> tuple[int, int]:
    """[lo, hi) of rank's share of n items, calcShareGeneral's split."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_frames(nframes: int, rank: int, world: int) -> list[int]:
    """Frames rendered by this rank (round robin)."""
    return list(range(rank, nframes, world))


def composite_additive(pic, group=None):
    """Sum the ranks' additive images in place (torch tensor), like the
    reference's image allreduce."""
    import torch.distributed as dist

    dist.all_reduce(pic, op=dist.ReduceOp.SUM, group=group)
    return pic


def gather_frames(images: dict[int, np.ndarray], nframes: int, rank: int, world: int,
                  shape: tuple, group=None) -> list[np.ndarray] | None:
    """Collect every rank's frames on rank 0 (None elsewhere)."""
    import torch
    import torch.distributed as dist

    out = [None] * nframes
    if rank == 0:
        for f, img in images.items():
            out[f] = img
        for src in range(1, world):
            for f in shard_frames(nframes, src, world):
                t = torch.empty(shape, dtype=torch.float32)
                dist.recv(t, src=src, group=group)
                out[f] = t.numpy()
        return out
    for f in shard_frames(nframes, rank, world):
        dist.send(torch.from_numpy(np.ascontiguousarray(images[f])), dst=0, group=group)
    return None
