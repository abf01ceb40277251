"""Multi-GPU use of the feature path: images are independent, so ranks are
replicas that each extract a contiguous shard of the image list; the rows are
gathered afterwards (no collective inside the data path).  The reference's own
equivalent is several wndchrm processes sharing one dataset through locked
.sig files (src/wndchrm_src/WORMfile.h) or a multiprocessing pool
(wndcharm/utils.py:406-440)."""
import numpy as np


def shard(n, rank, world):
    """Contiguous, balanced [lo, hi) of n items for `rank` of `world`."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def extract_sharded(images, extract_fn, group=None):
    """Every rank extracts its shard with extract_fn(list_of_images) -> (k, F)
    rows; returns the full (n, F) matrix on every rank, in input order."""
    import torch.distributed as dist
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    lo, hi = shard(len(images), rank, world)
    rows = np.asarray(extract_fn(images[lo:hi])) if hi > lo else None
    if world == 1:
        return rows
    parts = [None] * world
    dist.all_gather_object(parts, (lo, rows), group=group)
    F = next(p[1].shape[1] for p in parts if p[1] is not None)
    out = np.zeros((len(images), F))
    for lo_r, r in parts:
        if r is not None:
            out[lo_r: lo_r + len(r)] = r
    return out


def max_over_ranks(seconds, group=None):
    """The slowest rank's time: a step ends when every replica has finished."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        return seconds
    t = torch.tensor([float(seconds)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
