"""Splitting CRM columns over ranks (one process per GPU).

In per-column mode every CRM column is independent of the others, so a batch
of GCM columns is partitioned into contiguous blocks, one per rank, with no
exchange between ranks while the CRMs run; the only collectives are the
barrier and the max-over-ranks of the timings (and, for checking, a gather of
results).  The reference runs the CRMs of one MPI task's chunks serially
(crm_physics.F90:1145-1156); its columns are distributed by the GCM's own
physics decomposition, which this mirrors.
"""
import numpy as np


def column_shard(ncols, rank, world):
    """(first, count) of the contiguous block of `ncols` columns owned by
    `rank` out of `world`; the first ncols % world ranks get one extra."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError('rank %d outside world %d' % (rank, world))
    base, extra = divmod(int(ncols), int(world))
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def shard_bounds(ncols, world):
    """All ranks' (first, count) pairs."""
    return [column_shard(ncols, r, world) for r in range(world)]


def gather_columns(local, ncols, world, all_gather):
    """Reassemble a (count, ...) array per rank into the (ncols, ...) whole.

    `all_gather(tensor_list, tensor)` is torch.distributed.all_gather (or a
    stand-in); shards are padded to the largest block so every rank sends the
    same shape."""
    import torch
    bounds = shard_bounds(ncols, world)
    width = max(c for _, c in bounds)
    pad = np.zeros((width,) + local.shape[1:], dtype=local.dtype)
    pad[:local.shape[0]] = local
    t = torch.from_numpy(pad)
    parts = [torch.empty_like(t) for _ in range(world)]
    all_gather(parts, t)
    out = np.empty((ncols,) + local.shape[1:], dtype=local.dtype)
    for (first, count), p in zip(bounds, parts):
        out[first:first + count] = p.numpy()[:count]
    return out
