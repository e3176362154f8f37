"""Row-sharded kNN over several GPUs (one process per GPU).

knn_rms / knn_data rows (fit frames) are independent: every rank holds the
whole reference set and computes a contiguous block of fit rows, with no
collective on the data path. The blocks are gathered to rank 0 in row order
afterwards, so rank 0 ends with exactly what one process would compute
(the reference's row order, knn_rms.cpp:213-293). The eigensolve and the
serving model are not sharded: each process keeps a full replica.

The process group may be NCCL or gloo; the gather goes through
torch.distributed's object collectives (host memory).
"""
from __future__ import annotations

import numpy as np


def row_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous block of rows [r0, r1) of rank `rank`; the first n % world
    ranks get one row more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n, world)
    r0 = rank * base + min(rank, extra)
    return r0, r0 + base + (1 if rank < extra else 0)


def _gather_rows(parts, group=None):
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    out = [None] * world if rank == 0 else None
    dist.gather_object(parts, out, dst=0, group=group)
    if rank != 0:
        return None
    return tuple(np.concatenate([o[j] for o in out]) for j in range(len(parts)))


def knn_sharded(compute, ref, fit, k, group=None, **kw):
    """Row-sharded kNN. compute(ref, fit_block, k, **kw) -> (distances,
    indices) of the block, e.g. Context.knn_rms bound with masses, or
    Context.knn_data. fit None = fit is ref (the reference's default:
    each row's nearest, itself, is dropped the same way in every block,
    because the block is passed as a separate fit set of the same frames).
    Returns the full (distances, indices) on rank 0, None elsewhere."""
    import torch.distributed as dist

    rows = ref if fit is None else fit
    r0, r1 = row_range(len(rows), dist.get_rank(group), dist.get_world_size(group))
    d, i = compute(ref, rows[r0:r1], k, **kw)
    return _gather_rows((np.asarray(d), np.asarray(i)), group)
