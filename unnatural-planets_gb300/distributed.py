"""Sharding chunk work over ranks (one process per GPU).

The path shards without a data-path collective: every chunk is independent
(a 1-cell halo is part of its grid), so a rank contours its own chunks with
up_batch_run. The one exchange is host-side: the per-chunk vertex and index
counts, all-gathered so that every rank knows where its vertices and indices
land in the concatenated mesh (an exclusive prefix sum in global chunk order).
The reference fans the same chunk work out over CPU tasks
(sources/generator.cpp:159,215).
"""
from __future__ import annotations

import numpy as np


def shard_chunks(chunks, rank: int, world: int) -> list[int]:
    """Indices of the chunks rank `rank` of `world` processes.

    Greedy balance by sample count: chunks in decreasing size go to the
    least-loaded rank (ties to the lower rank), so every rank computes the
    same assignment without communication. Returned in ascending order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    sizes = [int(g.count) for _, g in chunks]
    order = sorted(range(len(chunks)), key=lambda c: (-sizes[c], c))
    load = [0] * world
    owner = [0] * len(chunks)
    for c in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[c] = r
        load[r] += sizes[c]
    return [c for c in range(len(chunks)) if owner[c] == rank]


def global_offsets(mine: list[int], vertex_counts, index_counts, n_chunks: int, group=None):
    """All-gather the per-chunk counts of this rank's chunks `mine` and return
    (vertex_offset, index_offset) arrays over all n_chunks + 1 in global chunk
    order (offset[c] = sum of counts of chunks before c; offset[n] = totals).
    Every rank gets the same arrays. Uses torch.distributed (any backend; the
    counts travel as one int64 tensor per rank)."""
    import torch
    import torch.distributed as dist

    local = torch.zeros((n_chunks, 2), dtype=torch.int64)
    for c, v, i in zip(mine, vertex_counts, index_counts):
        local[c, 0] = int(v)
        local[c, 1] = int(i)
    if dist.is_available() and dist.is_initialized():
        t = local.cuda() if dist.get_backend(group) == "nccl" else local
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)  # each chunk is owned by exactly one rank
        local = t.cpu()
    counts = local.numpy()
    vo = np.zeros(n_chunks + 1, np.int64)
    io = np.zeros(n_chunks + 1, np.int64)
    vo[1:] = np.cumsum(counts[:, 0])
    io[1:] = np.cumsum(counts[:, 1])
    return vo, io
