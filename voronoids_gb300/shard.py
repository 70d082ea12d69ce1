"""Independent point sets across GPUs (one process per GPU).

A single triangulation does not shard (rounds are globally dependent); the
sets of a batched build or a serving stream do.  ``lpt_assign`` gives each
rank a share of the sets by the longest-processing-time rule (largest set
first, to the least-loaded rank; cost = points), and ``batch_distributed``
builds the local share with a batched build and gathers the edge lists on
rank 0.  The only collective is that final host gather.
"""
import heapq

import numpy as np


def lpt_assign(sizes, world):
    """Set indices per rank, balancing the summed sizes (LPT)."""
    sizes = np.asarray(sizes, dtype=np.int64)
    order = np.argsort(-sizes, kind="stable")
    heap = [(0, r) for r in range(world)]
    heapq.heapify(heap)
    parts = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(int(i))
        heapq.heappush(heap, (load + int(sizes[i]), r))
    return [sorted(p) for p in parts]


def batch_distributed(point_sets, seed=0, build=None, group=None):
    """Triangulate ``point_sets`` across the ranks of the default process group.

    Every rank passes the same list; each builds its LPT share (``build``,
    default :func:`voronoids_gb300.delaunay_batch`) and rank 0 returns all
    edge arrays in input order (other ranks return None)."""
    import torch.distributed as dist
    if build is None:
        from .tree import delaunay_batch as build
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    share = lpt_assign([len(p) for p in point_sets], world)[rank]
    local = build([point_sets[i] for i in share], seed=seed) if share else []
    got = [None] * world if rank == 0 else None
    dist.gather_object(list(zip(share, local)), got, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * len(point_sets)
    for part in got:
        for i, e in part:
            out[i] = e
    return out
