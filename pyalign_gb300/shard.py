"""One bag of pairs over several GPUs: every rank of a torch.distributed group solves a share
of the pairs on its own GPU and the results are put back in bag order.

Pairs are independent (each lane's result depends only on its own sequences and lengths,
pyalign/solve.py:536-562 solves them batch by batch in any grouping), so the bag splits
with no exchange during the solve: `shard_pairs` deals the pairs out by their cell counts
(largest first, each to the rank with the fewest cells so far -- every rank computes the
same split from the lengths alone, no communication), `gather_results` collects each
rank's scores and maps into bag order with one all-gather of host arrays at the end.
"""

import numpy as np


def shard_pairs(len_s, len_t, world, rank):
    """Indices (ascending) of the pairs rank `rank` of `world` solves: the pairs sorted by
    cells |s| * |t|, largest first (ties by index), each given to the rank with the fewest
    cells so far (the lowest rank on a tie).  Every pair goes to exactly one rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    ls = np.asarray(len_s, dtype=np.int64)
    lt = np.asarray(len_t, dtype=np.int64)
    if ls.shape != lt.shape or ls.ndim != 1:
        raise ValueError("len_s and len_t must be 1-d arrays of one length")
    cells = np.maximum(ls, 0) * np.maximum(lt, 0)
    order = np.lexsort((np.arange(len(cells)), -cells))
    load = np.zeros(world, dtype=np.int64)
    owner = np.empty(len(cells), dtype=np.int64)
    for k in order:
        r = int(np.argmin(load))
        owner[k] = r
        load[r] += cells[k]
    return np.flatnonzero(owner == rank)


def gather_results(index, scores, maps, map_sizes, n, group=None):
    """Results of every rank in bag order, on every rank: `index` = this rank's pair indices
    (shard_pairs), `scores` its scores in that order, `maps` its alignment maps concatenated
    in that order with `map_sizes` entries each.  Returns (scores (n,), maps concatenated in
    bag order, map offsets (n,))."""
    import torch.distributed as dist

    index = np.asarray(index, dtype=np.int64)
    part = (index, np.asarray(scores), np.asarray(maps), np.asarray(map_sizes, dtype=np.int64))
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, part, group=group)
    # element types from the ranks that solved pairs (a rank with none may pass empty lists)
    dt_s = [p[1].dtype for p in parts if p[1].size] or [part[1].dtype]
    dt_m = [p[2].dtype for p in parts if p[2].size] or [part[2].dtype]
    all_scores = np.zeros(n, dtype=np.result_type(*dt_s))
    sizes = np.zeros(n, dtype=np.int64)
    for idx, _, _, ms in parts:
        sizes[idx] = ms
    offs = np.zeros(n, dtype=np.int64)
    if n > 1:
        np.cumsum(sizes[:-1], out=offs[1:])
    all_maps = np.zeros(int(sizes.sum()), dtype=np.result_type(*dt_m))
    seen = np.zeros(n, dtype=bool)
    for idx, sc, mp, ms in parts:
        if seen[idx].any():
            raise ValueError("a pair was solved by two ranks")
        seen[idx] = True
        all_scores[idx] = sc
        src = np.zeros(len(idx) + 1, dtype=np.int64)
        np.cumsum(ms, out=src[1:])
        for k, i in enumerate(idx):
            all_maps[offs[i]:offs[i] + ms[k]] = mp[src[k]:src[k + 1]]
    if not seen.all():
        raise ValueError(f"{int((~seen).sum())} pairs were solved by no rank")
    return all_scores, all_maps, offs
