"""Batches of clouds across ranks (one GPU per rank).

A single cloud's EMST does not shard: every Boruvka round needs a global
union-find.  A batch does: its clouds are independent.  Each rank takes a
contiguous range of the cloud list, balanced by cumulative point count,
solves it with one emst_solve_batch call on its own GPU, and the per-cloud
edge lists and lengths are gathered to rank 0 -- the only exchange, a host
gather, no collective on the data path.
"""
import numpy as np


def partition(sizes, world):
    """Contiguous ranges [start, stop) of the cloud list, one per rank, with
    about equal point counts (cut where the cumulative count crosses k/world)."""
    sizes = np.asarray(sizes, np.int64)
    if world < 1:
        raise ValueError("world must be >= 1")
    cum = np.concatenate([[0], np.cumsum(sizes)])
    total = int(cum[-1])
    cuts = [0]
    for k in range(1, world):
        cuts.append(int(np.searchsorted(cum, total * k / world, side="left")))
    cuts.append(len(sizes))
    cuts = np.maximum.accumulate(np.minimum(cuts, len(sizes)))
    return [(int(cuts[r]), int(cuts[r + 1])) for r in range(world)]


def solve_sharded(clouds, rank, world, solve, dist=None):
    """Solve this rank's share with `solve(list of clouds) -> (edge lists,
    lengths)` and gather every cloud's result to rank 0.  Returns the full
    (edge lists, lengths) on rank 0 and this rank's share elsewhere."""
    start, stop = partition([len(c) for c in clouds], world)[rank]
    mine = clouds[start:stop]
    uvs, lens = solve(mine) if mine else ([], np.zeros(0))
    part = (start, [np.asarray(u) for u in uvs], np.asarray(lens, np.float64))
    if dist is None or world == 1:
        return part[1], part[2]
    parts = [None] * world if rank == 0 else None
    dist.gather_object(part, parts, dst=0)
    if rank != 0:
        return part[1], part[2]
    out_uv, out_len = [None] * len(clouds), np.zeros(len(clouds))
    for s, u, ln in parts:
        for i, (ui, li) in enumerate(zip(u, ln)):
            out_uv[s + i] = ui
            out_len[s + i] = li
    return out_uv, out_len
