"""Sharding independent systems over GPUs (one process per GPU): longest-processing-time-first
assignment by estimated cost, no collective on the data path -- every rank solves its own systems
and only the timings are reduced (max over ranks)."""
import heapq

import numpy as np


def lpt_partition(costs, nranks):
    """Greedy LPT: systems in decreasing cost (ties by index) each go to the least-loaded rank
    (ties by rank).  Returns per rank the sorted system indices."""
    costs = np.asarray(costs, dtype=np.float64)
    order = sorted(range(len(costs)), key=lambda s: (-costs[s], s))
    heap = [(0.0, r) for r in range(nranks)]
    parts = [[] for _ in range(nranks)]
    for s in order:
        load, r = heapq.heappop(heap)
        parts[r].append(s)
        heapq.heappush(heap, (load + float(costs[s]), r))
    return [sorted(p) for p in parts]


def system_costs(nnz, rhs):
    """The cost model: one pass over the matrix per right-hand side (nnz x rhs)."""
    return np.asarray(nnz, dtype=np.float64) * np.asarray(rhs, dtype=np.float64)


def subset_arena(mix, systems):
    """Host arena (n, rhs, row_ptr, col, val, b, xstar) of the listed systems of a gen.Mix, in order."""
    n = mix.n[systems].astype(np.int32)
    rhs = mix.rhs[systems].astype(np.int32)
    rp = np.concatenate([mix.row_ptr[mix.rp_off[s]:mix.rp_off[s + 1]] for s in systems]).astype(np.int64)
    col = np.concatenate([mix.col[mix.nz_off[s]:mix.nz_off[s + 1]] for s in systems])
    val = np.concatenate([mix.val[mix.nz_off[s]:mix.nz_off[s + 1]] for s in systems])
    b = np.concatenate([mix.b[mix.xb_off[s]:mix.xb_off[s + 1]] for s in systems])
    xs = np.concatenate([mix.xstar[mix.xb_off[s]:mix.xb_off[s + 1]] for s in systems])
    return n, rhs, rp, col, val, b, xs
