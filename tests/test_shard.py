"""Sharding the batched mix over ranks: the LPT partition (host logic) and the replica protocol of
bench.py (gloo, world size 2, on CPU: every rank takes its shard, times are reduced by max)."""
import os
import socket
import sys

import numpy as np
import pytest

from sptrsv_gb300 import gen
from sptrsv_gb300.shard import lpt_partition, subset_arena, system_costs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_lpt_partition_properties():
    rng = np.random.default_rng(0)
    costs = np.exp(rng.uniform(0, 8, 300))
    for k in (1, 2, 3, 8):
        parts = lpt_partition(costs, k)
        flat = sorted(s for p in parts for s in p)
        assert flat == list(range(len(costs)))
        loads = [costs[p].sum() for p in parts]
        # LPT bound: max load <= 4/3 of the optimum, and the optimum >= max(mean load, largest item)
        lower = max(costs.sum() / k, costs.max())
        assert max(loads) <= 4.0 / 3.0 * lower + 1e-9
    assert lpt_partition([5.0, 5.0], 2) == [[0], [1]]


def test_subset_arena_matches_systems():
    M = gen.mix(count=10, seed=4, nmin=200, nmax=3000, rhs_max=4)
    part = lpt_partition(system_costs(M.nnz, M.rhs), 3)[1]
    n, rhs, rp, col, val, b, xs = subset_arena(M, part)
    off = 0
    for k, s in enumerate(part):
        m, xs_s, b_s = M.system(s)
        assert n[k] == m.n and rhs[k] == M.rhs[s]
        assert np.array_equal(rp[off:off + m.n + 1], m.row_ptr)
        off += m.n + 1
    assert len(col) == sum(int(M.nnz[s]) for s in part) and len(b) == len(xs) == sum(int(M.n[s] * M.rhs[s]) for s in part)
    M.close()


def _worker(rank, ws, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    M = gen.mix(count=12, seed=4, nmin=200, nmax=3000, rhs_max=4)
    parts = lpt_partition(system_costs(M.nnz, M.rhs), d.ws)
    mine = parts[d.rank]
    d.barrier()
    t = float(len(mine)) + 0.5 * d.rank  # a stand-in per-rank time
    out.put((d.rank, mine, d.max(t)))
    d.close()
    M.close()


def test_replicas_over_gloo_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, t0), (r1, m1, t1) = res
    assert sorted(m0 + m1) == list(range(12)) and not set(m0) & set(m1)
    expect = max(len(m0), len(m1) + 0.5)
    assert t0 == t1 == expect
