"""sptrsv_solve_noalloc: the solve for callers that cannot allocate device memory (their whole
GPU belongs to their own pool, or their loop cannot pay for cudaMalloc's synchronisation).

The entry point is called through the C ABI on device arrays the test owns, twice in a row with
different right-hand sides (the fixed scratch array keeps the previous call's contents, so the
second call checks that nothing stale leaks in), and each result is compared with the existing
handle-based solve of the same schedule at the parity tolerance of the other GPU tests.  This
file is collected last so that a run stopping at its first failure has run every other test."""
import ctypes

import numpy as np
import pytest

import sptrsv_gb300 as sp
from sptrsv_gb300 import _lib, gen

pytestmark = pytest.mark.gpu

ELEM_TOL = 1e-10
MAX_ROWS = 1 << 20


def _elem_err(x, ref):
    scale = max(np.max(np.abs(ref)), 1e-300)
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-12 * scale)))


def test_noalloc_matches_existing_solve_twice():
    torch = pytest.importorskip("torch")
    L = _lib.lib()
    m = gen.random_upper(150_000, 8.0, 0.9, 64, 77)
    dev = torch.device("cuda:0")
    rp = torch.tensor(m.row_ptr.astype(np.int32), device=dev)
    col = torch.tensor(m.col, device=dev)
    val = torch.tensor(m.val, device=dev)
    x = torch.empty(m.n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    with sp.Solver(0) as s:
        s.analyse(m.row_ptr, m.col, m.val)
        for seed in (101, 102):
            b_host = gen.uniform(seed, m.n)
            b = torch.tensor(b_host, device=dev)
            torch.cuda.synchronize()
            rc = L.sptrsv_solve_noalloc(m.n, m.nnz, rp.data_ptr(), col.data_ptr(), val.data_ptr(), b.data_ptr(),
                                        x.data_ptr(), None)
            assert rc == 0, sp.status_string(rc)
            ref = s.solve(b_host, schedule="syncfree_warp")
            assert _elem_err(x.cpu().numpy(), ref) <= ELEM_TOL


def test_noalloc_rejects_sizes_beyond_its_array():
    torch = pytest.importorskip("torch")
    L = _lib.lib()
    d = torch.zeros(4, dtype=torch.float64, device="cuda:0")
    i = torch.zeros(4, dtype=torch.int32, device="cuda:0")
    n = MAX_ROWS + 1
    rc = L.sptrsv_solve_noalloc(n, n, i.data_ptr(), i.data_ptr(), d.data_ptr(), d.data_ptr(), d.data_ptr(), None)
    assert rc == -11 and "maximum" in sp.status_string(rc)
