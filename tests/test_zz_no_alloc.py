"""sptrsv_solve_noalloc: the solve for callers that cannot allocate device memory (their whole
GPU belongs to their own pool, or their loop cannot pay for cudaMalloc's synchronisation).

The entry point is called through the C ABI on device arrays the test owns.  Two calls in a row
with different right-hand sides (the fixed scratch array keeps the previous call's contents, so
the second call checks that nothing stale leaks in) are compared with the serial CPU solve of the
oracle and with the existing handle-based solve of the same schedule, at the parity tolerance of
the other GPU tests.  Invalid matrices must return their status, and a valid call right after a
failed one must still be correct (the control block is cleared per call).  The largest accepted
size, n = SPTRSV_NOALLOC_MAX_ROWS, uses the last slot of the array.  This file is collected last
so that a run stopping at its first failure has run every other test."""
import numpy as np
import pytest

import sptrsv_gb300 as sp
from oracle import oracle as orc
from sptrsv_gb300 import _lib, gen

pytestmark = pytest.mark.gpu

ELEM_TOL = 1e-10
RES_TOL = 1e-12
MAX_ROWS = 1 << 20


def _torch():
    return pytest.importorskip("torch")


class _Dev:
    """Device copies of one CSR system (int32 row pointer), owned by the test."""

    def __init__(self, torch, row_ptr, col, val):
        dev = torch.device("cuda:0")
        self.n = len(row_ptr) - 1
        self.nnz = len(col)
        self.rp = torch.tensor(np.asarray(row_ptr, dtype=np.int32), device=dev)
        self.col = torch.tensor(np.asarray(col, dtype=np.int32), device=dev)
        self.val = torch.tensor(np.asarray(val, dtype=np.float64), device=dev)
        self.x = torch.empty(self.n, dtype=torch.float64, device=dev)
        self.torch = torch

    def solve(self, b_host):
        b = self.torch.tensor(np.asarray(b_host, dtype=np.float64), device="cuda:0")
        self.torch.cuda.synchronize()
        rc = _lib.lib().sptrsv_solve_noalloc(self.n, self.nnz, self.rp.data_ptr(), self.col.data_ptr(),
                                             self.val.data_ptr(), b.data_ptr(), self.x.data_ptr(), None)
        return rc, self.x.cpu().numpy()


def _check(m, b, x):
    rpu = np.asarray(m.row_ptr, dtype=np.uint64)
    ref = orc.base_gauss_upper(rpu, m.col, m.val, b, 1)
    err = orc.max_elem_rel_error(ref, x, 1e-12)
    res = orc.rel_residual(rpu, m.col, m.val, x, b, 1)
    assert err <= ELEM_TOL and res <= RES_TOL, (err, res)
    return ref


def test_noalloc_matches_oracle_and_handle_twice():
    torch = _torch()
    m = gen.random_upper(150_000, 8.0, 0.9, 64, 77)
    d = _Dev(torch, m.row_ptr, m.col, m.val)
    with sp.Solver(0) as s:
        s.analyse(m.row_ptr, m.col, m.val)
        for seed in (101, 102):
            b = gen.uniform(seed, m.n)
            rc, x = d.solve(b)
            assert rc == 0, sp.status_string(rc)
            ref = _check(m, b, x)
            xh = s.solve(b, schedule="syncfree_warp")
            assert orc.max_elem_rel_error(ref, xh, 1e-12) <= ELEM_TOL
            assert orc.max_elem_rel_error(xh, x, 1e-12) <= ELEM_TOL


def _broken(kind):
    """A small valid chain system and a copy broken in one row."""
    m = gen.random_upper(5_000, 6.0, 0.9, 32, 5)
    rp = np.asarray(m.row_ptr, dtype=np.int64)
    col = np.array(m.col, dtype=np.int32)
    val = np.array(m.val, dtype=np.float64)
    r = 1234
    if kind == "missing_diag":
        assert rp[r + 1] - rp[r] >= 2
        col[rp[r]] = col[rp[r] + 1]  # the row's first entry is no longer its diagonal
        status = -5
    else:
        val[rp[r]] = 0.0
        status = -8
    return m, (rp, col, val), status


@pytest.mark.parametrize("kind", ["missing_diag", "zero_pivot"])
def test_noalloc_invalid_matrix_then_valid_call(kind):
    torch = _torch()
    m, (rp, col, val), status = _broken(kind)
    bad = _Dev(torch, rp, col, val)
    b = gen.uniform(9, m.n)
    rc, _ = bad.solve(b)
    assert rc == status, (rc, sp.status_string(rc))
    good = _Dev(torch, m.row_ptr, m.col, m.val)
    rc, x = good.solve(b)
    assert rc == 0, sp.status_string(rc)
    _check(m, b, x)


def test_noalloc_largest_size():
    torch = _torch()
    n = MAX_ROWS
    # diagonal plus superdiagonal: a chain through every row, the last row in the array's last slot
    rng = np.random.default_rng(3)
    rp = np.zeros(n + 1, dtype=np.int64)
    rp[1:] = np.cumsum(np.where(np.arange(n) < n - 1, 2, 1))
    col = np.empty(rp[-1], dtype=np.int32)
    val = np.empty(rp[-1], dtype=np.float64)
    col[rp[:-1]] = np.arange(n, dtype=np.int32)
    val[rp[:-1]] = rng.uniform(2.0, 3.0, n)
    sup = rp[:-2] + 1
    col[sup] = np.arange(1, n, dtype=np.int32)
    val[sup] = rng.uniform(-1.0, 1.0, n - 1)
    d = _Dev(torch, rp, col, val)
    b = rng.uniform(-1.0, 1.0, n)
    rc, x = d.solve(b)
    assert rc == 0, sp.status_string(rc)
    rpu = rp.astype(np.uint64)
    ref = orc.base_gauss_upper(rpu, col, val, b, 1)
    assert orc.max_elem_rel_error(ref, x, 1e-12) <= ELEM_TOL
    assert orc.rel_residual(rpu, col, val, x, b, 1) <= RES_TOL


def test_noalloc_rejects_sizes_beyond_its_array():
    torch = _torch()
    L = _lib.lib()
    d = torch.zeros(4, dtype=torch.float64, device="cuda:0")
    i = torch.zeros(4, dtype=torch.int32, device="cuda:0")
    n = MAX_ROWS + 1
    rc = L.sptrsv_solve_noalloc(n, n, i.data_ptr(), i.data_ptr(), d.data_ptr(), d.data_ptr(), d.data_ptr(), None)
    assert rc == -11 and "maximum" in sp.status_string(rc)
