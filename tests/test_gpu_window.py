"""The one-CTA window kernel (window.cu): the FP64 sync-free solve (schedule syncfree_window, FP64
AUTO for one right-hand side) and the level analysis (the default levels kernel), against the
reference's own outputs and the CPU oracle.

The cases cover the ring protocol's regions: dependencies inside a 32-row block, on the blocks
in flight, on finished blocks still in the shared-memory ring, and beyond the ring's reach (read
from global memory) -- including a band of 4,000 columns that straddles the reach (3,040 rows at
16 warps).  Tolerances are those of the other FP64 paths: elementwise relative error <= 1e-10
against the serial solve, relative residual <= 1e-12; levels bit for bit.
"""
import numpy as np
import pytest

import sptrsv_gb300 as sp
from sptrsv_gb300 import gen

pytestmark = pytest.mark.gpu

ELEM_TOL = 1e-10
RES_TOL = 1e-12
GOLDEN_CASES = ["csr_5_upper", "csr_6_upper", "rand3000", "lap12", "chain500", "snr800"]


def elem_err(x, ref):
    x = np.asarray(x).reshape(-1)
    ref = np.asarray(ref).reshape(-1)
    scale = max(np.max(np.abs(ref)), 1e-300)
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-12 * scale)))


@pytest.fixture(scope="module")
def solver():
    s = sp.Solver(0)
    yield s
    s.close()


def _solve_check(orc, solver, rp, col, val, b, rhs=1, **opts):
    solver.analyse(rp, col, val)
    rpu = np.asarray(rp, dtype=np.uint64)
    ref = orc.base_gauss_upper(rpu, col, val, b, rhs)
    x = solver.solve(b, rhs=rhs, **opts)
    assert elem_err(x, ref) <= ELEM_TOL
    assert orc.rel_residual(rpu, col, val, x, b, rhs) <= RES_TOL
    return x


@pytest.mark.parametrize("tag", GOLDEN_CASES)
def test_window_matches_reference(golden, orc, solver, tag):
    rp = golden[tag + "/row_ptr"].astype(np.int64)
    col, val = golden[tag + "/col"], golden[tag + "/val"]
    n = len(rp) - 1
    b = golden[tag + "/b"][:n] if tag + "/b" in golden else np.ones(n)
    solver.analyse(rp, col, val)
    x = solver.solve(b, schedule="syncfree_window")
    assert elem_err(x, golden[tag + "/base"][:n]) <= ELEM_TOL
    assert orc.rel_residual(rp.astype(np.uint64), col, val, x, b, 1) <= RES_TOL


@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 1000, 4096, 4097, 70_001])
def test_window_sizes(orc, solver, n):
    m = gen.random_upper(n, 6.0, 0.9, 64, n % 97 + 3)
    _solve_check(orc, solver, m.row_ptr, m.col, m.val, gen.uniform(n + 1, n), schedule="syncfree_window")


@pytest.mark.parametrize("band,p_near", [(4000, 1.0), (4000, 0.5), (3040, 1.0), (1, 1.0), (200, 0.0)])
def test_window_ring_regions(orc, solver, band, p_near):
    """Near offsets up to `band` (straddling the ring's reach), far ones uniform over the rest."""
    m = gen.random_upper(150_000, 8.0, p_near, band, band + 7)
    _solve_check(orc, solver, m.row_ptr, m.col, m.val, gen.uniform(band, m.n), schedule="syncfree_window")


def test_window_levels_match_oracle_regions(orc, solver):
    for band, p_near in ((4000, 0.9), (64, 0.9), (1, 1.0)):
        m = gen.random_upper(150_000, 8.0, p_near, band, 11)
        solver.analyse(m.row_ptr, m.col, m.val)
        lv, ml = orc.levels(m.row_ptr.astype(np.uint64), m.col)
        assert solver.info()["max_level"] == ml
        assert np.array_equal(solver.levels(), lv)


def test_window_band_laplace_full(orc, solver):
    m, _, b = gen.band_laplace_case()
    _solve_check(orc, solver, m.row_ptr, m.col, m.val, b, schedule="syncfree_window")


def test_window_irregular_2m_full(orc, solver):
    m, xs, b = gen.irregular_case()
    x = _solve_check(orc, solver, m.row_ptr, m.col, m.val, b, schedule="syncfree_window")
    assert np.max(np.abs(x - xs)) <= 1e-9
    # FP64 AUTO with one RHS is this kernel (the analysis already ran)
    assert elem_err(solver.solve(b), x) <= ELEM_TOL
    # levels of the 2M system, bit for bit
    lv, ml = orc.levels(m.row_ptr.astype(np.uint64), m.col)
    assert solver.info()["max_level"] == ml
    assert np.array_equal(solver.levels(), lv)


@pytest.mark.parametrize("rhs", [2, 5])
def test_window_column_major_columns(orc, solver, rhs):
    m = gen.random_upper(60_000, 8.0, 0.9, 64, 5)
    b = gen.uniform(40 + rhs, m.n * rhs)
    _solve_check(orc, solver, m.row_ptr, m.col, m.val, b, rhs=rhs, schedule="syncfree_window")


def test_window_row_major_rhs_falls_back(orc, solver):
    m = gen.random_upper(20_000, 8.0, 0.9, 64, 6)
    rhs = 3
    b_cm = gen.uniform(9, m.n * rhs)
    solver.analyse(m.row_ptr, m.col, m.val)
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b_cm, rhs)
    x_rm = solver.solve(b_cm.reshape(rhs, m.n).T.copy().reshape(-1), rhs=rhs, layout=sp.ROW_MAJOR,
                        schedule="syncfree_window")
    assert elem_err(x_rm.reshape(m.n, rhs).T.reshape(-1), ref) <= ELEM_TOL


def test_window_mixed_inner(orc, solver):
    m = gen.random_upper(100_000, 8.0, 0.9, 64, 8)
    b = gen.uniform(3, m.n)
    solver.analyse(m.row_ptr, m.col, m.val)
    x = solver.solve(b, precision="mixed", schedule="syncfree_window")
    assert solver.last_refine()[1] <= RES_TOL
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b, 1)
    assert elem_err(x, ref) <= 1e-8


def test_window_timeout_then_recovers(orc, solver):
    """A 1 ns spin budget on a chain ends with the timeout status (no hang); the same handle then
    solves correctly."""
    n = 20_000
    rp = np.zeros(n + 1, dtype=np.int64)
    rp[1:] = np.cumsum(np.where(np.arange(n) < n - 1, 2, 1))
    col = np.empty(rp[-1], dtype=np.int32)
    val = np.empty(rp[-1])
    col[rp[:-1]] = np.arange(n)
    val[rp[:-1]] = 2.0
    col[rp[:-2] + 1] = np.arange(1, n)
    val[rp[:-2] + 1] = -1.0
    solver.analyse(rp, col, val)
    b = np.ones(n)
    with pytest.raises(sp.SptrsvError) as e:
        solver.solve(b, schedule="syncfree_window", spin_budget_ns=1)
    assert e.value.status == -9
    x = solver.solve(b, schedule="syncfree_window")
    ref = orc.base_gauss_upper(rp.astype(np.uint64), col, val, b, 1)
    assert elem_err(x, ref) <= ELEM_TOL


@pytest.mark.parametrize("band,p_near", [(4000, 0.5), (64, 0.9)])
def test_window_unsorted_rows(orc, solver, band, p_near):
    """Rows whose off-diagonal entries are stored in a shuffled order (the diagonal stays first):
    far columns then follow near ones, and the rounds must read them from global x."""
    m = gen.random_upper(120_000, 8.0, p_near, band, band + 3)
    rp = m.row_ptr.astype(np.int64)
    col = np.array(m.col, dtype=np.int32)
    val = np.array(m.val, dtype=np.float64)
    rng = np.random.default_rng(17)
    for r in range(m.n):
        a, e = rp[r] + 1, rp[r + 1]
        if e - a > 1:
            perm = a + rng.permutation(e - a)
            col[a:e] = col[perm]
            val[a:e] = val[perm]
    b = gen.uniform(band, m.n)
    _solve_check(orc, solver, rp, col, val, b, schedule="syncfree_window")
    lv, ml = orc.levels(rp.astype(np.uint64), col)
    assert solver.info()["max_level"] == ml
    assert np.array_equal(solver.levels(), lv)
