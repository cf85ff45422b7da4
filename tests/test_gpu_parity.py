"""GPU parity: every schedule and every reference-signature entry point, through the C ABI,
against the reference's own outputs (golden.npz) and the CPU oracle.

Tolerances (FP64 paths): elementwise relative error <= 1e-10 against the reference's serial
solve, relative residual ||b - U x||_2 / ||b||_2 <= 1e-12.  Integer outputs (levels,
in-degree, level buckets and tasks, padded index arrays) are compared bit for bit.
"""
import ctypes
import hashlib

import numpy as np
import pytest

import sptrsv_gb300 as sp
from sptrsv_gb300 import gen

pytestmark = pytest.mark.gpu

ELEM_TOL = 1e-10
RES_TOL = 1e-12
# The refined mixed path is specified by its residual (<= 1e-12); its elementwise error
# against the FP64 solve is then bounded by the conditioning, checked here at 1e-8.
MIXED_ELEM_TOL = 1e-8
GOLDEN_CASES = ["csr_5_upper", "csr_6_upper", "rand3000", "lap12", "chain500", "snr800"]
FP64_SCHEDULES = [("syncfree_warp", 1), ("syncfree_warp", 2), ("syncfree_warp", 4), ("syncfree_warp", 8),
                  ("syncfree_thread", 0), ("syncfree_block", 0), ("syncfree_csc", 0), ("levelset", 0),
                  ("jacobi", 0)]  # FP64 accuracy through refinement (FP32 sweeps, FP64 residuals)


def _case(g, tag):
    rp, col, val = g[tag + "/row_ptr"].astype(np.int64), g[tag + "/col"], g[tag + "/val"]
    rhs = int(g[tag + "/rhs"][0]) if tag + "/rhs" in g else 2
    b = g[tag + "/b"] if tag + "/b" in g else np.ones((len(rp) - 1) * rhs)
    return rp, col, val, b, rhs


def elem_err(x, ref):
    x = np.asarray(x).reshape(-1)
    ref = np.asarray(ref).reshape(-1)
    scale = max(np.max(np.abs(ref)), 1e-300)
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-12 * scale)))


def term_err(m, x, ref, rhs):
    """Elementwise error of a column-major solution relative to the size of the terms its row sums,
    max(|x_i|, sum_j |U_ij x_j| / |U_ii|): the measure for solves whose summation order is not
    fixed (the CSC push adds with atomics, as the reference's CAS kernel does).  Reordering the
    oracle's own sum already moves a nearly cancelling component of this test's systems by 1.5e-10
    relative to |x_i|."""
    import scipy.sparse as sps
    U = sps.csr_matrix((m.val, m.col, m.row_ptr), shape=(m.n, m.n))
    d = np.abs(U.diagonal())
    X = np.asarray(ref).reshape(rhs, m.n).T
    mag = np.maximum(np.abs(X), (abs(U) @ np.abs(X)) / d[:, None] - np.abs(X))
    err = np.abs(np.asarray(x).reshape(rhs, m.n).T - X)
    return float(np.max(err / np.maximum(mag, 1e-300)))


@pytest.fixture(scope="module")
def solver():
    s = sp.Solver(0)
    yield s
    s.close()


@pytest.mark.parametrize("tag", GOLDEN_CASES)
def test_analysis_bit_exact(golden, orc, solver, tag):
    rp, col, val, _, _ = _case(golden, tag)
    solver.analyse(rp, col, val)
    assert np.array_equal(solver.levels(), golden[tag + "/levels"])
    assert solver.info()["max_level"] == int(golden[tag + "/max_level"][0])
    assert np.array_equal(solver.in_degree(), np.diff(rp).astype(np.int32))
    lv, ml = orc.levels(rp.astype(np.uint64), col)
    ptr_o, rows_o = orc.level_buckets(lv, ml)
    ptr, rows = solver.level_buckets()
    assert np.array_equal(ptr, ptr_o) and np.array_equal(rows, rows_o)
    for T in (1, 3, 16):
        assert np.array_equal(solver.level_tasks(T), orc.level_tasks(ml, ptr_o, rows_o, rp.astype(np.uint64), T))


def _csc_matches_oracle(orc, solver, rp, col, val):
    """The device CSR -> CSC transpose against utils.cpp:128-159 restated: integer arrays bit for
    bit, values moved exactly (a permutation, no arithmetic)."""
    solver.analyse(rp, col, val)
    cp, ri, cv = solver.csc()
    cp_o, ri_o, cv_o = orc.transpose(np.asarray(rp, dtype=np.uint64), col, val)
    assert np.array_equal(cp, cp_o)
    assert np.array_equal(ri.astype(np.uint64), ri_o)
    assert np.array_equal(cv.view(np.uint64), cv_o.view(np.uint64))


@pytest.mark.parametrize("tag", GOLDEN_CASES)
def test_device_csc_bit_exact(golden, orc, solver, tag):
    rp, col, val, _, _ = _case(golden, tag)
    _csc_matches_oracle(orc, solver, rp, col, val)


def test_device_csc_bit_exact_2m(orc, solver):
    m, _, _ = gen.irregular_case()
    _csc_matches_oracle(orc, solver, m.row_ptr, m.col, m.val)


def test_levels_200k_digest(golden, solver):
    m = gen.random_upper(200_000, 8.0, 0.9, 64, 1)
    solver.analyse(m.row_ptr, m.col, m.val)
    lv = solver.levels()
    assert solver.info()["max_level"] == int(golden["rand200k/max_level"][0])
    assert hashlib.sha256(lv.tobytes()).digest() == golden["rand200k/levels_sha256"].tobytes()


@pytest.mark.parametrize("tag", GOLDEN_CASES)
@pytest.mark.parametrize("sched,rpw", FP64_SCHEDULES)
def test_fp64_schedules_match_reference(golden, orc, solver, tag, sched, rpw):
    rp, col, val, b, rhs = _case(golden, tag)
    solver.analyse(rp, col, val)
    ref = golden[tag + "/base"]
    if sched in ("syncfree_thread", "syncfree_block"):
        rhs_run, bb, ref = 1, b[: len(rp) - 1], ref[: len(rp) - 1]
    else:
        rhs_run, bb = rhs, b
    x = solver.solve(bb, rhs=rhs_run, schedule=sched, rows_per_warp=rpw or None)
    assert elem_err(x, ref) <= ELEM_TOL
    assert orc.rel_residual(rp.astype(np.uint64), col, val, x, bb, rhs_run) <= RES_TOL


@pytest.fixture(scope="module")
def nd16():
    return gen.laplace3d_nd_cholesky(16, leaf=4)  # n = 4,096, 119 entries per row


@pytest.mark.parametrize("rhs", [3, 8])
@pytest.mark.parametrize("layout", [sp.COL_MAJOR, sp.ROW_MAJOR])
@pytest.mark.parametrize("sched", ["auto", "syncfree_block"])
def test_multi_rhs_long_rows(orc, solver, nd16, rhs, layout, sched):
    """Several right-hand sides of a factor with long rows and no supernode partition: the block
    sync-free kernel once per column (column-major), the RHS-tiled warp kernel (row-major)."""
    m = nd16
    solver.analyse(m.row_ptr, m.col, m.val)
    b_cm = gen.uniform(31 + rhs, m.n * rhs)
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b_cm, rhs)
    if layout == sp.COL_MAJOR:
        x = solver.solve(b_cm, rhs=rhs, layout=layout, schedule=sched)
    else:
        x_rm = solver.solve(b_cm.reshape(rhs, m.n).T.copy().reshape(-1), rhs=rhs, layout=layout, schedule=sched)
        x = x_rm.reshape(m.n, rhs).T.reshape(-1)
    assert elem_err(x, ref) <= ELEM_TOL
    assert orc.rel_residual(m.row_ptr.astype(np.uint64), m.col, m.val, x, b_cm, rhs) <= RES_TOL


@pytest.mark.parametrize("rhs", [2, 5, 8, 33])
@pytest.mark.parametrize("layout", [sp.COL_MAJOR, sp.ROW_MAJOR])
@pytest.mark.parametrize("sched", ["syncfree_warp", "syncfree_csc", "levelset"])
def test_multi_rhs(orc, solver, rhs, layout, sched):
    m = gen.random_upper(5000, 6.0, 0.9, 64, 31)
    solver.analyse(m.row_ptr, m.col, m.val)
    b_cm = gen.uniform(32 + rhs, m.n * rhs)
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b_cm, rhs)
    if layout == sp.ROW_MAJOR:
        b = b_cm.reshape(rhs, m.n).T.copy().reshape(-1)
        x = solver.solve(b, rhs=rhs, layout=layout, schedule=sched).reshape(m.n, rhs).T.reshape(-1)
    else:
        x = solver.solve(b_cm, rhs=rhs, layout=layout, schedule=sched)
    if sched == "syncfree_csc":
        assert term_err(m, x, ref, rhs) <= ELEM_TOL
        assert np.linalg.norm(x - ref) <= 1e-13 * np.linalg.norm(ref)
    else:
        assert elem_err(x, ref) <= ELEM_TOL


@pytest.mark.parametrize("inner", ["jacobi", "syncfree_warp", "syncfree_thread", "syncfree_block", "levelset"])
@pytest.mark.parametrize("tag", ["rand3000", "lap12", "snr800"])
def test_mixed_refinement_reaches_1e12(golden, orc, solver, inner, tag):
    rp, col, val, b, rhs = _case(golden, tag)
    rhs_run = 1 if inner in ("syncfree_thread", "syncfree_block") else rhs
    bb = b[: (len(rp) - 1) * rhs_run]
    solver.analyse(rp, col, val)
    x = solver.solve(bb, rhs=rhs_run, precision="mixed", schedule=inner, max_refine=20)
    steps, res = solver.last_refine()
    assert res <= RES_TOL and steps >= 1
    assert orc.rel_residual(rp.astype(np.uint64), col, val, x, bb, rhs_run) <= 2 * RES_TOL
    assert elem_err(x, golden[tag + "/base"][: len(x)]) <= MIXED_ELEM_TOL


@pytest.mark.parametrize("layout", ["jds", "batch8", "sell"])
def test_mixed_sweep_layouts(golden, orc, monkeypatch, layout):
    """The selectable layouts of the Jacobi sweep (SPTRSV_SWEEP_KERNEL, read when a handle is
    created) reach the same tolerances as the default paired layout: rows of every length, groups
    and slices cut by n, and the 2-8-row tails of the golden systems."""
    monkeypatch.setenv("SPTRSV_SWEEP_KERNEL", layout)
    m = gen.random_upper(50_003, 8.0, 0.9, 64, 5)
    xs, b = gen.system(m, 11)
    cases = [(m.row_ptr, m.col, m.val, b)]
    for t in ("rand3000", "snr800", "csr_5_upper"):
        rp, col, val, bt, _ = _case(golden, t)
        cases.append((rp, col, val, bt[: len(rp) - 1]))
    with sp.Solver(0) as s:
        for rp, col, val, bb in cases:
            s.analyse(rp, col, val)
            x = s.solve(bb, precision="mixed", schedule="jacobi", max_refine=20)
            assert s.last_refine()[1] <= RES_TOL, layout
            ref = orc.base_gauss_upper(np.asarray(rp).astype(np.uint64), col, val, bb, 1)
            assert orc.rel_residual(np.asarray(rp).astype(np.uint64), col, val, x, bb, 1) <= 2 * RES_TOL
            assert elem_err(x, ref) <= MIXED_ELEM_TOL, layout


def _tiny_cases():
    rng = np.random.default_rng(21)
    out = [("n1", np.array([0, 1]), np.array([0], dtype=np.int32), np.array([2.0]))]
    for n in (2, 31, 32, 33, 65):
        m = gen.random_upper(n, 3.0, 0.9, 8, n)
        out.append((f"rand{n}", m.row_ptr, m.col, m.val))
    n = 1000  # diagonal only: no off-diagonal anywhere
    out.append(("diag1000", np.arange(n + 1), np.arange(n, dtype=np.int32), rng.uniform(1.0, 2.0, n)))
    n = 96  # dense upper triangle: rows far longer than the short-row sweeps take
    rp = np.concatenate([[0], np.cumsum(np.arange(n, 0, -1))])
    col = np.concatenate([np.arange(i, n) for i in range(n)]).astype(np.int32)
    val = rng.uniform(-1.0, 1.0, len(col))
    for i in range(n):
        val[rp[i]] = 1.0 + np.abs(val[rp[i] + 1:rp[i + 1]]).sum()
    out.append(("dense96", rp, col, val))
    return out


@pytest.mark.parametrize("case", _tiny_cases(), ids=lambda c: c[0])
def test_tiny_and_degenerate_systems(orc, solver, case):
    """One-row, diagonal-only, warp-boundary sizes and a dense triangle through every FP64
    schedule, the mixed path and several right-hand sides, against the serial solve."""
    _, rp, col, val = case
    n = len(rp) - 1
    rpu = np.asarray(rp).astype(np.uint64)
    solver.analyse(rp, col, val)
    lv, ml = orc.levels(rpu, col)
    assert solver.info()["max_level"] == ml and np.array_equal(solver.levels(), lv)
    b = gen.uniform(n + 5, n * 3)
    ref1 = orc.base_gauss_upper(rpu, col, val, b[:n], 1)
    for sched, rpw in FP64_SCHEDULES:
        x = solver.solve(b[:n], schedule=sched, rows_per_warp=rpw)
        assert elem_err(x, ref1) <= ELEM_TOL, sched
    x = solver.solve(b[:n], precision="mixed", max_refine=20)
    assert solver.last_refine()[1] <= RES_TOL
    assert elem_err(x, ref1) <= MIXED_ELEM_TOL
    ref3 = orc.base_gauss_upper(rpu, col, val, b, 3)
    for sched in ("syncfree_warp", "syncfree_csc", "levelset"):
        x = solver.solve(b, rhs=3, schedule=sched)
        assert elem_err(x, ref3) <= ELEM_TOL, sched


def test_empty_system_is_an_error(solver):
    with pytest.raises(sp.SptrsvError) as e:
        solver.analyse(np.array([0]), np.zeros(0, dtype=np.int32), np.zeros(0))
    assert e.value.status == -2  # SPTRSV_ERR_INVALID_ARG
    # the handle stays usable
    solver.analyse(np.array([0, 1]), np.array([0], dtype=np.int32), np.array([4.0]))
    assert solver.solve(np.array([2.0]))[0] == 0.5


def test_device_pointer_api(orc, solver):
    torch = pytest.importorskip("torch")
    m = gen.random_upper(20_000, 8.0, 0.9, 64, 41)
    rhs = 4
    dev = torch.device("cuda:0")
    rp = torch.tensor(m.row_ptr.astype(np.int32), device=dev)
    col = torch.tensor(m.col, device=dev)
    val = torch.tensor(m.val, device=dev)
    b_cm = gen.uniform(42, m.n * rhs)
    b_rm = torch.tensor(b_cm.reshape(rhs, m.n).T.copy(), device=dev)
    x = torch.empty_like(b_rm)
    solver.analyse_device(m.n, m.nnz, rp.data_ptr(), col.data_ptr(), val.data_ptr())
    torch.cuda.synchronize()
    solver.solve_device(b_rm.data_ptr(), x.data_ptr(), rhs=rhs, layout=sp.ROW_MAJOR)
    assert solver.sync() == 0
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b_cm, rhs)
    assert elem_err(x.cpu().numpy().T.reshape(-1), ref) <= ELEM_TOL


def test_host_buffers_pinned_and_pageable(orc):
    """sptrsv_solve_host with pinned host x: the refinement's residual kernels write x to the host
    directly (no copy after the solve).  Same solution as the device-pointer solve and the oracle
    tolerances; a zero right-hand side, an unconverged solve (its status, and the same x as the
    device path) and pageable numpy buffers (the copy path) behave as before."""
    L = sp._lib.lib()
    m = gen.random_upper(50_000, 8.0, 0.9, 64, 43)
    xs, b = gen.system(m, 44)
    n, nb = m.n, 8 * m.n
    rpu = m.row_ptr.astype(np.uint64)
    ref = orc.base_gauss_upper(rpu, m.col, m.val, b, 1)
    with sp.Solver(0) as s:
        s.analyse(m.row_ptr, m.col, m.val)
        h = s.handle
        hb, hx, db, dx = (ctypes.c_void_p() for _ in range(4))
        assert L.sptrsv_host_alloc(h, nb, ctypes.byref(hb)) == 0 and L.sptrsv_host_alloc(h, nb, ctypes.byref(hx)) == 0
        assert L.sptrsv_device_alloc(h, nb, ctypes.byref(db)) == 0 and L.sptrsv_device_alloc(h, nb, ctypes.byref(dx)) == 0
        hb_np = np.ctypeslib.as_array(ctypes.cast(hb, ctypes.POINTER(ctypes.c_double)), shape=(n,))
        hx_np = np.ctypeslib.as_array(ctypes.cast(hx, ctypes.POINTER(ctypes.c_double)), shape=(n,))

        def device_x(o, bb):
            L.sptrsv_copy_h2d(h, db, bb.ctypes.data, nb)
            rc = L.sptrsv_solve(h, ctypes.byref(o), db, dx, 1, sp.COL_MAJOR)
            rc = rc or s.sync()
            out = np.empty(n)
            L.sptrsv_copy_d2h(h, out.ctypes.data, dx, nb)
            assert s.sync() in (0, -10)
            return rc, out

        try:
            o = sp.make_opts(precision="mixed", schedule="jacobi")
            rc_d, x_dev = device_x(o, b)
            assert rc_d == 0
            for _ in range(2):  # the second call replays the cached graph
                hb_np[:] = b
                hx_np[:] = np.nan
                assert L.sptrsv_solve_host(h, ctypes.byref(o), hb, hx, 1, sp.COL_MAJOR) == 0
                x = hx_np.copy()
                assert s.last_refine()[1] <= RES_TOL
                assert orc.rel_residual(rpu, m.col, m.val, x, b, 1) <= 2 * RES_TOL
                assert elem_err(x, ref) <= MIXED_ELEM_TOL
                assert np.max(np.abs(x - x_dev)) <= 1e-13 * np.max(np.abs(x_dev))
            # zero right-hand side: converged on x = 0 before any residual of a nonzero x
            hb_np[:] = 0.0
            hx_np[:] = np.nan
            assert L.sptrsv_solve_host(h, ctypes.byref(o), hb, hx, 1, sp.COL_MAJOR) == 0
            assert np.all(hx_np == 0.0)
            # unconverged: one correction of a loose inner solve
            o1 = sp.make_opts(precision="mixed", schedule="jacobi", max_refine=1, inner_tol_exp=1)
            rc_d, x_dev1 = device_x(o1, b)
            hb_np[:] = b
            hx_np[:] = np.nan
            assert L.sptrsv_solve_host(h, ctypes.byref(o1), hb, hx, 1, sp.COL_MAJOR) == rc_d == -10
            assert np.array_equal(hx_np, x_dev1)
        finally:
            L.sptrsv_host_free(h, hb)
            L.sptrsv_host_free(h, hx)
            L.sptrsv_device_free(h, db)
            L.sptrsv_device_free(h, dx)
        # pageable numpy buffers take the copy path
        x = s.solve(b, precision="mixed", schedule="jacobi")
        assert elem_err(x, ref) <= MIXED_ELEM_TOL


# ---------------------------------------------------------------------------------------
# The reference-signature entry points

@pytest.mark.parametrize("tag", GOLDEN_CASES)
def test_dropin_base_and_barrier(golden, tag):
    rp, col, val, b, rhs = _case(golden, tag)
    n = len(rp) - 1
    rpu = rp.astype(np.uint64)
    for name, key in (("base_gauss_upper", "base"), ("base_gauss_upper_new", "base_new")):
        x = np.zeros(n * rhs)
        t = getattr(sp, name)(n, val, rpu, col, x, b.copy(), rhs)
        assert t >= 0, sp.status_string(int(t))
        assert elem_err(x, golden[f"{tag}/{key}"]) <= ELEM_TOL
    for name in ("barrier_upper", "barrier_upper_new"):
        x = np.zeros(n * rhs)
        t = getattr(sp, name)(n, x, b.copy(), val, col, rpu, 4, rhs)
        assert t >= 0
        assert elem_err(x, golden[f"{tag}/barrier_t3"]) <= ELEM_TOL
    lv = np.zeros(n, dtype=np.uint64)
    ml = sp.setLevelUpAndGetMaxLevel(n, col, rpu, lv)
    assert ml == int(golden[tag + "/max_level"][0]) and np.array_equal(lv, golden[tag + "/levels"])


@pytest.mark.parametrize("tag", ["csr_6_upper", "snr800"])
def test_dropin_supernodal(golden, tag):
    rp, col, val, b, rhs = _case(golden, tag)
    n = len(rp) - 1
    rpu = rp.astype(np.uint64)
    snodes = golden[tag + "/snodes"].astype(np.int32)
    sn = len(snodes) - 1
    for name, key in (("supernodal_upper", "super"), ("supernodal_upper_new", "super_new")):
        x = b.copy()
        t = getattr(sp, name)(sn, snodes, x, val, col, rpu, n, rhs)
        assert t >= 0
        assert elem_err(x, golden[f"{tag}/{key}"]) <= ELEM_TOL
    w = np.diff(snodes).astype(np.int64)
    total = int(rp[-1]) + int(np.sum(w * (w - 1) // 2))
    vp = np.zeros(total)
    cp = np.zeros(total, dtype=np.uint64)
    rpp = np.zeros(n + 1, dtype=np.int32)
    sn_c, nz_c = ctypes.c_int(sn), ctypes.c_int(0)
    t = sp.ccs2ccs_pad(val, col, rpu, vp, cp, rpp, snodes, sn_c, nz_c)
    assert t >= 0 and nz_c.value == len(golden[tag + "/pad_val"])
    assert np.array_equal(vp, golden[tag + "/pad_val"])
    assert np.array_equal(cp, golden[tag + "/pad_col"])
    assert np.array_equal(rpp, golden[tag + "/pad_rowptr"])
    for name in ("supernodal_blas_upper", "supernodal_blas_upper_new"):
        x = b.copy()
        t = getattr(sp, name)(n, nz_c.value, sn, snodes, x, vp, cp, rpp, rhs)
        assert t >= 0
        assert elem_err(x, golden[tag + "/blas"]) <= ELEM_TOL


@pytest.mark.parametrize("tag", GOLDEN_CASES)
def test_dropin_syncfree_opencl(golden, orc, tag):
    rp, col, val, b, rhs = _case(golden, tag)
    n = len(rp) - 1
    cp, rt, vt = orc.transpose(rp.astype(np.uint64), col, val)
    rt32 = rt.astype(np.int32)
    ref_cm = golden[tag + "/base"]
    b_rm = b.reshape(rhs, n).T.copy().reshape(-1)
    x = np.zeros(n * rhs)
    t = sp.sptrsv_syncfree_opencl(cp, rt32, vt, n, n, len(vt), x, b_rm, rhs)
    assert t >= 0
    assert elem_err(x.reshape(n, rhs).T.reshape(-1), ref_cm) <= ELEM_TOL
    x1 = np.zeros(n)
    assert sp.sptrsv_syncfree2_opencl(cp, rt32, vt, n, n, len(vt), x1, b[:n].copy()) >= 0
    assert elem_err(x1, ref_cm[:n]) <= ELEM_TOL
    x3 = np.zeros(n)
    assert sp.sptrsv_syncfree3_opencl(col, rp.astype(np.int32), val, n, n, len(val), x3, b[:n].copy()) >= 0
    assert elem_err(x3, ref_cm[:n]) <= ELEM_TOL
    assert sp.sptrsv_syncfree_opencl(cp, rt32, vt, n, n + 1, len(vt), x, b_rm, rhs) == -1.0


# ---------------------------------------------------------------------------------------
# Invalid inputs are reported, never hang or fault

def _bad(kind):
    m = gen.random_upper(3000, 5.0, 0.9, 32, 51)
    rp, col, val = m.row_ptr.copy(), m.col.copy(), m.val.copy()
    i = 1234
    s = rp[i]
    if kind == "missing_diag":
        col[s] = col[s + 1] if rp[i + 1] - s > 1 else i + 1
        want = -5
    elif kind == "lower":
        col[s + 1] = i - 3
        want = -6
    elif kind == "col_range":
        col[s + 1] = m.n + 7
        want = -7
    elif kind == "row_ptr":
        rp[i] = rp[i + 1] + 2
        want = -4
    elif kind == "zero_pivot":
        val[s] = 0.0
        want = -8
    elif kind == "nan_pivot":
        val[s] = np.nan
        want = -8
    return m.n, rp, col, val, want


@pytest.mark.parametrize("kind", ["missing_diag", "lower", "col_range", "row_ptr", "zero_pivot", "nan_pivot"])
def test_invalid_matrix_statuses(solver, kind):
    n, rp, col, val, want = _bad(kind)
    if kind == "lower" and rp[1235] - rp[1234] < 2:
        pytest.skip("row too short for this injection")
    with pytest.raises(sp.SptrsvError) as e:
        solver.analyse(rp, col, val)
    assert e.value.status == want
    x = np.zeros(n)
    t = sp.base_gauss_upper(n, val, rp.astype(np.uint64), col, x, np.ones(n), 1)
    assert t == float(want) and sp.last_status() == want


def test_spin_budget_timeout_then_recovery(orc, solver):
    # a pure chain: row i depends on row i+1; a 1 ns wait budget must run out
    n = 200_000
    rp = np.arange(0, 2 * n, 2, dtype=np.int64)
    rp = np.append(rp, 2 * n - 1)
    col = np.empty(2 * n - 1, dtype=np.int32)
    col[0::2] = np.arange(n)
    col[1::2] = np.arange(1, n)
    val = np.empty(2 * n - 1)
    val[0::2] = 2.0
    val[1::2] = -1.0
    solver.analyse(rp, col, val)
    b = np.ones(n)
    for sched in ("syncfree_warp", "syncfree_block"):
        with pytest.raises(sp.SptrsvError) as e:
            solver.solve(b, schedule=sched, spin_budget_ns=1)
        assert e.value.status == -9
    x = solver.solve(b, schedule="syncfree_block")
    ref = orc.base_gauss_upper(rp.astype(np.uint64), col, val, b, 1)
    assert elem_err(x, ref) <= ELEM_TOL


# ---------------------------------------------------------------------------------------
# Full-size workloads

def test_band_laplace_full(orc, solver):
    m, xs, b = gen.band_laplace_case()
    solver.analyse(m.row_ptr, m.col, m.val)
    assert solver.info()["max_level"] == 4096
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b, 1)
    for sched in ("syncfree_warp", "syncfree_thread", "syncfree_csc", "levelset"):
        x = solver.solve(b, schedule=sched)
        assert elem_err(x, ref) <= ELEM_TOL, sched
        assert orc.rel_residual(m.row_ptr.astype(np.uint64), m.col, m.val, x, b, 1) <= RES_TOL
    x = solver.solve(b, precision="mixed")
    assert solver.last_refine()[1] <= RES_TOL
    assert elem_err(x, ref) <= MIXED_ELEM_TOL
    # FP64 AUTO on this skyline matrix (every row one contiguous band): exact FP64 panels over
    # uniform 256-row chunks, one and three right-hand sides, and the drop-in
    x = solver.solve(b)
    assert elem_err(x, ref) <= ELEM_TOL
    b3 = gen.uniform(77, m.n * 3)
    ref3 = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b3, 3)
    assert elem_err(solver.solve(b3, rhs=3), ref3) <= ELEM_TOL
    xd = np.zeros(m.n)
    assert sp.base_gauss_upper(m.n, m.val, m.row_ptr.astype(np.uint64), m.col, xd, b, 1) > 0
    assert sp.last_status() == 0 and elem_err(xd, ref) <= ELEM_TOL


def test_irregular_2m_full(orc, solver):
    m, xs, b = gen.irregular_case()
    solver.analyse(m.row_ptr, m.col, m.val)
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b, 1)
    for sched in ("syncfree_warp", "syncfree_block"):
        x = solver.solve(b, schedule=sched)
        assert elem_err(x, ref) <= ELEM_TOL, sched
    x = solver.solve(b, precision="mixed", schedule="jacobi")
    steps, res = solver.last_refine()
    assert res <= RES_TOL
    assert elem_err(x, ref) <= MIXED_ELEM_TOL
    # property at full size: the solution of U x = U x* is x*
    assert np.max(np.abs(x - xs)) <= 1e-9
    # FP64 accuracy through refinement, explicitly and through the drop-in (348,506 levels: the
    # drop-in's cost model takes the refinement here)
    x = solver.solve(b, schedule="jacobi")
    assert solver.last_refine()[1] <= 1e-15
    assert elem_err(x, ref) <= ELEM_TOL
    xd = np.zeros(m.n)
    secs = sp.base_gauss_upper(m.n, m.val, m.row_ptr.astype(np.uint64), m.col, xd, b, 1)
    assert secs > 0 and sp.last_status() == 0
    assert elem_err(xd, ref) <= ELEM_TOL
    assert orc.rel_residual(m.row_ptr.astype(np.uint64), m.col, m.val, xd, b, 1) <= RES_TOL


@pytest.mark.parametrize("tag", ["csr_6_lower", "lower3000"])
def test_dropin_base_gauss_lower(golden, tag):
    """core.h:9: the lower solve, run as the reversed upper system on the GPU."""
    rp = golden[tag + "/row_ptr"].astype(np.uint64)
    col, val, b = golden[tag + "/col"], golden[tag + "/val"], golden[tag + "/b"]
    n = len(rp) - 1
    x = np.zeros(n)
    secs = sp.base_gauss_lower(n, val.copy(), rp.copy(), col.copy(), x, b.copy())
    assert secs >= 0
    assert elem_err(x, golden[tag + "/lower"]) <= ELEM_TOL


def test_dropin_base_gauss_lower_deep(orc):
    """A deep lower system with dominant rows (the reversal of a 200k-row dominant upper factor,
    ~60k levels): the drop-in takes FP64 accuracy through refinement on the reversed system."""
    m = gen.random_upper(200_000, 8.0, 0.9, 64, 17)
    n, nnz = m.n, m.nnz
    lrp = (nnz - m.row_ptr[::-1]).astype(np.uint64)
    lcol = (n - 1 - m.col[::-1]).astype(np.int32)
    lval = m.val[::-1].copy()
    b = gen.uniform(18, n)
    ref = orc.base_gauss_lower(lrp, lcol, lval, b)
    x = np.zeros(n)
    assert sp.base_gauss_lower(n, lval.copy(), lrp.copy(), lcol.copy(), x, b.copy()) > 0
    assert sp.last_status() == 0
    assert elem_err(x, ref) <= ELEM_TOL


def test_dropin_base_gauss_upper_deep_multi_rhs(orc):
    """Three column-major right-hand sides of a deep dominant system through the drop-in (the
    refinement path with rhs > 1), against the serial solve."""
    m = gen.random_upper(200_000, 8.0, 0.9, 64, 19)
    rpu = m.row_ptr.astype(np.uint64)
    b = gen.uniform(20, m.n * 3)
    ref = orc.base_gauss_upper(rpu, m.col, m.val, b, 3)
    x = np.zeros(m.n * 3)
    assert sp.base_gauss_upper(m.n, m.val, rpu, m.col, x, b, 3) > 0 and sp.last_status() == 0
    assert elem_err(x, ref) <= ELEM_TOL
    assert orc.rel_residual(rpu, m.col, m.val, x, b, 3) <= RES_TOL


def test_dropin_base_gauss_lower_rejects_upper(golden):
    rp = golden["csr_6_upper/row_ptr"].astype(np.uint64)
    col, val = golden["csr_6_upper/col"], golden["csr_6_upper/val"]
    x = np.zeros(6)
    assert sp.base_gauss_lower(6, val.copy(), rp.copy(), col.copy(), x, np.ones(6)) < 0


@pytest.mark.parametrize("p_near", [0.0, 0.9])
@pytest.mark.parametrize("warps", [None, 32, 100_000])
def test_levelset_grids(orc, solver, p_near, warps):
    """The level-set solve on one CTA (its barrier the CTA barrier) and on one CTA per SM (the grid
    barrier through L2), and as the analysis' cost model picks, on a wide DAG (every column far:
    few wide levels) and a narrow one (near columns: many narrow levels), one and three RHS.  The
    all-far matrix has tiny solution components, so the elementwise bound is the larger of 1e-10
    and ten times the reordering floor (the serial solve against itself summed in reverse) on the
    same inputs; every grid must also give the same x."""
    m = gen.random_upper(100_000, 5.0, p_near, 64, 13)
    solver.analyse(m.row_ptr, m.col, m.val)
    rpu = m.row_ptr.astype(np.uint64)
    for rhs in (1, 3):
        b = gen.uniform(60 + rhs, m.n * rhs)
        ref = orc.base_gauss_upper(rpu, m.col, m.val, b, rhs)
        floor = elem_err(orc.base_gauss_upper_rev(rpu, m.col, m.val, b, rhs), ref)
        x = solver.solve(b, rhs=rhs, schedule="levelset", resident_warps=warps)
        assert elem_err(x, ref) <= max(ELEM_TOL, 10 * floor), (rhs, warps, floor)
        assert orc.rel_residual(rpu, m.col, m.val, x, b, rhs) <= RES_TOL
        assert np.array_equal(x, solver.solve(b, rhs=rhs, schedule="levelset", resident_warps=32))
