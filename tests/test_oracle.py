"""The CPU oracle (oracle/oracle.c) against the reference's own outputs (golden.npz, made by
tests/golden/make_golden.py from the reference's core.cpp) and, where it is built here,
against the reference core.cpp live."""
import numpy as np
import pytest

GOLDEN_CASES = ["csr_5_upper", "csr_6_upper", "rand3000", "lap12", "chain500", "snr800"]


def _case(g, tag):
    rp, col, val = g[tag + "/row_ptr"], g[tag + "/col"], g[tag + "/val"]
    rhs = int(g[tag + "/rhs"][0]) if tag + "/rhs" in g else 2
    b = g[tag + "/b"] if tag + "/b" in g else np.ones((len(rp) - 1) * rhs)
    return rp.astype(np.uint64), col.astype(np.int32), val, b, rhs


@pytest.mark.parametrize("tag", GOLDEN_CASES)
def test_base_gauss_upper_matches_reference(golden, orc, tag):
    rp, col, val, b, rhs = _case(golden, tag)
    for new, key in ((False, "base"), (True, "base_new")):
        x = orc.base_gauss_upper(rp, col, val, b, rhs, new=new)
        ref = golden[f"{tag}/{key}"]
        assert np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)) <= 1e-13


@pytest.mark.parametrize("tag", GOLDEN_CASES)
def test_levels_bit_exact(golden, orc, tag):
    rp, col, _, _, _ = _case(golden, tag)
    lv, ml = orc.levels(rp, col)
    assert np.array_equal(lv, golden[tag + "/levels"])
    assert ml == int(golden[tag + "/max_level"][0])


def test_levels_digest_200k(golden, orc):
    import hashlib
    from sptrsv_gb300 import gen
    m = gen.random_upper(200_000, 8.0, 0.9, 64, 1)
    assert m.nnz == int(golden["rand200k/nnz"][0])
    lv, ml = orc.levels(m.row_ptr.astype(np.uint64), m.col)
    assert ml == int(golden["rand200k/max_level"][0])
    assert hashlib.sha256(lv.tobytes()).digest() == golden["rand200k/levels_sha256"].tobytes()


@pytest.mark.parametrize("tag", GOLDEN_CASES)
@pytest.mark.parametrize("threads", [1, 3])
def test_barrier_matches_reference(golden, orc, tag, threads):
    rp, col, val, b, rhs = _case(golden, tag)
    for new, key in ((False, "barrier"), (True, "barrier_new")):
        x = orc.barrier_upper(rp, col, val, b, rhs, num_threads=threads, new=new)
        ref = golden[f"{tag}/{key}_t{threads}"]
        assert np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)) <= 1e-13


@pytest.mark.parametrize("tag", ["csr_6_upper", "snr800"])
def test_supernodal_matches_reference(golden, orc, tag):
    rp, col, val, b, rhs = _case(golden, tag)
    sn = golden[tag + "/snodes"]
    for new, key in ((False, "super"), (True, "super_new")):
        x = orc.supernodal_upper(sn, rp, col, val, b, rhs, new=new)
        ref = golden[f"{tag}/{key}"]
        assert np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)) <= 1e-13
    rpp, cp, vp = orc.ccs2ccs_pad(sn, rp, col, val)
    assert np.array_equal(rpp[1:], golden[tag + "/pad_rowptr"][1:])
    assert np.array_equal(cp, golden[tag + "/pad_col"])
    assert np.array_equal(vp, golden[tag + "/pad_val"])
    x = orc.supernodal_blas_upper(sn, rpp, cp, vp, b, rhs)
    ref = golden[tag + "/blas"]
    assert np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)) <= 1e-12
    # the same algorithm with its dgemm / dtrsm on numpy's OpenBLAS (the CPU baseline's BLAS)
    xo = orc.supernodal_blas_upper_openblas(sn, rpp, cp, vp, b, rhs)
    if xo is not None:
        assert np.max(np.abs(xo - ref) / np.maximum(np.abs(ref), 1e-300)) <= 1e-12


def test_shipped_fixture_known_answers(golden):
    # the values the reference's core.cpp produced on its own fixtures (b = 1)
    x6 = golden["csr_6_upper/base"][:6]
    assert np.allclose(x6, [0.5, 0.875, 1 / 12, 0.5, 5 / 24, 1 / 6], rtol=1e-14)
    assert list(golden["csr_6_upper/levels"]) == [2, 4, 3, 1, 2, 1]
    x5 = golden["csr_5_upper/base"][:5]
    assert np.allclose(x5, [0.6, 1 / 3, 0.25, 0.2, 1 / 6], rtol=1e-14)
    assert list(golden["csr_5_upper/levels"]) == [2, 1, 1, 1, 1]


@pytest.mark.parametrize("tag", GOLDEN_CASES)
def test_level_buckets_and_tasks(golden, orc, tag):
    rp, col, _, _, _ = _case(golden, tag)
    lv, ml = orc.levels(rp, col)
    ptr, rows = orc.level_buckets(lv, ml)
    assert ptr[0] == 0 and ptr[1] == 0 and ptr[-1] == len(lv)
    for l in range(1, ml + 1):
        seg = rows[ptr[l]:ptr[l + 1]]
        assert np.all(np.diff(seg) > 0) and np.all(lv[seg] == l)
    for T in (1, 4):
        tasks = orc.level_tasks(ml, ptr, rows, rp, T)
        assert np.all(tasks[:, 0] == 0)
        assert np.array_equal(tasks[:, -1], np.diff(ptr)[: ml + 1])


@pytest.mark.parametrize("tag", GOLDEN_CASES)
def test_transpose_and_csc_solve(golden, orc, tag):
    rp, col, val, b, rhs = _case(golden, tag)
    n = len(rp) - 1
    cp, rt, vt = orc.transpose(rp, col, val)
    for j in range(0, n, max(1, n // 50)):
        seg = rt[cp[j]:cp[j + 1]]
        assert np.all(np.diff(seg.astype(np.int64)) > 0) and int(seg[-1]) == j
    indeg = orc.in_degree_csc(n, rt.astype(np.int32))
    assert np.array_equal(indeg, np.diff(rp.astype(np.int64)).astype(np.int32))
    bm = b.reshape(rhs, n).T.copy().reshape(-1)   # row-major for the CSC interface
    x = orc.syncfree_csc(cp, rt.astype(np.int32), vt, bm, rhs).reshape(n, rhs).T.reshape(-1)
    ref = golden[tag + "/base"]
    assert np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-12)) <= 1e-10


def test_oracle_against_live_reference(orc):
    R = orc.ref()
    if R is None:
        pytest.skip("reference core.cpp not built here (no reference checkout)")
    from sptrsv_gb300 import gen
    m = gen.random_upper(20_000, 6.0, 0.85, 48, 21)
    rp = m.row_ptr.astype(np.uint64)
    b = gen.uniform(4, m.n * 2)
    x_ref = np.zeros(m.n * 2)
    R.ref_base_gauss_upper(m.n, m.val, rp, m.col, x_ref, b.copy(), 2)
    x = orc.base_gauss_upper(rp, m.col, m.val, b, 2)
    assert np.max(np.abs(x - x_ref) / np.maximum(np.abs(x_ref), 1e-300)) <= 1e-13
    lv = np.zeros(m.n, dtype=np.uint64)
    ml = R.ref_set_levels(m.n, m.col, rp, lv)
    lv2, ml2 = orc.levels(rp, m.col)
    assert ml == ml2 and np.array_equal(lv, lv2)


@pytest.mark.parametrize("tag", ["csr_6_lower", "lower3000"])
def test_base_gauss_lower_matches_reference(golden, orc, tag):
    rp, col, val = golden[tag + "/row_ptr"].astype(np.uint64), golden[tag + "/col"], golden[tag + "/val"]
    x = orc.base_gauss_lower(rp, col, val, golden[tag + "/b"])
    ref = golden[tag + "/lower"]
    assert np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)) <= 1e-13
