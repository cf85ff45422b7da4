"""The upstream step on the GPU: sptrsv_factor_multifrontal (factor.cu), the multifrontal Cholesky
A = U^T U of the nested-dissection 3D Laplacian, against the host generator's factor of the same
matrix and fronts (gen.laplace3d_nd_cholesky: numpy/scipy dense fronts).  The pattern, row pointer
and supernode partition must match exactly; the values to 1e-12 of the largest entry (the same
FP64 arithmetic in another order).  The GPU factor then solves A x = b through the library (U^T y
= b as the reversed upper solve, U x = y on the supernodal panels), checked against A itself.
Statuses: a matrix that is not positive definite, and a front tree that is not a postorder."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sps

import sptrsv_gb300 as sp
from sptrsv_gb300 import _lib, gen

pytestmark = pytest.mark.gpu


def _same_factor(a, b):
    assert np.array_equal(a.row_ptr, b.row_ptr)
    assert np.array_equal(a.col, b.col)
    assert np.array_equal(a.snodes, b.snodes)
    assert np.max(np.abs(a.val - b.val)) <= 1e-12 * np.max(np.abs(b.val))


@pytest.mark.parametrize("g,leaf,width", [(6, 2, 400), (12, 4, 400), (16, 8, 48)])
def test_factor_matches_host_generator(g, leaf, width):
    _same_factor(gen.laplace3d_nd_cholesky_gpu(g, leaf, width), gen.laplace3d_nd_cholesky(g, leaf, width))


def test_factor_solves_A():
    g = 14
    U = gen.laplace3d_nd_cholesky_gpu(g, 4)
    rp, col, val, _, _, _ = gen.laplace3d_nd_matrix(g, 4)
    n = U.n
    Au = sps.csr_matrix((val, col, rp), shape=(n, n))
    A = (Au + Au.T - sps.diags(Au.diagonal())).tocsr()
    b = gen.uniform(5, n)
    with sp.Solver(0) as s:
        s.analyse(U.row_ptr, U.col, U.val).set_supernodes(U.snodes)
        # U^T y = b: the library's lower solve (the reference's base_gauss_lower, core.cpp:4-16)
        Ut = sps.csr_matrix((U.val, U.col, U.row_ptr), shape=(n, n)).T.tocsr()
        Ut.sort_indices()
        y = np.zeros(n)
        sp.base_gauss_lower(n, Ut.data.copy(), Ut.indptr.astype(np.uint64), Ut.indices.astype(np.int32), y, b.copy())
        x = s.solve(y, schedule="supernodal")
    assert np.linalg.norm(A @ x - b) <= 1e-12 * np.linalg.norm(b)


def test_factor_rejects_indefinite_and_bad_trees():
    rp, col, val, fs, fp, _ = gen.laplace3d_nd_matrix(6, 2)
    L = _lib.lib()
    h = ctypes.c_void_p()
    bad = val.copy()
    bad[rp[100]] = -6.0  # a negative diagonal: not positive definite
    rc = L.sptrsv_factor_multifrontal(0, len(rp) - 1, rp, col, bad, len(fs) - 1, fs, fp, 400, ctypes.byref(h))
    assert rc == -8 and not h.value, sp.status_string(rc)
    fp2 = fp.copy()
    fp2[1] = 0  # a parent before its child: not a postorder
    rc = L.sptrsv_factor_multifrontal(0, len(rp) - 1, rp, col, val, len(fs) - 1, fs, fp2, 400, ctypes.byref(h))
    assert rc == -2 and not h.value, sp.status_string(rc)


def _factor_dense(A, fs, fp, width=400):
    """The library's factor of the dense SPD matrix A (passed as full symmetric CSR) under the
    fronts fs / parents fp, returned as a dense upper U, with its partition."""
    As = sps.csr_matrix(A)
    As.sort_indices()
    L = _lib.lib()
    h = ctypes.c_void_p()
    fs = np.asarray(fs, dtype=np.int32)
    fp = np.asarray(fp, dtype=np.int32)
    rc = L.sptrsv_factor_multifrontal(0, A.shape[0], As.indptr.astype(np.int64), As.indices.astype(np.int32),
                                      As.data.astype(np.float64), len(fs) - 1, fs, fp, width, ctypes.byref(h))
    assert rc == 0, sp.status_string(rc)
    try:
        n, nnz, nsn = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int()
        L.sptrsv_factor_info(h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(nsn))
        rp = np.empty(n.value + 1, dtype=np.int64)
        cl = np.empty(nnz.value, dtype=np.int32)
        vl = np.empty(nnz.value, dtype=np.float64)
        sn = np.empty(nsn.value + 1, dtype=np.int32)
        L.sptrsv_factor_copy(h, rp, cl, vl, sn)
        t_sym, t_num = ctypes.c_double(-1.0), ctypes.c_double(-1.0)
        assert L.sptrsv_factor_times(h, ctypes.byref(t_sym), ctypes.byref(t_num)) == 0
        assert t_sym.value >= 0.0 and t_num.value > 0.0
    finally:
        L.sptrsv_factor_free(h)
    return sps.csr_matrix((vl, cl, rp), shape=(n.value, n.value)).toarray(), sn


def _check_dense(A, fs, fp, width=400):
    U, _ = _factor_dense(A, fs, fp, width)
    ref = np.linalg.cholesky(A).T  # the unique upper factor with a positive diagonal
    assert np.max(np.abs(U - ref)) <= 1e-12 * np.max(np.abs(ref))


def _tridiag(n, d=4.0):
    return np.diag(np.full(n, d)) - np.diag(np.ones(n - 1), 1) - np.diag(np.ones(n - 1), -1)


def test_factor_chain_of_fronts():
    # 25 fronts of 8 rows, each the parent of the one before: 25 levels of one front each, the
    # arena regions alternating
    n = 200
    _check_dense(_tridiag(n), np.arange(0, n + 1, 8), [t + 1 for t in range(24)] + [-1])


def test_factor_forest():
    # two independent chains: two roots
    A = np.zeros((208, 208))
    A[:104, :104] = _tridiag(104)
    A[104:, 104:] = _tridiag(104, 5.0)
    fs = np.arange(0, 209, 8)
    fp = [t + 1 for t in range(12)] + [-1] + [t + 1 for t in range(13, 25)] + [-1]
    _check_dense(A, fs, fp)


def test_factor_front_with_three_children_and_wide_panels():
    # three leaves of 70 rows (two panels each, the second 6 wide) under one root of 150 rows
    # (three panels): three extend-add launches into the root, coupling to every root row
    rng = np.random.default_rng(4)
    n = 3 * 70 + 150
    A = np.zeros((n, n))
    for k in range(3):
        s = slice(70 * k, 70 * (k + 1))
        A[s, s] = _tridiag(70, 6.0)
    for i in range(210):
        for j in rng.choice(150, size=5, replace=False):
            A[i, 210 + j] = A[210 + j, i] = rng.uniform(-0.3, 0.3)
    R = rng.uniform(-0.05, 0.05, size=(150, 150))
    A[210:, 210:] = (R + R.T) / 2
    A += np.diag(np.sum(np.abs(A), axis=1) + 1.0)
    _check_dense(A, [0, 70, 140, 210, n], [3, 3, 3, -1], width=64)


def test_factor_rejects_a_root_with_an_update():
    # the second chain's rows couple to the first, whose root takes no parent: its update would
    # go nowhere
    A = _tridiag(64)
    L = _lib.lib()
    As = sps.csr_matrix(A)
    h = ctypes.c_void_p()
    fs = np.array([0, 32, 64], dtype=np.int32)
    fp = np.array([-1, -1], dtype=np.int32)
    rc = L.sptrsv_factor_multifrontal(0, 64, As.indptr.astype(np.int64), As.indices.astype(np.int32),
                                      As.data.astype(np.float64), 2, fs, fp, 400, ctypes.byref(h))
    assert rc == -2 and not h.value, sp.status_string(rc)


def test_factor_device_arrays_feed_the_solver():
    # U straight from the factor's device arrays (sptrsv_factor_device -> sptrsv_analyse_device)
    # solves exactly as the host copy analysed from host memory
    rp, col, val, fs, fp, _ = gen.laplace3d_nd_matrix(14, 4)
    L = _lib.lib()
    h = ctypes.c_void_p()
    assert L.sptrsv_factor_multifrontal(0, len(rp) - 1, rp, col, val, len(fs) - 1, fs, fp, 400, ctypes.byref(h)) == 0
    try:
        n, nnz, nsn = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int()
        L.sptrsv_factor_info(h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(nsn))
        urp = np.empty(n.value + 1, dtype=np.int64)
        ucol = np.empty(nnz.value, dtype=np.int32)
        uval = np.empty(nnz.value, dtype=np.float64)
        usn = np.empty(nsn.value + 1, dtype=np.int32)
        assert L.sptrsv_factor_copy(h, urp, ucol, uval, usn) == 0
        d_rp, d_col, d_val = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        assert L.sptrsv_factor_device(h, ctypes.byref(d_rp), ctypes.byref(d_col), ctypes.byref(d_val)) == 0
        b = gen.uniform(11, n.value)
        with sp.Solver(0) as s_host, sp.Solver(0) as s_dev:
            s_host.analyse(urp, ucol, uval).set_supernodes(usn)
            s_dev.analyse_device(n.value, int(nnz.value), d_rp, d_col, d_val).set_supernodes(usn)
            x_host = s_host.solve(b, schedule="supernodal")
            x_dev = s_dev.solve(b, schedule="supernodal")
        assert np.array_equal(x_host, x_dev)
        Um = sps.csr_matrix((uval, ucol, urp), shape=(n.value, n.value))
        assert np.linalg.norm(Um @ x_dev - b) <= 1e-12 * np.linalg.norm(b)
    finally:
        L.sptrsv_factor_free(h)


def _scaled_spd(n, seed, spread=20):
    """A dense SPD matrix D S D: S random and diagonally dominant, D powers of two in
    2^-spread .. 2^spread (U(D S D) = U(S) D, so every column of U keeps S's relative accuracy)."""
    rng = np.random.default_rng(seed)
    R = rng.uniform(-1, 1, (n, n))
    S = (R + R.T) / 2
    S += np.diag(np.sum(np.abs(S), axis=1) + 1.0)
    d = np.ldexp(1.0, rng.integers(-spread, spread + 1, n))
    return S, d


@pytest.mark.parametrize("update", ["tc", "fp64"])
def test_factor_wide_trailing_updates(update, monkeypatch):
    # a 100-pivot front (panels of 64 and 36 columns) over a 600-row root: 600 and 536 rows below
    # the panels, the tensor-core update's range (and its K padding), with rows scaled over 40 binades
    if update == "fp64":
        monkeypatch.setenv("SPTRSV_FACTOR_UPDATE", "fp64")
    S, d = _scaled_spd(700, 8)
    A = S * d[:, None] * d[None, :]
    U, _ = _factor_dense(A, [0, 100, 700], [1, -1])
    Us = np.linalg.cholesky(S).T
    assert np.max(np.abs(U / d[None, :] - Us)) <= 1e-12 * np.max(np.abs(Us))


def test_factor_update_forms_agree(monkeypatch):
    # the 24^3 nested-dissection factor by both trailing-update forms, and against the host factor
    tc_form = gen.laplace3d_nd_cholesky_gpu(24)
    monkeypatch.setenv("SPTRSV_FACTOR_UPDATE", "fp64")
    fp64_form = gen.laplace3d_nd_cholesky_gpu(24)
    monkeypatch.delenv("SPTRSV_FACTOR_UPDATE")
    host = gen.laplace3d_nd_cholesky(24)
    _same_factor(tc_form, host)
    _same_factor(fp64_form, host)
    assert np.max(np.abs(tc_form.val - fp64_form.val)) <= 1e-13 * np.max(np.abs(host.val))
