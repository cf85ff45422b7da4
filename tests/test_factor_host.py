"""Host-side checks of the multifrontal factor's entry points (csrc/factor.cu), without a GPU:
every input the symbolic step rejects returns its status before any CUDA call, and the accessors
reject a null factor.  The numeric step and its results are tested on the GPU
(tests/test_gpu_factor.py)."""
import ctypes

import numpy as np
import scipy.sparse as sps

from sptrsv_gb300 import _lib, gen

INVALID_ARG, ROW_PTR, COL_RANGE = -2, -4, -7


def _call(rp, col, val, fs, fp, width=400):
    L = _lib.lib()
    h = ctypes.c_void_p()
    rc = L.sptrsv_factor_multifrontal(0, len(rp) - 1, np.ascontiguousarray(rp, dtype=np.int64),
                                      np.ascontiguousarray(col, dtype=np.int32),
                                      np.ascontiguousarray(val, dtype=np.float64), len(fs) - 1,
                                      np.ascontiguousarray(fs, dtype=np.int32),
                                      np.ascontiguousarray(fp, dtype=np.int32), width, ctypes.byref(h))
    assert not h.value  # nothing is handed back on a rejection
    return rc


def _nd6():
    return gen.laplace3d_nd_matrix(6, 2)


def test_rejects_a_tree_that_is_not_a_postorder():
    rp, col, val, fs, fp, _ = _nd6()
    fp = fp.copy()
    fp[1] = 0  # a parent before its child
    assert _call(rp, col, val, fs, fp) == INVALID_ARG
    fp[1] = len(fs) - 1  # a parent past the last front
    assert _call(rp, col, val, fs, fp) == INVALID_ARG


def test_rejects_fronts_that_do_not_tile_the_rows():
    rp, col, val, fs, fp, _ = _nd6()
    short = fs.copy()
    short[-1] -= 1  # the last row belongs to no front
    assert _call(rp, col, val, short, fp) == INVALID_ARG
    empty = fs.copy()
    empty[1] = empty[0]  # a front without pivots
    assert _call(rp, col, val, empty, fp) == INVALID_ARG


def test_rejects_bad_row_pointers_and_columns():
    rp, col, val, fs, fp, _ = _nd6()
    bad = rp.copy()
    bad[5], bad[6] = bad[6], bad[5]  # not monotone
    assert _call(bad, col, val, fs, fp) == ROW_PTR
    shifted = rp + 1  # does not start at 0
    assert _call(shifted, np.concatenate([[0], col]), np.concatenate([[1.0], val]), fs, fp) == ROW_PTR
    far = col.copy()
    far[3] = len(rp) - 1  # column n
    assert _call(rp, far, val, fs, fp) == COL_RANGE


def test_rejects_updates_that_no_ancestor_takes():
    # two sibling leaves coupled to each other: leaf 0's update reaches a row of leaf 1, which is
    # not its ancestor (the parent's pivots start after it)
    n = 30
    A = np.diag(np.full(n, 4.0))
    for i in range(n - 1):
        if i not in (9, 19):
            A[i, i + 1] = A[i + 1, i] = -1.0
    for i in range(10):
        A[i, 20 + i] = A[20 + i, i] = -0.5
        A[10 + i, 20 + i] = A[20 + i, 10 + i] = -0.5
    A[5, 15] = A[15, 5] = -0.5
    As = sps.csr_matrix(A)
    assert _call(As.indptr, As.indices, As.data, [0, 10, 20, 30], [2, 2, -1]) == INVALID_ARG
    # a root whose rows couple to a later root: its update has no parent
    T = sps.csr_matrix(np.diag(np.full(8, 4.0)) - np.diag(np.ones(7), 1) - np.diag(np.ones(7), -1))
    assert _call(T.indptr, T.indices, T.data, [0, 4, 8], [-1, -1]) == INVALID_ARG


def test_rejects_null_and_empty_arguments():
    L = _lib.lib()
    rp, col, val, fs, fp, _ = _nd6()
    assert L.sptrsv_factor_multifrontal(0, len(rp) - 1, rp, col, val, len(fs) - 1, fs, fp, 400, None) == INVALID_ARG
    assert _call(rp, col, val, fs, fp, width=0) == INVALID_ARG
    assert _call(rp[:1], col[:0], val[:0], np.array([0, 0]), np.array([-1])) == INVALID_ARG  # n = 0


def test_accessors_reject_a_null_factor():
    L = _lib.lib()
    n, nnz, nsn = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int()
    assert L.sptrsv_factor_info(None, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(nsn)) == INVALID_ARG
    d = ctypes.c_void_p()
    assert L.sptrsv_factor_device(None, ctypes.byref(d), ctypes.byref(d), ctypes.byref(d)) == INVALID_ARG
    t = ctypes.c_double()
    assert L.sptrsv_factor_times(None, ctypes.byref(t), ctypes.byref(t)) == INVALID_ARG
    L.sptrsv_factor_free(None)  # a no-op
