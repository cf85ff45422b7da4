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
