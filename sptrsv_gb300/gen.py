"""Seeded synthetic systems (front end of libsptrsv_gen.so; see csrc/gen.cpp for the exact
recipes and the random-number transforms).

Workloads:
* ``laplace2d_cholesky(g)``: exact upper Cholesky factor of the 5-point Laplacian on a g x g
  grid, natural ordering, full band (bandwidth g).  g = 64 is the plain FP64 single-RHS case
  (n = 4,096, nnz = 264,160).
* ``random_upper(n, mean, p_near, band, seed)``: Poisson(mean) off-diagonals per row, each at
  i + U{1..band} with probability p_near else U{i+1..n-1}, values U[-1,1], diagonal
  1 + sum |off|.  n = 2,000,000, mean 8, p_near 0.9, band 64, seed 1 is the large irregular
  case.
* ``supernodal_random``: random U with true supernode structure (dense triangles + shared
  rectangle columns), with its partition.
"""
import ctypes

import numpy as np

from . import _lib


class Csr:
    def __init__(self, row_ptr, col, val, snodes=None):
        self.row_ptr = row_ptr   # int64[n+1]
        self.col = col           # int32[nnz]
        self.val = val           # float64[nnz]
        self.snodes = snodes     # int32[sn+1] or None
        self.n = len(row_ptr) - 1
        self.nnz = int(row_ptr[-1])

    @property
    def row_ptr_u64(self):
        return self.row_ptr.astype(np.uint64)


def _take(h):
    G = _lib.gen()
    if not h:
        raise ValueError("generator rejected its arguments")
    try:
        n, nnz = G.sptrsv_gen_n(h), G.sptrsv_gen_nnz(h)
        rp = np.empty(n + 1, dtype=np.int64)
        col = np.empty(nnz, dtype=np.int32)
        val = np.empty(nnz, dtype=np.float64)
        G.sptrsv_gen_copy(h, rp, col, val)
    finally:
        G.sptrsv_gen_free(h)
    return Csr(rp, col, val)


def laplace2d_cholesky(g):
    return _take(_lib.gen().sptrsv_gen_laplace2d_cholesky(int(g)))


def random_upper(n, mean=8.0, p_near=0.9, band=64, seed=1):
    return _take(_lib.gen().sptrsv_gen_random_upper(int(n), float(mean), float(p_near), int(band), int(seed)))


def supernodal_random(n, wmin=1, wmax=16, mean_rect=6.0, p_near=0.8, band=64, seed=3):
    G = _lib.gen()
    sp = ctypes.POINTER(ctypes.c_int)()
    sn = ctypes.c_int()
    h = G.sptrsv_gen_supernodal_random(int(n), int(wmin), int(wmax), float(mean_rect), float(p_near), int(band),
                                       int(seed), ctypes.byref(sp), ctypes.byref(sn))
    m = _take(h)
    m.snodes = np.ctypeslib.as_array(sp, shape=(sn.value + 1,)).astype(np.int32).copy()
    G.sptrsv_gen_free_ints(ctypes.cast(sp, ctypes.c_void_p))
    return m


def uniform(seed, count, lo=-1.0, hi=1.0):
    out = np.empty(int(count), dtype=np.float64)
    _lib.gen().sptrsv_gen_uniform(int(seed), int(count), float(lo), float(hi), out)
    return out


def spmv(m, x, rhs=1):
    """b = U x (FP64, column-major RHS)."""
    b = np.empty(m.n * rhs, dtype=np.float64)
    _lib.gen().sptrsv_gen_spmv(m.n, m.row_ptr, m.col, m.val, np.ascontiguousarray(x, dtype=np.float64).reshape(-1), b,
                               rhs)
    return b


XSTAR_SALT = 0x9E3779B97F4A7C15


def system(m, seed, rhs=1):
    """x* ~ U[-1,1] from mt19937_64(seed + XSTAR_SALT mod 2^64), b = U x*."""
    xs = uniform((int(seed) + XSTAR_SALT) % (1 << 64), m.n * rhs)
    return xs, spmv(m, xs, rhs)


def band_laplace_case():
    """The plain FP64 single-RHS case: g = 64 Laplacian factor, x* seed 0."""
    m = laplace2d_cholesky(64)
    xs, b = system(m, 0)
    return m, xs, b


def irregular_case(n=2_000_000, seed=1):
    """The large irregular single-RHS case (n = 2M, Poisson(8), p_near 0.9, band 64, seed 1)."""
    m = random_upper(n, 8.0, 0.9, 64, seed)
    xs, b = system(m, seed)
    return m, xs, b
