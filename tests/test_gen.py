"""Generators: the shapes, counts and determinism the measured workloads depend on."""
import hashlib

import numpy as np

from sptrsv_gb300 import gen


def _upper_ok(m):
    rp = m.row_ptr
    assert rp[0] == 0 and np.all(np.diff(rp) >= 1)
    rows = np.repeat(np.arange(m.n), np.diff(rp))
    first = rp[:-1]
    assert np.all(m.col[first] == np.arange(m.n))
    off = np.ones(m.nnz, dtype=bool)
    off[first] = False
    assert np.all(m.col[off] > rows[off]) and np.all(m.col < m.n)


def test_laplace_band_factor():
    m = gen.laplace2d_cholesky(64)
    assert m.n == 4096 and m.nnz == 4096 * 65 - 64 * 65 // 2 == 264160
    _upper_ok(m)
    # U^T U reproduces the Laplacian on a small grid
    g = 6
    s = gen.laplace2d_cholesky(g)
    U = np.zeros((s.n, s.n))
    for i in range(s.n):
        U[i, s.col[s.row_ptr[i]:s.row_ptr[i + 1]]] = s.val[s.row_ptr[i]:s.row_ptr[i + 1]]
    A = U.T @ U
    T = 4 * np.eye(g) - np.eye(g, k=1) - np.eye(g, k=-1)
    L = np.kron(np.eye(g), T) - np.kron(np.eye(g, k=1) + np.eye(g, k=-1), np.eye(g))
    assert np.allclose(A, L, atol=1e-12)


def test_random_upper_shape_and_determinism():
    a = gen.random_upper(50_000, 8.0, 0.9, 64, 1)
    b = gen.random_upper(50_000, 8.0, 0.9, 64, 1)
    _upper_ok(a)
    assert np.array_equal(a.col, b.col) and np.array_equal(a.val, b.val)
    mean_off = a.nnz / a.n - 1
    assert 7.0 < mean_off < 8.2
    rows = np.repeat(np.arange(a.n), np.diff(a.row_ptr))
    off = a.col != rows
    near = np.mean((a.col[off] - rows[off]) <= 64)
    assert 0.88 < near < 0.95
    d = a.val[a.row_ptr[:-1]]
    offsum = np.add.reduceat(np.abs(a.val), a.row_ptr[:-1]) - d
    assert np.allclose(d, 1 + offsum)
    # the x86 and Arm hosts must build the same matrix: pin a digest
    h = hashlib.sha256(a.col.tobytes() + a.val.tobytes()).hexdigest()
    assert h == hashlib.sha256(b.col.tobytes() + b.val.tobytes()).hexdigest()


def test_supernodal_random_structure():
    m = gen.supernodal_random(2000, 2, 20, 6.0, 0.8, 64, 5)
    _upper_ok(m)
    sn = m.snodes
    assert sn[0] == 0 and sn[-1] == m.n and np.all(np.diff(sn) >= 1)
    for s in range(len(sn) - 1):
        a, b = sn[s], sn[s + 1]
        tails = [tuple(m.col[m.row_ptr[i] + (b - i):m.row_ptr[i + 1]]) for i in range(a, b)]
        assert all(t == tails[0] for t in tails)
        for i in range(a, b):
            assert list(m.col[m.row_ptr[i]:m.row_ptr[i] + (b - i)]) == list(range(i, b))
