"""CPU checks of the selector's FP64 MLP oracle: its gradient against central finite differences
(the mathematics it restates), and the selector's pure host logic."""
import numpy as np

from oracle import mlp_oracle as mo


def _data(rng, n, dims):
    X = rng.normal(size=(n, dims[0]))
    Y = rng.normal(size=(n, dims[3]))
    M = (rng.random((n, dims[3])) < 0.7).astype(np.float64)
    return X, Y, M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    dims = (5, 7, 6, 4)
    n_par = sum(int(np.prod(s)) for _, s in mo.sizes(dims))
    p = rng.normal(scale=0.5, size=n_par)
    X, Y, M = _data(rng, 9, dims)
    mean, scale = X.mean(0), 1.0 / X.std(0)
    loss, g = mo.loss_grad(p, dims, X, Y, M, mean, scale)
    h = 1e-6
    fd = np.empty_like(p)
    for k in range(n_par):
        e = np.zeros_like(p)
        e[k] = h
        fd[k] = (mo.loss_grad(p + e, dims, X, Y, M, mean, scale)[0] - mo.loss_grad(p - e, dims, X, Y, M, mean, scale)[0]) / (2 * h)
    assert np.max(np.abs(fd - g)) <= 1e-6 * max(1.0, np.max(np.abs(g)))
    assert loss > 0


def test_pack_unpack_roundtrip():
    dims = (24, 64, 64, 16)
    n_par = sum(int(np.prod(s)) for _, s in mo.sizes(dims))
    assert n_par == 24 * 64 + 64 + 64 * 64 + 64 + 16 * 64 + 16
    p = np.arange(n_par, dtype=np.float64)
    assert np.array_equal(mo.pack(mo.unpack(p, dims), dims), p)


def test_selector_host_logic():
    from sptrsv_gb300 import selector as sel
    T = np.array([[1.0, 2.0, np.inf], [3.0, 1.0, 0.5], [2.0, 2.0, 1.0]], dtype=np.float32)
    Y, M = sel.targets(T)
    assert M.tolist() == [[1, 1, 0], [1, 1, 1], [1, 1, 1]]
    assert abs(Y[1, 2] - np.log(0.5)) < 1e-6
    assert sel.fixed_default(T) == 0 or sel.fixed_default(T) == 1  # candidate 2 failed once
    A = np.array([[1, 1, 0], [1, 1, 1], [0, 1, 1]])
    pred = np.array([[0.1, 0.0, -5.0], [0.0, 1.0, 2.0], [0.0, 1.0, 0.5]])
    assert sel.pick(pred, A).tolist() == [1, 0, 2]
    specs = sel.sample_specs(9, 3)
    assert [s["kind"] for s in specs] == [0, 1, 2] * 3
    assert all(1 <= s["rhs"] <= 16 for s in specs)
    assert specs == sel.sample_specs(9, 3)
