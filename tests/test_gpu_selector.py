"""GPU tests of the learned schedule selector: the MLP's forward, backward and Adam kernels against
the FP64 oracle (oracle/mlp_oracle.py), and what the trained network gains over the method
without it (a fixed default schedule) on held-out matrices, judged by the exhaustive autotuner's
timings (the committed GB300 timing dataset)."""
import os

import numpy as np
import pytest

from oracle import mlp_oracle as mo
from sptrsv_gb300 import selector as sel

pytestmark = pytest.mark.gpu

DIMS = sel.DIMS


def _data(seed, n):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, DIMS[0])).astype(np.float32)
    Y = rng.normal(size=(n, DIMS[3])).astype(np.float32)
    M = (rng.random((n, DIMS[3])) < 0.8).astype(np.float32)
    return X, Y, M


def test_forward_matches_oracle():
    m = sel.Mlp(seed=3)
    X, _, _ = _data(1, 37)
    m.fit_norm(X)
    P = m.predict(X)
    _, _, _, Po = mo.forward(m.params.astype(np.float64), DIMS, X, m.mean.astype(np.float64),
                             m.scale.astype(np.float64))
    assert np.max(np.abs(P - Po)) <= 1e-4 * max(1.0, np.max(np.abs(Po)))


@pytest.mark.parametrize("n", [1, 17, 300])
def test_gradient_matches_oracle(n):
    m = sel.Mlp(seed=5)
    X, Y, M = _data(2 + n, n)
    m.fit_norm(X) if n > 1 else m.set_norm(np.zeros(DIMS[0]), np.ones(DIMS[0]))
    loss, g = m.grad(X, Y, M)
    lo, go = mo.loss_grad(m.params.astype(np.float64), DIMS, X, Y, M, m.mean.astype(np.float64),
                          m.scale.astype(np.float64))
    assert abs(loss - lo) <= 1e-4 * max(1.0, abs(lo))
    # FP32 kernels against FP64: relative to the gradient's scale
    assert np.max(np.abs(g - go)) <= 2e-4 * max(1e-3, np.max(np.abs(go)))


def test_adam_step_matches_oracle():
    m = sel.Mlp(seed=9)
    X, Y, M = _data(4, 64)
    m.fit_norm(X)
    p0 = m.params.astype(np.float64)
    _, go = mo.loss_grad(p0, DIMS, X, Y, M, m.mean.astype(np.float64), m.scale.astype(np.float64))
    m.train(X, Y, M, epochs=1, batch=64, lr=1e-2, seed=0)  # one full-batch step
    p1, _, _ = mo.adam_step(p0, go, np.zeros_like(p0), np.zeros_like(p0), 1, 1e-2)
    assert np.max(np.abs(m.params - p1)) <= 1e-4


def test_training_fits_a_known_function():
    rng = np.random.default_rng(0)
    X = rng.normal(size=(512, DIMS[0])).astype(np.float32)
    W = rng.normal(size=(DIMS[0], DIMS[3])).astype(np.float32) / 5
    Y = np.tanh(X @ W).astype(np.float32)
    M = np.ones_like(Y)
    m = sel.Mlp(seed=1)
    m.fit_norm(X)
    losses = m.train(X, Y, M, epochs=200, batch=64, lr=3e-3, seed=1)
    assert losses[-1] < 0.1 * losses[0]
    assert m.launches() > 200 * 8 * 10


@pytest.mark.skipif(not os.path.exists(sel.DATA), reason="no timing dataset")
def test_selector_beats_fixed_default_on_held_out():
    d = sel.load_dataset()
    n = len(d["X"])
    held = max(20, min(200, n // 10))
    tr, te = sel.split(n, held)
    mlp, losses = sel.train(d["X"][tr], d["T"][tr], epochs=300)
    assert losses[-1] < losses[0]
    rep = sel.evaluate(mlp, d["X"][te], d["T"][te], d["A"][te], sel.fixed_default(d["T"][tr]))
    print("selector held-out:", rep)
    assert rep["speedup_vs_default_geomean"] > 1.0
    assert rep["geomean_regret"] < rep["default_geomean_regret"]
