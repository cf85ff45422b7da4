"""GPU tests of the exhaustive autotuner and the selector's matrix features, through the C ABI.

The autotuner times every applicable candidate of its table on the resident matrix; every
candidate that finishes must reach the accuracy contract (checked here on the pick: FP64
candidates elementwise <= 1e-10 against the serial oracle, mixed ones at residual <= 1e-12),
and AUTO must use the cached pick afterwards."""
import math

import numpy as np
import pytest

import sptrsv_gb300 as sp
from sptrsv_gb300 import gen

pytestmark = pytest.mark.gpu

ELEM_TOL = 1e-10
MIXED_ELEM_TOL = 1e-8
RES_TOL = 1e-12


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


def _check_pick(orc, solver, m, best, rhs):
    """FP64 picks: elementwise <= 1e-10 against the serial solve.  Mixed picks are specified by
    their residual (<= 1e-12); their forward error follows the conditioning, so it is checked
    normwise and elementwise on components above 1e-3 of the largest."""
    b = gen.uniform(41 + rhs, m.n * rhs)
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b, rhs)
    x = solver.solve(b, rhs=rhs)  # AUTO -> the tuned pick
    o = sp.candidate(best)
    if o.precision == 1:
        assert solver.last_refine()[1] <= RES_TOL
        assert np.linalg.norm(x - ref) / np.linalg.norm(ref) <= 1e-9
        big = np.abs(ref) >= 1e-3 * np.max(np.abs(ref))
        assert np.max(np.abs(x - ref)[big] / np.abs(ref)[big]) <= MIXED_ELEM_TOL
    else:
        assert elem_err(x, ref) <= ELEM_TOL


@pytest.mark.parametrize("rhs", [1, 4])
def test_autotune_random(orc, solver, rhs):
    m = gen.random_upper(30_000, 8.0, 0.9, 64, 11)
    solver.analyse(m.row_ptr, m.col, m.val)
    best, ms = solver.autotune(rhs=rhs, cap_ms=20.0, reps=1)
    assert 0 <= best < sp.N_CANDIDATES
    for k in range(sp.N_CANDIDATES):
        if solver.applicable(k, rhs):
            assert math.isfinite(ms[k]) and ms[k] > 0, k
        else:
            assert math.isinf(ms[k]), k
    assert ms[best] == np.min(ms)
    _check_pick(orc, solver, m, best, rhs)


def test_autotune_band_with_supernodes(orc, solver):
    m = gen.laplace2d_cholesky(40)
    sn = np.arange(0, m.n + 1, 40, dtype=np.int32)
    if sn[-1] != m.n:
        sn = np.append(sn, m.n).astype(np.int32)
    solver.analyse(m.row_ptr, m.col, m.val).set_supernodes(sn)
    best, ms = solver.autotune(rhs=8, cap_ms=20.0, reps=1)
    assert solver.applicable(11, 8) and math.isfinite(ms[11])  # FP64 supernodal ran
    assert not solver.applicable(0, 8)  # the block kernel is single-RHS only
    assert math.isinf(ms[0])
    _check_pick(orc, solver, m, best, 8)


def test_features(solver):
    m = gen.random_upper(10_000, 6.0, 0.9, 64, 3)
    solver.analyse(m.row_ptr, m.col, m.val)
    f = solver.features()
    assert f.shape == (sp.N_FEATURES,) and np.all(np.isfinite(f))
    assert abs(f[0] - math.log2(m.n)) < 1e-5 and abs(f[1] - math.log2(m.nnz)) < 1e-5
    info = solver.info()
    assert abs(f[4] - math.log2(info["max_level"])) < 1e-5
    assert abs(float(np.sum(f[8:16])) - 1.0) < 1e-5  # level-width histogram sums to 1
    assert f[7] == 1.0  # the generator's rows are diagonally dominant


def test_bounded_autotune_cancels_slow_candidates_and_stays_usable(orc, solver):
    """A deep chain-heavy system: the FP64 sync-free candidates run for many milliseconds, so with
    a small abort bound they are cancelled from the host (abort flag), reported as censored, and
    the handle solves correctly afterwards."""
    m = gen.random_upper(1_000_000, 8.0, 0.9, 64, 21)
    solver.analyse(m.row_ptr, m.col, m.val)
    best, ms, cens = solver.autotune(rhs=8, cap_ms=5.0, reps=1, abort_ms=2.0, with_censored=True)
    assert cens.sum() >= 1
    assert cens[best] == 0 and math.isfinite(ms[best])
    for k in range(sp.N_CANDIDATES):
        if cens[k]:
            assert ms[k] >= 2.0
    _check_pick(orc, solver, m, best, 8)
    x = solver.solve(gen.uniform(5, m.n), schedule="syncfree_warp")  # a plain FP64 solve after cancels
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, gen.uniform(5, m.n), 1)
    assert elem_err(x, ref) <= ELEM_TOL
