"""The alternative panel products of the exact FP64 schedules, selected with sptrsv_set_panels_mode:
the tensor cores ("tc": tcgen05 with TMEM accumulators over BF16 digit slices; panels_tc.cu) and
double-FP32 on the FP32 pipes ("df": scaled FP32 pairs, error-free products, compensated sums;
panels64.cu), each against the serial FP64 oracle: the single-system supernodal
solve on the reference's golden supernode case and on a 12^3 nested-dissection factor at 1, 8 and
33 right-hand sides in both layouts, and the batched exact FP64 panels.

Bounds: relative residual <= 1e-12; the term-relative error (against the size of the terms each
component is summed from, oracle.term_rel_error) <= 1e-12, as for every FP64 form; elementwise error
<= max(1e-10, 10 x the reordering floor measured on the same inputs) for the tensor cores (56-bit
digit products).  Double-FP32 pairs carry 48 bits, a unit roundoff 32 times FP64's, so tiny
solution components see that much more error: max(1e-9, 100 x the floor)."""
import numpy as np
import pytest

import sptrsv_gb300 as sp
from sptrsv_gb300 import gen

pytestmark = pytest.mark.gpu


def elem_err(x, ref):
    x = np.asarray(x).reshape(-1)
    ref = np.asarray(ref).reshape(-1)
    scale = max(np.max(np.abs(ref)), 1e-300)
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-12 * scale)))


@pytest.fixture(params=["tc", "df"])
def tc_mode(request):
    prev = sp.set_panels_mode(request.param)
    yield request.param
    sp.set_panels_mode(prev)


ELEM_BOUND = {"tc": (1e-10, 10.0), "df": (1e-9, 100.0)}  # (minimum, factor on the reordering floor)


def _check(orc, rp, col, val, b, rhs, x, mode):
    rpu = np.asarray(rp, dtype=np.uint64)
    ref = orc.base_gauss_upper(rpu, col, val, b, rhs)
    floor = elem_err(orc.base_gauss_upper_rev(rpu, col, val, b, rhs), ref)
    assert orc.rel_residual(rpu, col, val, x, b, rhs) <= 1e-12
    assert orc.term_rel_error(rpu, col, val, ref, x, b, rhs) <= 1e-12
    lo, fac = ELEM_BOUND[mode]
    assert elem_err(x, ref) <= max(lo, fac * floor)


def test_tc_panels_golden(golden, orc, tc_mode):
    tag = "snr800"
    rp = golden[tag + "/row_ptr"].astype(np.int64)
    col, val, sn = golden[tag + "/col"], golden[tag + "/val"], golden[tag + "/snodes"]
    b = golden[tag + "/b"]
    with sp.Solver(0) as s:
        s.analyse(rp, col, val).set_supernodes(sn)
        x = s.solve(b, rhs=2, schedule="supernodal")
    assert elem_err(x, golden[tag + "/super"]) <= ELEM_BOUND[tc_mode][0]
    _check(orc, rp, col, val, b, 2, x, tc_mode)


@pytest.mark.parametrize("rhs", [1, 8, 33])
@pytest.mark.parametrize("layout", [sp.COL_MAJOR, sp.ROW_MAJOR])
def test_tc_panels_nested_dissection(orc, tc_mode, rhs, layout):
    m = gen.laplace3d_nd_cholesky(12)
    b_cm = gen.uniform(170 + rhs, m.n * rhs)
    with sp.Solver(0) as s:
        s.analyse(m.row_ptr, m.col, m.val).set_supernodes(m.snodes)
        if layout == sp.COL_MAJOR:
            x = s.solve(b_cm, rhs=rhs, layout=layout, schedule="supernodal")
        else:
            xr = s.solve(b_cm.reshape(rhs, m.n).T.copy().reshape(-1), rhs=rhs, layout=layout, schedule="supernodal")
            x = xr.reshape(m.n, rhs).T.reshape(-1)
    _check(orc, m.row_ptr, m.col, m.val, b_cm, rhs, x, tc_mode)


def test_tc_panels_batch(orc, tc_mode):
    M = gen.mix(count=12, seed=31, nmin=500, nmax=6000, rhs_max=16)
    items = []
    for s in range(M.count):
        m, _, b = M.system(s)
        items.append((gen.Csr(np.array(m.row_ptr), np.array(m.col), np.array(m.val)), int(M.rhs[s]), np.array(b)))
    n = np.array([m.n for m, _, _ in items], dtype=np.int32)
    rhs = np.array([r for _, r, _ in items], dtype=np.int32)
    bb = np.concatenate([b.reshape(-1) for _, _, b in items])
    with sp.Batch(n, rhs, np.concatenate([m.row_ptr for m, _, _ in items]).astype(np.int64),
                  np.concatenate([m.col for m, _, _ in items]), np.concatenate([m.val for m, _, _ in items])) as B:
        sched = B.schedule.copy()
        sched[0::2] = sp.BATCH_SCHED["panel64"]  # the banded systems on the exact panels
        B.schedule = sched
        x = B.solve(bb, mode="chosen")
        assert np.all(B.stats()["status"] == 0)
        parts = B.split(x)
    M.close()
    for s in range(0, len(items), 2):
        m, r, b = items[s]
        cm = lambda a: np.ascontiguousarray(np.asarray(a).reshape(m.n, r).T).reshape(-1)
        _check(orc, m.row_ptr, m.col, m.val, cm(b), r, cm(parts[s]), tc_mode)
