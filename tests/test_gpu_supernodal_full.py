"""Parity at the full supernodal workload: the exact upper Cholesky factor of the 7-point 3D
Laplacian on a 40^3 grid under nested dissection (n = 64,000, 24.7M entries, 1,028 supernode
chunks), B uniform on [-1, 1] with m = 1, 8, 32 and 128 columns, against the serial FP64 solve
of the oracle (core.cpp:18-32).

Two elementwise measures are checked, as the oracle states them:
  * plain: max_i |x_i - ref_i| / max(|ref_i|, 1e-12 ||ref||_inf).  On this system two correct FP64
    solves that differ only in summation order (the oracle against itself with every row summed
    in reverse) already lie 1.9e-11 / 2.1e-10 / 1.9e-10 / 5.9e-9 apart at 1 / 8 / 32 / 128
    columns, because some of the 64,000 m solution components are tiny (down to 8e-9 at 128
    columns).  The bound is therefore max(1e-10, 10 x that measured floor), with the floor
    measured in the test on the same inputs;
  * term-relative: max_i |x_i - ref_i| / max(|ref_i|, (|b_i| + sum_j |U_ij ref_j|) / |U_ii|), the
    error against the size of the terms component i is computed from.  The reordering floor is
    ~1e-14 there; the FP64 forms must stay within 1e-12, the mixed one within 1e-10.
The relative residual ||B - U X||_F / ||B||_F must be <= 1e-12 for every form.  The FP64 panel
products run both on FP64 FMAs and in double-FP32 on the FP32 pipes (panel mode "df")."""
import numpy as np
import pytest

import sptrsv_gb300 as sp
from sptrsv_gb300 import gen

pytestmark = pytest.mark.gpu

RES_TOL = 1e-12
ELEM_TOL = 1e-10
TERM_TOL = {"fp64": 1e-12, "mixed": 1e-10}
FLOOR_FACTOR = 10.0


def elem_err(x, ref):
    x = np.asarray(x).reshape(-1)
    ref = np.asarray(ref).reshape(-1)
    scale = max(np.max(np.abs(ref)), 1e-300)
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-12 * scale)))


@pytest.fixture(scope="module")
def nd40():
    return gen.laplace3d_nd_cholesky(40)


@pytest.fixture(scope="module")
def solver(nd40):
    s = sp.Solver(0)
    s.analyse(nd40.row_ptr, nd40.col, nd40.val)
    yield s
    s.close()


FORMS = {
    # FP64 on the supernode panels [T^-1 | -T^-1 Rect] (the partition is set for these)
    "fp64_panels": dict(schedule="supernodal", precision="fp64"),
    # the same products in double-FP32 on the FP32 pipes (panel mode "df")
    "df_panels": dict(schedule="supernodal", precision="fp64"),
    # BF16x3 tensor-core panels inside the FP64 refinement
    "mixed_panels": dict(schedule="supernodal", precision="mixed", max_refine=20),
    # the plain FP64 sync-free forms, no partition: one column at a time
    "fp64_block": dict(schedule="syncfree_block", precision="fp64"),
    "fp64_window": dict(schedule="syncfree_window", precision="fp64"),
}


@pytest.mark.parametrize("rhs", [1, 8, 32, 128])
def test_nd40_full(orc, nd40, solver, rhs):
    m = nd40
    rpu = m.row_ptr.astype(np.uint64)
    b = gen.uniform(900 + rhs, m.n * rhs)  # column-major n x rhs, uniform on [-1, 1]
    ref = orc.base_gauss_upper(rpu, m.col, m.val, b, rhs)
    floor = elem_err(orc.base_gauss_upper_rev(rpu, m.col, m.val, b, rhs), ref)
    bound = max(ELEM_TOL, FLOOR_FACTOR * floor)
    report = {"floor": floor}
    for name, opts in FORMS.items():
        if name.endswith("panels"):
            prev = sp.set_panels_mode("df" if name == "df_panels" else "fp64")
            try:
                solver.set_supernodes(m.snodes)
            finally:
                sp.set_panels_mode(prev)
        else:
            solver.analyse(m.row_ptr, m.col, m.val)  # no partition: the plain sync-free kernels
        x = solver.solve(b, rhs=rhs, **opts)
        prec = opts["precision"]
        res = orc.rel_residual(rpu, m.col, m.val, x, b, rhs)
        err = elem_err(x, ref)
        term = orc.term_rel_error(rpu, m.col, m.val, ref, x, b, rhs)
        report[name] = (err, term, res)
        assert res <= RES_TOL, (name, report)
        assert term <= TERM_TOL[prec], (name, report)
        if name == "df_panels":  # 48-bit pairs: a unit roundoff 32 times FP64's
            assert err <= max(1e-9, 100 * floor), (name, report)
        else:
            assert err <= (bound if prec == "fp64" else max(1e-8, FLOOR_FACTOR * floor)), (name, report)
    print("nd40 rhs=%d" % rhs, report)


def test_nd40_gpu_factor_matches(nd40):
    """The full workload's factor from the GPU multifrontal Cholesky (sptrsv_factor_multifrontal)
    against the host generator's: same pattern and partition, values to 1e-12 of the largest."""
    f = gen.laplace3d_nd_cholesky_gpu(40)
    assert np.array_equal(f.row_ptr, nd40.row_ptr) and np.array_equal(f.col, nd40.col)
    assert np.array_equal(f.snodes, nd40.snodes)
    assert np.max(np.abs(f.val - nd40.val)) <= 1e-12 * np.max(np.abs(nd40.val))

