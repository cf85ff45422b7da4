"""GPU parity of the supernodal path: dense supernode panels [T^-1 | -T^-1 Rect] solved sync-free,
in FP64 on CUDA cores and as BF16x3 tensor-core products inside the FP64 refinement, against the
reference's supernodal solve (golden.npz) and the serial oracle."""
import numpy as np
import pytest

import sptrsv_gb300 as sp
from sptrsv_gb300 import gen

pytestmark = pytest.mark.gpu

ELEM_TOL = 1e-10
RES_TOL = 1e-12
MIXED_ELEM_TOL = 1e-8


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


@pytest.fixture(scope="module")
def nd12():
    return gen.laplace3d_nd_cholesky(12)


@pytest.mark.parametrize("tag", ["csr_6_upper", "snr800"])
def test_supernodal_fp64_matches_reference(golden, orc, solver, tag):
    rp = golden[tag + "/row_ptr"].astype(np.int64)
    col, val, sn = golden[tag + "/col"], golden[tag + "/val"], golden[tag + "/snodes"]
    n = len(rp) - 1
    b = golden[tag + "/b"] if tag + "/b" in golden else np.ones(n * 2)
    solver.analyse(rp, col, val).set_supernodes(sn)
    x = solver.solve(b, rhs=2, schedule="supernodal")
    assert elem_err(x, golden[tag + "/super"]) <= ELEM_TOL
    x = solver.solve(b, rhs=2, precision="mixed", schedule="supernodal", max_refine=20)
    assert solver.last_refine()[1] <= RES_TOL
    assert elem_err(x, golden[tag + "/super"]) <= MIXED_ELEM_TOL


@pytest.mark.parametrize("rhs", [1, 8, 33])
@pytest.mark.parametrize("layout", [sp.COL_MAJOR, sp.ROW_MAJOR])
def test_nested_dissection_factor(orc, solver, nd12, rhs, layout):
    m = nd12
    solver.analyse(m.row_ptr, m.col, m.val).set_supernodes(m.snodes)
    b_cm = gen.uniform(70 + rhs, m.n * rhs)
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b_cm, rhs)
    b = b_cm if layout == sp.COL_MAJOR else b_cm.reshape(rhs, m.n).T.copy().reshape(-1)
    for prec in ("fp64", "mixed"):
        x = solver.solve(b, rhs=rhs, layout=layout, schedule="supernodal", precision=prec, max_refine=20)
        if layout == sp.ROW_MAJOR:
            x = x.reshape(m.n, rhs).T.reshape(-1)
        if prec == "fp64":
            assert elem_err(x, ref) <= ELEM_TOL
        else:
            assert solver.last_refine()[1] <= RES_TOL
            assert elem_err(x, ref) <= MIXED_ELEM_TOL
        assert orc.rel_residual(m.row_ptr.astype(np.uint64), m.col, m.val, x, b_cm, rhs) <= 2 * RES_TOL


def test_auto_picks_supernodal_and_wide_supernodes_split(orc, solver):
    m = gen.laplace3d_nd_cholesky(16, max_width=4096)  # fronts wider than the 256-row chunk
    assert int(np.max(np.diff(m.snodes))) > 256
    solver.analyse(m.row_ptr, m.col, m.val).set_supernodes(m.snodes)
    b = gen.uniform(91, m.n)
    x = solver.solve(b)
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b, 1)
    assert elem_err(x, ref) <= ELEM_TOL


def test_partition_without_shared_rectangle_is_rejected(solver):
    m = gen.random_upper(4000, 6.0, 0.9, 64, 5)
    solver.analyse(m.row_ptr, m.col, m.val)
    with pytest.raises(sp.SptrsvError) as e:
        solver.set_supernodes(np.array([0, 10, 4000], dtype=np.int32))
    assert e.value.status == -14
    with pytest.raises(sp.SptrsvError) as e:
        solver.set_supernodes(np.array([0, 10, 3999], dtype=np.int32))
    assert e.value.status == -14


@pytest.mark.parametrize("width", [16, 64, 300])
@pytest.mark.parametrize("rhs", [1, 8])
def test_band_factor_skyline_panels(orc, solver, width, rhs):
    """A banded factor stored with its explicit zeros, cut into uniform row chunks: every row is a
    contiguous range from its diagonal (skyline), so each chunk is a dense panel whose rectangle
    is the longest row's reach; shorter rows read zero there."""
    m = gen.laplace2d_cholesky(30)
    sn = np.unique(np.append(np.arange(0, m.n, width), m.n)).astype(np.int32)
    solver.analyse(m.row_ptr, m.col, m.val).set_supernodes(sn)
    b = gen.uniform(17 + rhs, m.n * rhs)
    ref = orc.base_gauss_upper(m.row_ptr.astype(np.uint64), m.col, m.val, b, rhs)
    x = solver.solve(b, rhs=rhs, schedule="supernodal")
    assert elem_err(x, ref) <= ELEM_TOL
    x = solver.solve(b, rhs=rhs, schedule="supernodal", precision="mixed", max_refine=20)
    assert solver.last_refine()[1] <= RES_TOL
    assert elem_err(x, ref) <= MIXED_ELEM_TOL


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_graph_replay_after_work_buffers_grow(orc, solver, nd12, prec):
    """The same device b and x solved at 1, then 8, then 1 right-hand side: the 8-column solve
    grows the handle's work buffers, and the second 1-column solve must not replay a graph
    captured with their old addresses."""
    import ctypes
    m = nd12
    L = sp._lib.lib()
    solver.analyse(m.row_ptr, m.col, m.val).set_supernodes(m.snodes)
    rpu = m.row_ptr.astype(np.uint64)
    nb = 8 * m.n * 8
    d_b, d_x = ctypes.c_void_p(), ctypes.c_void_p()
    assert L.sptrsv_device_alloc(solver.handle, nb, ctypes.byref(d_b)) == 0
    assert L.sptrsv_device_alloc(solver.handle, nb, ctypes.byref(d_x)) == 0
    o = sp.make_opts(schedule="supernodal", precision=prec, max_refine=20)
    try:
        for rhs in (1, 8, 1):
            b = gen.uniform(300 + rhs, m.n * rhs)
            L.sptrsv_copy_h2d(solver.handle, d_b, b.ctypes.data, 8 * m.n * rhs)
            solver.solve_device(d_b, d_x, rhs=rhs, opts=o)
            x = np.empty(m.n * rhs)
            L.sptrsv_copy_d2h(solver.handle, x.ctypes.data, d_x, 8 * m.n * rhs)
            assert solver.sync() == 0
            ref = orc.base_gauss_upper(rpu, m.col, m.val, b, rhs)
            assert elem_err(x, ref) <= (ELEM_TOL if prec == "fp64" else MIXED_ELEM_TOL)
    finally:
        L.sptrsv_device_free(solver.handle, d_b)
        L.sptrsv_device_free(solver.handle, d_x)
