"""ctypes front end of the CPU oracle (oracle.c) and, when built, of the reference's own
core.cpp (oracle/_ref/libref_core.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference legs.  The product package never imports this module.

Array conventions follow the reference: CSR with uint64 row_index and the diagonal first
in each row (core.h:10), X/B column-major (core.cpp:26-28).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_core.so")

_P = np.ctypeslib.ndpointer
_f64 = _P(dtype=np.float64, flags="C_CONTIGUOUS")
_u64 = _P(dtype=np.uint64, flags="C_CONTIGUOUS")
_i32 = _P(dtype=np.int32, flags="C_CONTIGUOUS")
_c_int, _c_dbl, _c_sz = ctypes.c_int, ctypes.c_double, ctypes.c_size_t


def build(force=False):
    """Compile oracle.c into liboracle.so (gcc, OpenMP) and, when the reference checkout
    is present, the reference's core.cpp into _ref/ (build_ref.sh)."""
    src = os.path.join(HERE, "oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-fopenmp", "-shared", "-o", LIB_PATH, src, "-lm"])
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")], stdout=subprocess.DEVNULL)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_base_gauss_upper.argtypes = [_c_int, _f64, _u64, _i32, _f64, _f64, _c_int]
        L.orc_base_gauss_upper_new.argtypes = [_c_int, _f64, _u64, _i32, _f64, _f64, _c_int]
        L.orc_base_gauss_upper_rev.argtypes = [_c_int, _f64, _u64, _i32, _f64, _f64, _c_int]
        L.orc_term_rel_error.argtypes = [_c_int, _f64, _u64, _i32, _f64, _f64, _f64, _c_int]
        L.orc_term_rel_error.restype = _c_dbl
        L.orc_base_gauss_lower.argtypes = [_c_int, _f64, _u64, _i32, _f64, _f64]
        L.orc_set_levels.argtypes = [_c_int, _i32, _u64, _u64]
        L.orc_set_levels.restype = _c_int
        L.orc_level_buckets.argtypes = [_c_int, _u64, _c_int, _i32, _i32]
        L.orc_level_tasks.argtypes = [_c_int, _i32, _i32, _u64, _c_int, _i32]
        L.orc_barrier_solve.argtypes = [_c_int, _f64, _f64, _f64, _i32, _u64, _c_int, _i32, _i32, _i32,
                                        _c_int, _c_int, _c_int]
        L.orc_in_degree_csc.argtypes = [_c_int, _c_int, _i32, _i32]
        L.orc_transpose.argtypes = [_c_int, ctypes.c_uint64, _f64, _i32, _u64, _f64, _u64, _i32]
        L.orc_syncfree_csc.argtypes = [_c_int, _i32, _i32, _f64, _f64, _f64, _c_int]
        L.orc_supernodal_upper.argtypes = [_c_sz, _i32, _f64, _f64, _i32, _u64, _c_int, _c_int]
        L.orc_supernodal_upper_new.argtypes = [_c_sz, _i32, _f64, _f64, _i32, _u64, _c_int, _c_int]
        L.orc_ccs2ccs_pad.argtypes = [_f64, _i32, _u64, _f64, _u64, _i32, _i32, _c_int]
        L.orc_ccs2ccs_pad.restype = _c_int
        L.orc_supernodal_blas_upper.argtypes = [_c_int, _c_sz, _i32, _f64, _f64, _u64, _i32, _c_int]
        L.orc_supernodal_blas_upper_cblas.argtypes = [_c_int, _c_sz, _i32, _f64, _f64, _u64, _i32, _c_int,
                                                      ctypes.c_void_p, ctypes.c_void_p]
        L.orc_rel_error.argtypes = [_c_sz, _f64, _f64]
        L.orc_rel_error.restype = _c_dbl
        L.orc_rel_residual.argtypes = [_c_int, _f64, _u64, _i32, _f64, _f64, _c_int]
        L.orc_rel_residual.restype = _c_dbl
        L.orc_max_threads.restype = _c_int
        _lib = L
    return _lib


def ref():
    """The reference's core.cpp built unmodified, or None where it was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = ctypes.CDLL(REF_PATH)
        for name in ("ref_base_gauss_upper", "ref_base_gauss_upper_new"):
            getattr(R, name).argtypes = [_c_int, _f64, _u64, _i32, _f64, _f64, _c_int]
            getattr(R, name).restype = _c_dbl
        if hasattr(R, "ref_base_gauss_lower"):
            R.ref_base_gauss_lower.argtypes = [_c_int, _f64, _u64, _i32, _f64, _f64]
            R.ref_base_gauss_lower.restype = _c_dbl
        for name in ("ref_supernodal_upper", "ref_supernodal_upper_new"):
            getattr(R, name).argtypes = [_c_sz, _i32, _f64, _f64, _i32, _u64, _c_int, _c_int]
            getattr(R, name).restype = _c_dbl
        R.ref_supernodal_blas_upper.argtypes = [_c_int, _c_int, _c_sz, _i32, _f64, _f64, _u64, _i32, _c_int]
        R.ref_supernodal_blas_upper.restype = _c_dbl
        R.ref_ccs2ccs_pad.argtypes = [_f64, _i32, _u64, _f64, _u64, _i32, _i32, _c_int]
        R.ref_ccs2ccs_pad.restype = _c_int
        R.ref_set_levels.argtypes = [_c_int, _i32, _u64, _u64]
        R.ref_set_levels.restype = _c_int
        for name in ("ref_barrier_upper", "ref_barrier_upper_new"):
            getattr(R, name).argtypes = [_c_int, _f64, _f64, _f64, _i32, _u64, _c_int, _c_int]
            getattr(R, name).restype = _c_dbl
        _ref = R
    return _ref


# ----------------------------------------------------------------------------------------
# numpy-level helpers (all return new arrays; inputs are CSR with uint64 row pointers)

def _csr(row_ptr, col, val):
    return (np.ascontiguousarray(row_ptr, dtype=np.uint64), np.ascontiguousarray(col, dtype=np.int32),
            np.ascontiguousarray(val, dtype=np.float64))


def base_gauss_upper(row_ptr, col, val, b, rhs=1, new=False):
    rp, c, v = _csr(row_ptr, col, val)
    n = len(rp) - 1
    b = np.ascontiguousarray(b, dtype=np.float64).reshape(-1)
    x = np.zeros(n * rhs)
    (lib().orc_base_gauss_upper_new if new else lib().orc_base_gauss_upper)(n, v, rp, c, x, b, rhs)
    return x


def base_gauss_upper_rev(row_ptr, col, val, b, rhs=1):
    """The serial solve with every row sum in the opposite order (not a reference routine): the
    distance between it and base_gauss_upper is the reordering floor of a system."""
    rp, c, v = _csr(row_ptr, col, val)
    n = len(rp) - 1
    b = np.ascontiguousarray(b, dtype=np.float64).reshape(-1)
    x = np.zeros(n * rhs)
    lib().orc_base_gauss_upper_rev(n, v, rp, c, x, b, rhs)
    return x


def term_rel_error(row_ptr, col, val, x_ref, x, b, rhs=1):
    """max_i |x_i - x_ref_i| / max(|x_ref_i|, (|b_i| + sum_j |U_ij x_ref_j|) / |U_ii|)."""
    rp, c, v = _csr(row_ptr, col, val)
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    return lib().orc_term_rel_error(len(rp) - 1, v, rp, c, f(x_ref), f(x), f(b), rhs)


def base_gauss_lower(row_ptr, col, val, b):
    """Forward substitution (core.cpp:4-16): lower CSR, diagonal last in every row, one RHS."""
    rp, c, v = _csr(row_ptr, col, val)
    n = len(rp) - 1
    x = np.zeros(n)
    lib().orc_base_gauss_lower(n, v, rp, c, x, np.ascontiguousarray(b, dtype=np.float64).reshape(-1))
    return x


def levels(row_ptr, col):
    rp = np.ascontiguousarray(row_ptr, dtype=np.uint64)
    n = len(rp) - 1
    lv = np.zeros(n, dtype=np.uint64)
    m = lib().orc_set_levels(n, np.ascontiguousarray(col, dtype=np.int32), rp, lv)
    return lv, m


def level_buckets(lv, max_level):
    n = len(lv)
    ptr = np.zeros(max_level + 2, dtype=np.int32)
    rows = np.zeros(max(n, 1), dtype=np.int32)
    lib().orc_level_buckets(n, np.ascontiguousarray(lv, dtype=np.uint64), max_level, ptr, rows)
    return ptr, rows[:n]


def level_tasks(max_level, level_ptr, level_rows, row_ptr, num_threads):
    tasks = np.zeros((max_level + 1) * (num_threads + 1), dtype=np.int32)
    rows = np.ascontiguousarray(level_rows, dtype=np.int32)
    if rows.size == 0:
        rows = np.zeros(1, dtype=np.int32)
    lib().orc_level_tasks(max_level, np.ascontiguousarray(level_ptr, dtype=np.int32), rows,
                          np.ascontiguousarray(row_ptr, dtype=np.uint64), num_threads, tasks)
    return tasks.reshape(max_level + 1, num_threads + 1)


def barrier_upper(row_ptr, col, val, b, rhs=1, num_threads=1, new=False):
    rp, c, v = _csr(row_ptr, col, val)
    n = len(rp) - 1
    lv, m = levels(rp, c)
    ptr, rows = level_buckets(lv, m)
    tasks = level_tasks(m, ptr, rows, rp, num_threads)
    x = np.zeros(n * rhs)
    lib().orc_barrier_solve(n, x, np.ascontiguousarray(b, dtype=np.float64).reshape(-1), v, c, rp, m, ptr,
                            rows, np.ascontiguousarray(tasks.reshape(-1)), num_threads, rhs, 1 if new else 0)
    return x


def in_degree_csc(n, csc_row_idx):
    out = np.zeros(n, dtype=np.int32)
    lib().orc_in_degree_csc(n, len(csc_row_idx), np.ascontiguousarray(csc_row_idx, dtype=np.int32), out)
    return out


def transpose(row_ptr, col, val):
    """utils.cpp:128-159: returns (col_ptr int32[n+1], row_idx uint64[nnz], val_t)."""
    rp, c, v = _csr(row_ptr, col, val)
    n = len(rp) - 1
    nz = int(rp[-1])
    vt = np.zeros(nz)
    rt = np.zeros(nz, dtype=np.uint64)
    ct = np.zeros(n + 1, dtype=np.int32)
    lib().orc_transpose(n, nz, v, c, rp, vt, rt, ct)
    return ct, rt, vt


def syncfree_csc(col_ptr, row_idx, val, b, rhs=1):
    n = len(col_ptr) - 1
    x = np.zeros(n * rhs)
    lib().orc_syncfree_csc(n, np.ascontiguousarray(col_ptr, dtype=np.int32),
                           np.ascontiguousarray(row_idx, dtype=np.int32),
                           np.ascontiguousarray(val, dtype=np.float64), x,
                           np.ascontiguousarray(b, dtype=np.float64).reshape(-1), rhs)
    return x


def supernodal_upper(supernodes, row_ptr, col, val, b, rhs=1, new=False):
    rp, c, v = _csr(row_ptr, col, val)
    n = len(rp) - 1
    sn = np.ascontiguousarray(supernodes, dtype=np.int32)
    x = np.array(np.ascontiguousarray(b, dtype=np.float64).reshape(-1), copy=True)
    f = lib().orc_supernodal_upper_new if new else lib().orc_supernodal_upper
    f(len(sn) - 1, sn, x, v, c, rp, n, rhs)
    return x


def ccs2ccs_pad(supernodes, row_ptr, col, val):
    """core.cpp:136-161: returns (rowptr_pad int32[n+1], colidx_pad uint64, val_pad)."""
    rp, c, v = _csr(row_ptr, col, val)
    n = len(rp) - 1
    sn = np.ascontiguousarray(supernodes, dtype=np.int32)
    widths = np.diff(sn).astype(np.int64)
    extra = int(np.sum(widths * (widths - 1) // 2))
    total = int(rp[-1]) + extra
    vp = np.zeros(max(total, 1))
    cp = np.zeros(max(total, 1), dtype=np.uint64)
    rpp = np.zeros(n + 1, dtype=np.int32)
    nz = lib().orc_ccs2ccs_pad(v, c, rp, vp, cp, rpp, sn, len(sn) - 1)
    return rpp, cp[:nz], vp[:nz]


def supernodal_blas_upper(supernodes, rowptr_pad, colidx_pad, val_pad, b, rhs=1):
    n = len(rowptr_pad) - 1
    sn = np.ascontiguousarray(supernodes, dtype=np.int32)
    x = np.array(np.ascontiguousarray(b, dtype=np.float64).reshape(-1), copy=True)
    lib().orc_supernodal_blas_upper(n, len(sn) - 1, sn, x, np.ascontiguousarray(val_pad, dtype=np.float64),
                                    np.ascontiguousarray(colidx_pad, dtype=np.uint64),
                                    np.ascontiguousarray(rowptr_pad, dtype=np.int32), rhs)
    return x


_cblas = None


def cblas64():
    """(library path, dgemm address, dtrsm address) of the ILP64 CBLAS that numpy bundles (its
    OpenBLAS, symbols scipy_cblas_dgemm64_ / scipy_cblas_dtrsm64_), or None where it is absent."""
    global _cblas
    if _cblas is None:
        import glob
        _cblas = False
        d = os.path.join(os.path.dirname(np.__file__), "..", "numpy.libs")
        for path in sorted(glob.glob(os.path.join(d, "libscipy_openblas64_*.so"))):
            try:
                B = ctypes.CDLL(path)
                g = ctypes.cast(B.scipy_cblas_dgemm64_, ctypes.c_void_p).value
                t = ctypes.cast(B.scipy_cblas_dtrsm64_, ctypes.c_void_p).value
                _cblas = (os.path.abspath(path), g, t, B)
                break
            except (OSError, AttributeError):
                continue
    return _cblas[:3] if _cblas else None


def supernodal_blas_upper_openblas(supernodes, rowptr_pad, colidx_pad, val_pad, b, rhs=1):
    """core.cpp:164-201 with its dgemm / dtrsm on numpy's OpenBLAS (all the threads OpenBLAS is
    given); None when that library is not present."""
    cb = cblas64()
    if cb is None:
        return None
    sn = np.ascontiguousarray(supernodes, dtype=np.int32)
    n = int(sn[-1])
    x = np.ascontiguousarray(b, dtype=np.float64).reshape(-1).copy()
    lib().orc_supernodal_blas_upper_cblas(n, len(sn) - 1, sn, x, np.ascontiguousarray(val_pad, dtype=np.float64),
                                          np.ascontiguousarray(colidx_pad, dtype=np.uint64),
                                          np.ascontiguousarray(rowptr_pad, dtype=np.int32), rhs, cb[1], cb[2])
    return x


def rel_error(x_ref, x):
    a = np.ascontiguousarray(x_ref, dtype=np.float64).reshape(-1)
    return lib().orc_rel_error(a.size, a, np.ascontiguousarray(x, dtype=np.float64).reshape(-1))


def rel_residual(row_ptr, col, val, x, b, rhs=1):
    rp, c, v = _csr(row_ptr, col, val)
    return lib().orc_rel_residual(len(rp) - 1, v, rp, c, np.ascontiguousarray(x, dtype=np.float64).reshape(-1),
                                  np.ascontiguousarray(b, dtype=np.float64).reshape(-1), rhs)


def max_elem_rel_error(x_ref, x, floor=1e-300):
    """max_i |x_i - x_ref_i| / max(|x_ref_i|, floor)."""
    a = np.asarray(x_ref, dtype=np.float64).reshape(-1)
    d = np.abs(np.asarray(x, dtype=np.float64).reshape(-1) - a)
    return float(np.max(d / np.maximum(np.abs(a), floor))) if a.size else 0.0


def read_txt_csr(path):
    """The reference's .txt matrix layout (utils.cpp:61-76): n nnz / val[nnz] / col[nnz] /
    row_index[n+1]."""
    tok = open(path).read().split()
    n, nz = int(tok[0]), int(tok[1])
    vals = np.array([float(t) for t in tok[2:2 + nz]])
    cols = np.array([int(t) for t in tok[2 + nz:2 + 2 * nz]], dtype=np.int32)
    rp = np.array([int(t) for t in tok[2 + 2 * nz:2 + 2 * nz + n + 1]], dtype=np.uint64)
    return rp, cols, vals


def read_txt_snodes(path):
    """The reference's .txt supernode layout (utils.cpp:99-105): sn / nodes[sn+1]."""
    tok = open(path).read().split()
    sn = int(tok[0])
    return np.array([int(t) for t in tok[1:sn + 2]], dtype=np.int32)
