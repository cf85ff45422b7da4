"""sptrsv_gb300 -- GPU sparse upper-triangular solver for the GB300 (sm_103a).

Python front end of libsptrsv_gb300.so.  Two layers, both straight onto the C ABI:

* the reference's interface (xnd-r/SPTRSV include/core.h:10-19 and
  include/sptrsv_syncfree_opencl.h:11-37): the same function names, argument order and
  meaning, on numpy arrays, returning elapsed seconds (negative status on failure);
* ``Solver``: a handle that keeps one matrix and its analysis on the device and solves many
  right-hand sides, with every schedule (sync-free warp / thread / CSC push, level-set,
  FP32 + FP64 refinement) selectable.

All numerical work happens in the CUDA kernels; nothing here computes a solution.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import Opts

SCHED = {"auto": 0, "syncfree_warp": 1, "syncfree_thread": 2, "syncfree_csc": 3, "levelset": 4, "jacobi": 5,
         "supernodal": 6, "syncfree_block": 7, "syncfree_window": 8}
PREC = {"fp64": 0, "mixed": 1}
COL_MAJOR, ROW_MAJOR = 0, 1


class SptrsvError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = _lib.lib().sptrsv_status_string(status).decode()
        super().__init__(f"{what}: status {status} ({msg})" if what else f"status {status} ({msg})")


def _check(rc, what=""):
    if rc != 0:
        raise SptrsvError(rc, what)


def status_string(s):
    return _lib.lib().sptrsv_status_string(int(s)).decode()


def last_status():
    return _lib.lib().sptrsv_last_status()


def make_opts(schedule="auto", precision="fp64", rows_per_warp=None, rhs_tile=None, inner="auto", inner_sweeps=None,
              max_refine=None, tol=None, spin_budget_ns=None, resident_warps=None, inner_tol_exp=None):
    """struct sptrsv_opts from sptrsv_default_opts, with the given fields replaced."""
    o = Opts()
    _lib.lib().sptrsv_default_opts(ctypes.byref(o))
    o.schedule = SCHED[schedule] if isinstance(schedule, str) else int(schedule)
    o.precision = PREC[precision] if isinstance(precision, str) else int(precision)
    o.inner = SCHED[inner] if isinstance(inner, str) else int(inner)
    for name, v in (("rows_per_warp", rows_per_warp), ("rhs_tile", rhs_tile), ("inner_sweeps", inner_sweeps),
                    ("max_refine", max_refine), ("tol", tol), ("spin_budget_ns", spin_budget_ns),
                    ("resident_warps", resident_warps), ("inner_tol_exp", inner_tol_exp)):
        if v is not None:
            setattr(o, name, v)
    return o


N_CANDIDATES = 16
N_FEATURES = 24


def measure_fp64(device=0):
    """(G FMA/s over every SM, SM cycles per dependent FMA) of the GPU's FP64 pipe, measured."""
    g, c = ctypes.c_double(), ctypes.c_double()
    _check(_lib.lib().sptrsv_measure_fp64(int(device), ctypes.byref(g), ctypes.byref(c)), "measure_fp64")
    return g.value, c.value


def set_panels_mode(mode):
    """Panel products of the exact FP64 schedules: "fp64" (FP64 FMAs), "tc" (tensor cores) or "df"
    (double-FP32 on the FP32 pipes), all FP64-accurate; applies to partitions and batches built
    afterwards; returns the previous mode."""
    rc = _lib.lib().sptrsv_set_panels_mode({"fp64": 0, "tc": 1, "df": 2}[mode])
    if rc < 0:
        raise SptrsvError(rc, "set_panels_mode")
    return ("fp64", "tc", "df")[rc]


def candidate(cand_id):
    """sptrsv_opts of entry `cand_id` of the autotuner's candidate table."""
    o = Opts()
    _check(_lib.lib().sptrsv_candidate(int(cand_id), ctypes.byref(o)), "candidate")
    return o


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


# --------------------------------------------------------------------------------------
# The reference interface (core.h / sptrsv_syncfree_opencl.h).  Arrays are numpy; outputs
# are written into the caller's arrays, as in the reference.

def base_gauss_lower(n, val, row_index, col, x, b):
    """core.h:9 -- x = L^{-1} b, one RHS; CSR (uint64 row_index, diagonal LAST in every row)."""
    return _lib.dropin("base_gauss_lower")(n, val, row_index, col, x, b)


def base_gauss_upper(n, val, row_index, col, x, b, rhs):
    """core.h:10 -- x = U^{-1} b; CSR (uint64 row_index, diagonal first), X/B column-major."""
    return _lib.dropin("base_gauss_upper")(n, val, row_index, col, x, b, rhs)


def base_gauss_upper_new(n, val, row_index, col, x, b, rhs):
    """core.h:11."""
    return _lib.dropin("base_gauss_upper_new")(n, val, row_index, col, x, b, rhs)


def supernodal_upper(sn, supernodes, x, val, row, col_index, n, rhs):
    """core.h:12 -- in place: x holds b on entry.  `row` = CSR columns, `col_index` = uint64 row pointer."""
    return _lib.dropin("supernodal_upper")(sn, supernodes, x, val, row, col_index, n, rhs)


def supernodal_upper_new(sn, supernodes, x, val, row, col_index, n, rhs):
    """core.h:13."""
    return _lib.dropin("supernodal_upper_new")(sn, supernodes, x, val, row, col_index, n, rhs)


def supernodal_blas_upper(n, nz, sn, supernodes, x, val, col_index, row, rhs):
    """core.h:14 -- padded format: val_pad, uint64 padded columns, int padded row pointer."""
    return _lib.dropin("supernodal_blas_upper")(n, nz, sn, supernodes, x, val, col_index, row, rhs)


def supernodal_blas_upper_new(n, nz, sn, supernodes, x, val, col_index, row, rhs):
    """core.h:15."""
    return _lib.dropin("supernodal_blas_upper_new")(n, nz, sn, supernodes, x, val, col_index, row, rhs)


def ccs2ccs_pad(val, row, col_index, val_pad, col_index_pad, row_pad, nodes, sn, nnz):
    """core.h:16 -- `sn` and `nnz` are ctypes.c_int (passed by reference, as int& there)."""
    return _lib.dropin("ccs2ccs_pad")(val, row, col_index, val_pad, col_index_pad, row_pad, nodes,
                                      ctypes.byref(sn), ctypes.byref(nnz))


def setLevelUpAndGetMaxLevel(n, col, row_index, levelsUp):  # noqa: N802 (reference name)
    """core.h:17 -- fills uint64 levelsUp, returns the largest level."""
    return _lib.dropin("setLevelUpAndGetMaxLevel")(n, col, row_index, levelsUp)


def barrier_upper(n, x, b, val, col, row, num_of_threads, rhs):
    """core.h:18 -- level-set solve (the GPU ignores num_of_threads)."""
    return _lib.dropin("barrier_upper")(n, x, b, val, col, row, num_of_threads, rhs)


def barrier_upper_new(n, x, b, val, col, row, num_of_threads, rhs):
    """core.h:19."""
    return _lib.dropin("barrier_upper_new")(n, x, b, val, col, row, num_of_threads, rhs)


def sptrsv_syncfree_opencl(cscColPtr, cscRowIdx, cscVal, m, n, nnz, x, b, rhs):  # noqa: N803
    """sptrsv_syncfree_opencl.h:11-19 -- CSC (diagonal last), X/B row-major."""
    return _lib.dropin("sptrsv_syncfree_opencl")(cscColPtr, cscRowIdx, cscVal, m, n, nnz, x, b, rhs)


def sptrsv_syncfree2_opencl(cscColPtr, cscRowIdx, cscVal, m, n, nnz, x, b):  # noqa: N803
    """sptrsv_syncfree_opencl.h:21-28."""
    return _lib.dropin("sptrsv_syncfree2_opencl")(cscColPtr, cscRowIdx, cscVal, m, n, nnz, x, b)


def sptrsv_syncfree3_opencl(csrColIdx, csrRowPtr, csrVal, m, n, nnz, x, b):  # noqa: N803
    """sptrsv_syncfree_opencl.h:30-37 -- CSR (diagonal first), one lane per row."""
    return _lib.dropin("sptrsv_syncfree3_opencl")(csrColIdx, csrRowPtr, csrVal, m, n, nnz, x, b)


# --------------------------------------------------------------------------------------
class Solver:
    """One device-resident matrix U (CSR, diagonal first) and its analysis."""

    def __init__(self, device=0):
        self._h = ctypes.c_void_p()
        _check(_lib.lib().sptrsv_create(ctypes.byref(self._h), device), "sptrsv_create")
        self.n = 0
        self.nnz = 0

    def close(self):
        if self._h:
            _lib.lib().sptrsv_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def analyse(self, row_ptr, col, val):
        rp = _c(row_ptr, np.int64)
        n = len(rp) - 1
        _check(_lib.lib().sptrsv_analyse_host(self._h, n, int(rp[-1]), rp, _c(col, np.int32), _c(val, np.float64)),
               "analyse")
        self.n, self.nnz = n, int(rp[-1])
        return self

    def analyse_device(self, n, nnz, d_row_ptr, d_col, d_val):
        _check(_lib.lib().sptrsv_analyse_device(self._h, n, nnz, d_row_ptr, d_col, d_val), "analyse_device")
        self.n, self.nnz = n, nnz
        return self

    def set_supernodes(self, supernodes):
        """Supernode partition (sn+1 boundaries); enables the supernodal schedule."""
        sn = _c(supernodes, np.int32)
        _check(_lib.lib().sptrsv_set_supernodes(self._h, len(sn) - 1, sn), "set_supernodes")
        return self

    def autotune(self, rhs=1, cap_ms=50.0, reps=2, abort_ms=0.0, with_censored=False):
        """Exhaustive tuning over the candidate table; returns (best id, times in ms per candidate)
        and, with_censored, the flags of candidates cancelled after abort_ms (their times are lower
        bounds).  The winner is cached for this RHS class and used by schedule="auto"."""
        ms = np.zeros(N_CANDIDATES, dtype=np.float32)
        cens = np.zeros(N_CANDIDATES, dtype=np.int32)
        best = ctypes.c_int(-1)
        _check(_lib.lib().sptrsv_autotune_bounded(self._h, rhs, cap_ms, reps, float(abort_ms), ms, cens,
                                                  ctypes.byref(best), None), "autotune")
        return (best.value, ms, cens) if with_censored else (best.value, ms)

    def features(self, rhs=1):
        f = np.zeros(N_FEATURES, dtype=np.float32)
        _check(_lib.lib().sptrsv_features(self._h, int(rhs), f), "features")
        return f

    def applicable(self, cand_id, rhs=1):
        return bool(_lib.lib().sptrsv_candidate_applicable(self._h, cand_id, rhs))

    def set_tuned(self, cand_id, rhs=1):
        o = candidate(cand_id)
        _check(_lib.lib().sptrsv_set_tuned(self._h, rhs, ctypes.byref(o)), "set_tuned")

    def info(self):
        n, nnz, ml = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(_lib.lib().sptrsv_info(self._h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(ml)), "info")
        return {"n": n.value, "nnz": nnz.value, "max_level": ml.value}

    def levels(self):
        out = np.zeros(self.n, dtype=np.uint64)
        _check(_lib.lib().sptrsv_get_levels(self._h, out), "levels")
        return out

    def in_degree(self):
        out = np.zeros(self.n, dtype=np.int32)
        _check(_lib.lib().sptrsv_get_in_degree(self._h, out), "in_degree")
        return out

    def csc(self):
        """(col_ptr, row_idx, val) of the device CSR -> CSC transpose (utils.cpp:128-159 layout)."""
        info = self.info()
        cp = np.zeros(self.n + 1, dtype=np.int32)
        ri = np.zeros(info["nnz"], dtype=np.int32)
        cv = np.zeros(info["nnz"], dtype=np.float64)
        _check(_lib.lib().sptrsv_get_csc(self._h, cp, ri, cv), "csc")
        return cp, ri, cv

    def level_buckets(self):
        ml = self.info()["max_level"]
        ptr = np.zeros(ml + 2, dtype=np.int32)
        rows = np.zeros(self.n, dtype=np.int32)
        _check(_lib.lib().sptrsv_get_level_buckets(self._h, ptr, rows), "level_buckets")
        return ptr, rows

    def level_tasks(self, num_threads):
        ml = self.info()["max_level"]
        out = np.zeros((ml + 1) * (num_threads + 1), dtype=np.int32)
        _check(_lib.lib().sptrsv_get_level_tasks(self._h, num_threads, out), "level_tasks")
        return out.reshape(ml + 1, num_threads + 1)

    def solve(self, b, rhs=1, layout=COL_MAJOR, **opts):
        """Host B (n*rhs float64) -> host X; raises SptrsvError on any failure."""
        o = make_opts(**opts)
        bb = _c(b, np.float64).reshape(-1)
        x = np.empty(self.n * rhs, dtype=np.float64)
        _check(_lib.lib().sptrsv_solve_host(self._h, ctypes.byref(o), bb.ctypes.data, x.ctypes.data, rhs, layout),
               "solve")
        return x

    def solve_device(self, d_b, d_x, rhs=1, layout=COL_MAJOR, opts=None):
        o = opts if opts is not None else make_opts()
        _check(_lib.lib().sptrsv_solve(self._h, ctypes.byref(o), d_b, d_x, rhs, layout), "solve_device")

    def sync(self):
        return _lib.lib().sptrsv_sync(self._h)

    def last_refine(self):
        """(refinement steps, relative residual) of the last mixed solve."""
        s, w, r = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _lib.lib().sptrsv_last_refine(self._h, ctypes.byref(s), ctypes.byref(w), ctypes.byref(r))
        return s.value, r.value

    def last_sweeps(self):
        """Total inner Jacobi sweeps of the last mixed solve (device-looped graphs)."""
        s, w, r = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _lib.lib().sptrsv_last_refine(self._h, ctypes.byref(s), ctypes.byref(w), ctypes.byref(r))
        return w.value

    def launches(self):
        return _lib.lib().sptrsv_kernel_launches(self._h)

    def sm_count(self):
        return _lib.lib().sptrsv_device_sm_count(self._h)

    def profile(self, enable=True):
        _check(_lib.lib().sptrsv_profile_enable(self._h, 1 if enable else 0), "profile_enable")

    def profile_read(self, cap=4096):
        """[(kind, ms)] of the last profiled solve, in launch order."""
        kinds = np.zeros(cap, dtype=np.int32)
        ms = np.zeros(cap, dtype=np.float32)
        k = _lib.lib().sptrsv_profile_read(self._h, kinds, ms, cap)
        if k < 0:
            raise SptrsvError(k, "profile_read")
        return list(zip(kinds[:k].tolist(), ms[:k].tolist()))



BATCH_SCHED = {"plain": 0, "jacobi": 1, "panel": 2, "sf32": 3, "panel64": 4}
BATCH_MODE = {"plain": 0, "chosen": 1}


class Batch:
    """Independent systems of uneven n and RHS count solved together (sptrsv_batch_* in
    include/sptrsv_gb300.h).  Inputs are the packed host arena: per-system n and rhs, the local
    row pointers one after another (int64), columns and values one after another.  Right-hand
    sides and solutions are row-major n x rhs per system, concatenated.

    mode "plain": every system by the exact FP64 sync-free pull in one persistent launch;
    mode "chosen": each system by its own schedule (``schedule``), the mixed ones inside the FP64
    refinement to ||b - U x||_F <= tol ||b||_F."""

    def __init__(self, n, rhs, row_ptr, col, val, device=0):
        self._h = None
        self.n = np.ascontiguousarray(n, dtype=np.int32)
        self.rhs = np.ascontiguousarray(rhs, dtype=np.int32)
        self.count = len(self.n)
        self.xb_off = np.concatenate([[0], np.cumsum(self.n.astype(np.int64) * self.rhs)]).astype(np.int64)
        h = ctypes.c_void_p()
        _check(_lib.lib().sptrsv_batch_create(ctypes.byref(h), int(device), self.count, self.n, self.rhs,
                                              np.ascontiguousarray(row_ptr, dtype=np.int64),
                                              np.ascontiguousarray(col, dtype=np.int32),
                                              np.ascontiguousarray(val, dtype=np.float64)), "batch_create")
        self._h = h

    @classmethod
    def from_mix(cls, mix, device=0):
        return cls(mix.n, mix.rhs, mix.row_ptr, mix.col, mix.val, device)

    def close(self):
        if self._h:
            _lib.lib().sptrsv_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def schedule(self):
        out = np.zeros(self.count, dtype=np.int32)
        _check(_lib.lib().sptrsv_batch_get_schedule(self._h, out), "batch_get_schedule")
        return out

    @schedule.setter
    def schedule(self, sched):
        a = np.array([BATCH_SCHED[v] if isinstance(v, str) else int(v) for v in sched], dtype=np.int32)
        _check(_lib.lib().sptrsv_batch_set_schedule(self._h, a), "batch_set_schedule")

    def set_options(self, tol=0.0, max_refine=0, inner_tol_exp=0, spin_budget_ns=0):
        _check(_lib.lib().sptrsv_batch_set_options(self._h, float(tol), int(max_refine), int(inner_tol_exp),
                                                   int(spin_budget_ns)), "batch_set_options")

    def info(self):
        t = np.zeros(6, dtype=np.int64)
        r = np.zeros(self.count, dtype=np.float32)
        _check(_lib.lib().sptrsv_batch_info(self._h, t, r), "batch_info")
        return {"rows": int(t[0]), "nnz": int(t[1]), "x_elems": int(t[2]), "count": int(t[3]),
                "g_entries_f64": int(t[4]), "g_fma_f64": int(t[5]), "ratio": r}

    def solve(self, b, mode="chosen"):
        """Host b (all systems) -> host x, through the host-buffer entry point."""
        b = np.ascontiguousarray(b, dtype=np.float64).reshape(-1)
        if b.size != self.xb_off[-1]:
            raise ValueError("b must hold sum n*rhs values")
        x = np.empty_like(b)
        self.solve_host(b.ctypes.data, x.ctypes.data, mode)
        self.sync()
        return x

    def solve_host(self, h_b, h_x, mode="chosen"):
        _check(_lib.lib().sptrsv_batch_solve_host(self._h, BATCH_MODE.get(mode, mode), ctypes.c_void_p(h_b),
                                                  ctypes.c_void_p(h_x)), "batch_solve_host")

    def solve_device(self, d_b, d_x, mode="chosen"):
        _check(_lib.lib().sptrsv_batch_solve(self._h, BATCH_MODE.get(mode, mode), ctypes.c_void_p(d_b),
                                             ctypes.c_void_p(d_x)), "batch_solve")

    def sync(self):
        k = ctypes.c_int64()
        _check(_lib.lib().sptrsv_batch_sync(self._h, ctypes.byref(k)), "batch_sync")
        return k.value

    def stats(self):
        st = np.zeros(self.count, dtype=np.int32)
        steps = np.zeros(self.count, dtype=np.int32)
        rel = np.zeros(self.count, dtype=np.float64)
        sw = np.zeros(self.count, dtype=np.int32)
        _check(_lib.lib().sptrsv_batch_stats(self._h, st, steps, rel, sw), "batch_stats")
        return {"status": st, "steps": steps, "rel": rel, "sweeps": sw}

    def features(self, s):
        f = np.zeros(N_FEATURES, dtype=np.float32)
        _check(_lib.lib().sptrsv_batch_features(self._h, int(s), f), "batch_features")
        return f

    KINDS = ("fill_x", "pull_f64", "state_init", "mixed_init", "step_begin", "fill_d", "panels_bf16x3",
             "pull_f32", "jacobi_sweep", "sweep_check", "axpy", "residual_f64", "step_check", "panels_f64")

    def profile(self, d_b, d_x, mode="chosen"):
        """One host-driven solve with CUDA events around every kernel:
        {kind: (total ms, launches, first launch ms)}."""
        ms = np.zeros(len(self.KINDS), dtype=np.float32)
        cnt = np.zeros(len(self.KINDS), dtype=np.int32)
        first = np.zeros(len(self.KINDS), dtype=np.float32)
        _check(_lib.lib().sptrsv_batch_profile(self._h, BATCH_MODE.get(mode, mode), ctypes.c_void_p(d_b),
                                               ctypes.c_void_p(d_x), ms, cnt, first), "batch_profile")
        return {k: (float(ms[i]), int(cnt[i]), float(first[i])) for i, k in enumerate(self.KINDS) if cnt[i]}

    def timer_begin(self):
        _check(_lib.lib().sptrsv_batch_timer_begin(self._h), "batch_timer")

    def timer_end(self):
        ms = ctypes.c_float()
        _check(_lib.lib().sptrsv_batch_timer_end(self._h, ctypes.byref(ms)), "batch_timer")
        return ms.value

    def launches(self):
        return int(_lib.lib().sptrsv_batch_launches(self._h))

    def split(self, x):
        """Per-system views (n x rhs) of a concatenated solution."""
        return [x[self.xb_off[s]:self.xb_off[s + 1]].reshape(int(self.n[s]), int(self.rhs[s])) for s in range(self.count)]


def read_csr(path):
    """The reference's matrix files (.matrix / .txt / .mtx, utils.cpp:9-80) -> (row_ptr int64,
    col int32, val float64), CSR with the diagonal first."""
    L = _lib.lib()
    n, nnz = ctypes.c_int(), ctypes.c_int64()
    rp, col, val = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    _check(L.sptrsv_read_csr(str(path).encode(), ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(rp),
                             ctypes.byref(col), ctypes.byref(val)), "read_csr")
    try:
        out = (np.ctypeslib.as_array(ctypes.cast(rp, ctypes.POINTER(ctypes.c_int64)), (n.value + 1,)).copy(),
               np.ctypeslib.as_array(ctypes.cast(col, ctypes.POINTER(ctypes.c_int32)), (max(1, nnz.value),))[:nnz.value].copy(),
               np.ctypeslib.as_array(ctypes.cast(val, ctypes.POINTER(ctypes.c_double)), (max(1, nnz.value),))[:nnz.value].copy())
    finally:
        for p in (rp, col, val):
            L.sptrsv_io_free(p)
    return out


def write_csr(path, row_ptr, col, val):
    """.matrix (binary) or .txt, the reference's layouts."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    _check(_lib.lib().sptrsv_write_csr(str(path).encode(), len(rp) - 1, int(rp[-1]), rp,
                                       np.ascontiguousarray(col, dtype=np.int32),
                                       np.ascontiguousarray(val, dtype=np.float64)), "write_csr")


def read_snodes(path):
    """.snodes (binary) or .txt supernode partition -> int32[sn+1]."""
    L = _lib.lib()
    sn, p = ctypes.c_int(), ctypes.c_void_p()
    _check(L.sptrsv_read_snodes(str(path).encode(), ctypes.byref(sn), ctypes.byref(p)), "read_snodes")
    try:
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_int32)), (sn.value + 1,)).copy()
    finally:
        L.sptrsv_io_free(p)


def write_snodes(path, snodes):
    s = np.ascontiguousarray(snodes, dtype=np.int32)
    _check(_lib.lib().sptrsv_write_snodes(str(path).encode(), len(s) - 1, s), "write_snodes")
