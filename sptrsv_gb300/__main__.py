"""Command-line front end with the reference's arguments (app/main.cpp:4-66, run() in
utils.cpp:166-343):

    python -m sptrsv_gb300 ALGO MATRIX SNODES NTHREADS NRHS OPT [check [verbose]]

ALGO: base | custom | blas | barrier | syncfree | write_first | mkl.  MATRIX: .matrix, .mtx or
.txt; SNODES: .snodes or .txt (read for custom and blas); OPT: opt_true selects the reference's
"_new" variants.  x and b start as ones (fill_x_b, utils.cpp:112-124).  Every algorithm runs on
the GPU through the drop-in entry point of the same name (mkl, which has no GPU counterpart in the
reference, runs the handle API's automatic schedule).  `check` reports the relative residual
||b - U x|| / ||b|| of the result and its normwise difference from the FP64 sync-free GPU solve;
`verbose` prints both solutions.
"""
import ctypes
import sys

import numpy as np

import sptrsv_gb300 as sp


def _row_major(x, n, rhs):
    return np.ascontiguousarray(np.asarray(x).reshape(rhs, n).T).reshape(-1)


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) < 5:
        print(__doc__)
        return 1
    algo, mpath, spath, nthreads, nrhs = argv[0], argv[1], argv[2], int(argv[3]), int(argv[4])
    opt = len(argv) > 5 and argv[5] == "opt_true"
    check = len(argv) > 6 and argv[6] == "check"
    verbose = len(argv) > 7 and argv[7] == "verbose"
    rp, col, val = sp.read_csr(mpath)
    n, nz = len(rp) - 1, int(rp[-1])
    rpu = rp.astype(np.uint64)
    print(f"N = {n}; NZ = {nz}")
    b = np.ones(n * nrhs)
    x = np.ones(n * nrhs)
    col_major = True
    if algo in ("custom", "blas"):
        sn = sp.read_snodes(spath)
        if algo == "custom":
            x = b.copy()
            f = sp.supernodal_upper_new if opt else sp.supernodal_upper
            t = f(len(sn) - 1, sn, x, val, col, rpu, n, nrhs)
        else:
            w = np.diff(sn).astype(np.int64)
            extra = int(np.sum(w * (w - 1) // 2))
            vp, cp, rpp = np.zeros(nz + extra), np.zeros(nz + extra, dtype=np.uint64), np.zeros(n + 1, dtype=np.int32)
            nz_pad, sn_c = ctypes.c_int(0), ctypes.c_int(len(sn) - 1)
            sp.ccs2ccs_pad(val, col, rpu, vp, cp, rpp, sn, sn_c, nz_pad)
            x = b.copy()
            f = sp.supernodal_blas_upper_new if opt else sp.supernodal_blas_upper
            t = f(n, nz_pad.value, len(sn) - 1, sn, x, vp, cp, rpp, nrhs)
    elif algo == "base":
        f = sp.base_gauss_upper_new if opt else sp.base_gauss_upper
        t = f(n, val, rpu, col, x, b, nrhs)
    elif algo == "barrier":
        f = sp.barrier_upper_new if opt else sp.barrier_upper
        t = f(n, x, b, val, col, rpu, nthreads, nrhs)
    elif algo == "write_first":
        nrhs, col_major = 1, False
        x, b = np.ones(n), np.ones(n)
        t = sp.sptrsv_syncfree3_opencl(col, rp.astype(np.int32), val, n, n, nz, x, b)
    elif algo == "syncfree":
        col_major = False
        import scipy.sparse as sps
        T = sps.csr_matrix((val, col, rp), shape=(n, n)).tocsc()
        T.sort_indices()
        t = sp.sptrsv_syncfree_opencl(T.indptr.astype(np.int32), T.indices.astype(np.int32), T.data.copy(), n, n, nz,
                                      x, b, nrhs)
    elif algo == "mkl":
        col_major = False
        with sp.Solver(0) as s:
            s.analyse(rp, col, val)
            x = s.solve(b, rhs=nrhs, layout=sp.ROW_MAJOR)
            t = 0.0
    else:
        print(f"Unknown algorithm {algo}. Exit")
        return 1
    print(f"Algorithm finished. Time: {t:.6f}")
    if t < 0:
        print("status:", sp.status_string(int(t)))
        return 2
    if check:
        xm = np.asarray(x).reshape(-1)
        xr = _row_major(xm, n, nrhs) if col_major else xm
        U = __import__("scipy.sparse", fromlist=["csr_matrix"]).csr_matrix((val, col, rp), shape=(n, n))
        X = xr.reshape(n, nrhs)
        B = np.ones((n, nrhs))
        res = np.linalg.norm(B - U @ X) / np.linalg.norm(B)
        with sp.Solver(0) as s:
            s.analyse(rp, col, val)
            xc = s.solve(np.ones(n * nrhs), rhs=nrhs, layout=sp.ROW_MAJOR, schedule="syncfree_warp")
        diff = np.linalg.norm(xr - xc) / np.linalg.norm(xc)
        print(f"relative residual {res:.3e}; difference from the FP64 sync-free solve {diff:.3e}")
        if verbose:
            print("x x_check")
            for a, c in zip(xr, xc):
                print(a, c)
    return 0


if __name__ == "__main__":
    sys.exit(main())
