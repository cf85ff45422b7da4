"""Regenerates tests/golden/golden.npz from the reference itself.

Builds the reference's own src/core.cpp (unmodified; oracle/build_ref.sh) and runs it on
  * the reference's shipped fixtures matrices/txt/csr_5_upper.txt, csr_6_upper.txt and
    csr_6_upper_snodes.txt (read from the reference checkout), with the reference's own
    right-hand side b = 1 (utils.cpp:113-126), rhs = 2, column-major;
  * small seeded matrices from sptrsv_gb300.gen (stored in full, so the golden tests do not
    depend on the generator), with random right-hand sides.
Outputs stored: x of base_gauss_upper / _new / barrier_upper / _new, levels and max level of
setLevelUpAndGetMaxLevel, supernodal_upper / _new, the ccs2ccs_pad arrays and
supernodal_blas_upper.  Usage (in a container that has the reference checkout):
    python tests/golden/make_golden.py [reference_dir]
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from sptrsv_gb300 import gen  # noqa: E402


def ref_solves(R, tag, rp, col, val, b, rhs, out, nthreads=(1, 3)):
    n = len(rp) - 1
    rp = rp.astype(np.uint64)
    col = col.astype(np.int32)
    val = val.astype(np.float64)
    x = np.zeros(n * rhs)
    R.ref_base_gauss_upper(n, val, rp, col, x, b.copy(), rhs)
    out[tag + "/base"] = x.copy()
    x = np.zeros(n * rhs)
    R.ref_base_gauss_upper_new(n, val, rp, col, x, b.copy(), rhs)
    out[tag + "/base_new"] = x.copy()
    for t in nthreads:
        x = np.zeros(n * rhs)
        R.ref_barrier_upper(n, x, b.copy(), val, col, rp, t, rhs)
        out[f"{tag}/barrier_t{t}"] = x.copy()
        x = np.zeros(n * rhs)
        R.ref_barrier_upper_new(n, x, b.copy(), val, col, rp, t, rhs)
        out[f"{tag}/barrier_new_t{t}"] = x.copy()
    lv = np.zeros(n, dtype=np.uint64)
    ml = R.ref_set_levels(n, col, rp, lv)
    out[tag + "/levels"] = lv
    out[tag + "/max_level"] = np.array([ml])


def ref_supernodal(R, tag, rp, col, val, sn, b, rhs, out):
    n = len(rp) - 1
    rp = rp.astype(np.uint64)
    col = col.astype(np.int32)
    sn = sn.astype(np.int32)
    for name, fn in (("super", R.ref_supernodal_upper), ("super_new", R.ref_supernodal_upper_new)):
        x = b.copy()
        fn(len(sn) - 1, sn, x, val, col, rp, n, rhs)
        out[f"{tag}/{name}"] = x
    w = np.diff(sn).astype(np.int64)
    total = int(rp[-1]) + int(np.sum(w * (w - 1) // 2))
    vp = np.zeros(total)
    cp = np.zeros(total, dtype=np.uint64)
    rpp = np.zeros(n + 1, dtype=np.int32)
    nz = R.ref_ccs2ccs_pad(val, col, rp, vp, cp, rpp, sn, len(sn) - 1)
    out[tag + "/pad_val"] = vp[:nz]
    out[tag + "/pad_col"] = cp[:nz]
    out[tag + "/pad_rowptr"] = rpp
    x = b.copy()
    R.ref_supernodal_blas_upper(n, nz, len(sn) - 1, sn, x, vp, cp, rpp, rhs)
    out[tag + "/blas"] = x


def main():
    refdir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPTRSV_REFERENCE", "")
    if not refdir:
        raise SystemExit("usage: make_golden.py REFERENCE_CHECKOUT (or set SPTRSV_REFERENCE)")
    os.environ["SPTRSV_REFERENCE"] = refdir
    oracle.build(force=True)
    R = oracle.ref()
    if R is None:
        raise SystemExit("reference core.cpp did not build")
    out = {}
    txt = os.path.join(refdir, "matrices", "txt")
    for name in ("csr_5_upper", "csr_6_upper"):
        rp, col, val = oracle.read_txt_csr(os.path.join(txt, name + ".txt"))
        n = len(rp) - 1
        out[name + "/row_ptr"] = rp.astype(np.int64)
        out[name + "/col"] = col
        out[name + "/val"] = val
        rhs = 2
        b = np.ones(n * rhs)  # fill_x_b: b = x = 1 (utils.cpp:123)
        ref_solves(R, name, rp, col, val, b, rhs, out)
    sn = oracle.read_txt_snodes(os.path.join(txt, "csr_6_upper_snodes.txt"))
    out["csr_6_upper/snodes"] = sn
    rp, col, val = (out["csr_6_upper/row_ptr"], out["csr_6_upper/col"], out["csr_6_upper/val"])
    ref_supernodal(R, "csr_6_upper", rp, col, val, sn, np.ones(6 * 2), 2, out)

    cases = [
        ("rand3000", gen.random_upper(3000, 8.0, 0.9, 64, 11), 3, 5),
        ("lap12", gen.laplace2d_cholesky(12), 1, 6),
        ("chain500", gen.random_upper(500, 2.0, 1.0, 1, 12), 2, 7),
    ]
    for tag, m, rhs, seed in cases:
        b = gen.uniform(seed, m.n * rhs)
        out[tag + "/row_ptr"], out[tag + "/col"], out[tag + "/val"] = m.row_ptr, m.col, m.val
        out[tag + "/b"] = b
        out[tag + "/rhs"] = np.array([rhs])
        ref_solves(R, tag, m.row_ptr, m.col, m.val, b, rhs, out)
    m = gen.supernodal_random(800, 1, 24, 6.0, 0.8, 64, 3)
    b = gen.uniform(8, m.n * 2)
    out["snr800/row_ptr"], out["snr800/col"], out["snr800/val"], out["snr800/snodes"] = m.row_ptr, m.col, m.val, m.snodes
    out["snr800/b"] = b
    ref_solves(R, "snr800", m.row_ptr, m.col, m.val, b, 2, out)
    ref_supernodal(R, "snr800", m.row_ptr, m.col, m.val, m.snodes, b, 2, out)

    # lower-triangular systems (core.cpp:4-16): transposes of upper ones, diagonal last per row
    import scipy.sparse as sps
    lowers = [("csr_6_lower", out["csr_6_upper/row_ptr"], out["csr_6_upper/col"], out["csr_6_upper/val"], None),
              ("lower3000", None, None, None, gen.random_upper(3000, 8.0, 0.9, 64, 13))]
    for tag, rp, col, val, m in lowers:
        if m is not None:
            rp, col, val = m.row_ptr, m.col, m.val
        n = len(rp) - 1
        L = sps.csr_matrix((val, col, rp), shape=(n, n)).T.tocsr()
        L.sort_indices()
        lrp, lcol, lval = L.indptr.astype(np.uint64), L.indices.astype(np.int32), L.data.astype(np.float64)
        b = np.ones(n) if m is None else gen.uniform(14, n)
        x = np.zeros(n)
        R.ref_base_gauss_lower(n, lval, lrp, lcol, x, b.copy())
        out[tag + "/row_ptr"], out[tag + "/col"], out[tag + "/val"] = lrp.astype(np.int64), lcol, lval
        out[tag + "/b"] = b
        out[tag + "/lower"] = x

    # levels of a larger matrix: only the max level and a digest are stored
    m = gen.random_upper(200_000, 8.0, 0.9, 64, 1)
    lv = np.zeros(m.n, dtype=np.uint64)
    ml = R.ref_set_levels(m.n, m.col, m.row_ptr.astype(np.uint64), lv)
    out["rand200k/max_level"] = np.array([ml])
    out["rand200k/levels_sha256"] = np.frombuffer(hashlib.sha256(lv.tobytes()).digest(), dtype=np.uint8)
    out["rand200k/nnz"] = np.array([m.nnz])

    path = os.path.join(HERE, "golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, len(out), "arrays,", os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
