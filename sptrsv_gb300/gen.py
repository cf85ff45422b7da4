"""Seeded synthetic systems (front end of libsptrsv_gen.so; see csrc/gen.cpp for the exact
recipes and the random-number transforms).

Workloads:
* ``laplace2d_cholesky(g)``: exact upper Cholesky factor of the 5-point Laplacian on a g x g
  grid, natural ordering, full band (bandwidth g).  g = 64 is the plain FP64 single-RHS case
  (n = 4,096, nnz = 264,160).
* ``random_upper(n, mean, p_near, band, seed)``: Poisson(mean) off-diagonals per row, each at
  i + U{1..band} with probability p_near else U{i+1..n-1}, values U[-1,1], diagonal
  1 + sum |off|.  n = 2,000,000, mean 8, p_near 0.9, band 64, seed 1 is the large irregular
  case.
* ``supernodal_random``: random U with true supernode structure (dense triangles + shared
  rectangle columns), with its partition.
"""
import ctypes

import numpy as np

from . import _lib


class Csr:
    def __init__(self, row_ptr, col, val, snodes=None):
        self.row_ptr = row_ptr   # int64[n+1]
        self.col = col           # int32[nnz]
        self.val = val           # float64[nnz]
        self.snodes = snodes     # int32[sn+1] or None
        self.n = len(row_ptr) - 1
        self.nnz = int(row_ptr[-1])

    @property
    def row_ptr_u64(self):
        return self.row_ptr.astype(np.uint64)


def _take(h):
    G = _lib.gen()
    if not h:
        raise ValueError("generator rejected its arguments")
    try:
        n, nnz = G.sptrsv_gen_n(h), G.sptrsv_gen_nnz(h)
        rp = np.empty(n + 1, dtype=np.int64)
        col = np.empty(nnz, dtype=np.int32)
        val = np.empty(nnz, dtype=np.float64)
        G.sptrsv_gen_copy(h, rp, col, val)
    finally:
        G.sptrsv_gen_free(h)
    return Csr(rp, col, val)


def laplace2d_cholesky(g):
    return _take(_lib.gen().sptrsv_gen_laplace2d_cholesky(int(g)))


def random_upper(n, mean=8.0, p_near=0.9, band=64, seed=1):
    return _take(_lib.gen().sptrsv_gen_random_upper(int(n), float(mean), float(p_near), int(band), int(seed)))


def supernodal_random(n, wmin=1, wmax=16, mean_rect=6.0, p_near=0.8, band=64, seed=3):
    G = _lib.gen()
    sp = ctypes.POINTER(ctypes.c_int)()
    sn = ctypes.c_int()
    h = G.sptrsv_gen_supernodal_random(int(n), int(wmin), int(wmax), float(mean_rect), float(p_near), int(band),
                                       int(seed), ctypes.byref(sp), ctypes.byref(sn))
    m = _take(h)
    m.snodes = np.ctypeslib.as_array(sp, shape=(sn.value + 1,)).astype(np.int32).copy()
    G.sptrsv_gen_free_ints(ctypes.cast(sp, ctypes.c_void_p))
    return m


def uniform(seed, count, lo=-1.0, hi=1.0):
    out = np.empty(int(count), dtype=np.float64)
    _lib.gen().sptrsv_gen_uniform(int(seed), int(count), float(lo), float(hi), out)
    return out


def spmv(m, x, rhs=1):
    """b = U x (FP64, column-major RHS)."""
    b = np.empty(m.n * rhs, dtype=np.float64)
    _lib.gen().sptrsv_gen_spmv(m.n, m.row_ptr, m.col, m.val, np.ascontiguousarray(x, dtype=np.float64).reshape(-1), b,
                               rhs)
    return b


XSTAR_SALT = 0x9E3779B97F4A7C15


def system(m, seed, rhs=1):
    """x* ~ U[-1,1] from mt19937_64(seed + XSTAR_SALT mod 2^64), b = U x*."""
    xs = uniform((int(seed) + XSTAR_SALT) % (1 << 64), m.n * rhs)
    return xs, spmv(m, xs, rhs)


def band_laplace_case():
    """The plain FP64 single-RHS case: g = 64 Laplacian factor, x* seed 0."""
    m = laplace2d_cholesky(64)
    xs, b = system(m, 0)
    return m, xs, b


def irregular_case(n=2_000_000, seed=1):
    """The large irregular single-RHS case (n = 2M, Poisson(8), p_near 0.9, band 64, seed 1)."""
    m = random_upper(n, 8.0, 0.9, 64, seed)
    xs, b = system(m, seed)
    return m, xs, b


# --------------------------------------------------------------------------------------------
# 3D Laplacian, nested dissection, supernodal Cholesky (the supernodal workload)

def _nd_tree(g, leaf):
    """Geometric nested dissection of the g^3 grid: recursive bisection of the longest side at its
    middle plane until no side exceeds `leaf`.  Returns (order, nodes): order[k] = grid index of
    the k-th unknown; nodes = postordered list of (first, last+1, parent) pivot ranges."""
    order = []
    nodes = []

    def rec(box):
        (x0, x1), (y0, y1), (z0, z1) = box
        sides = (x1 - x0, y1 - y0, z1 - z0)
        if min(sides) <= 0:
            return None
        if max(sides) <= leaf:
            first = len(order)
            for z in range(z0, z1):
                for y in range(y0, y1):
                    for x in range(x0, x1):
                        order.append((z * g + y) * g + x)
            nodes.append([first, len(order), -1])
            return len(nodes) - 1
        d = sides.index(max(sides))
        lo, hi = box[d]
        m = (lo + hi) // 2
        left = list(box)
        right = list(box)
        sep = list(box)
        left[d] = (lo, m)
        right[d] = (m + 1, hi)
        sep[d] = (m, m + 1)
        kids = [k for k in (rec(tuple(left)), rec(tuple(right))) if k is not None]
        first = len(order)
        (sx0, sx1), (sy0, sy1), (sz0, sz1) = sep
        for z in range(sz0, sz1):
            for y in range(sy0, sy1):
                for x in range(sx0, sx1):
                    order.append((z * g + y) * g + x)
        nodes.append([first, len(order), -1])
        me = len(nodes) - 1
        for k in kids:
            nodes[k][2] = me
        return me

    rec(((0, g), (0, g), (0, g)))
    return np.array(order, dtype=np.int64), nodes


def laplace3d_nd_cholesky(g=40, leaf=8, max_width=400):
    """Exact upper Cholesky factor U (A = U^T U) of the 7-point 3D Laplacian (diag 6, off -1) on a
    g^3 grid under geometric nested dissection (recursive coordinate-plane bisection down to
    leaf^3 boxes), with its supernode partition.  Multifrontal factorisation over the dissection
    tree with dense fronts; every front's pivot block is a supernode (dense triangle plus one
    shared set of columns to its right), split into chunks of at most `max_width` rows."""
    import scipy.linalg as sla
    order, nodes = _nd_tree(g, leaf)
    n = g ** 3
    inv = np.empty(n, dtype=np.int64)
    inv[order] = np.arange(n)

    def neighbours(p):
        z, rem = divmod(int(p), g * g)
        y, x = divmod(rem, g)
        out = []
        for dz, dy, dx in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
            zz, yy, xx = z + dz, y + dy, x + dx
            if 0 <= zz < g and 0 <= yy < g and 0 <= xx < g:
                out.append(inv[(zz * g + yy) * g + xx])
        return out

    children = [[] for _ in nodes]
    for k, (_, _, par) in enumerate(nodes):
        if par >= 0:
            children[par].append(k)
    upd = [None] * len(nodes)       # (structure, dense update matrix) handed to the parent
    cols = {}                       # pivot column -> (row indices, values) of L
    for t, (f0, f1, _) in enumerate(nodes):
        piv = np.arange(f0, f1)
        below = set()
        for p in piv:
            for q in neighbours(order[p]):
                if q >= f1:
                    below.add(int(q))
        for c in children[t]:
            below.update(int(v) for v in upd[c][0] if v >= f1)
        S = np.concatenate([piv, np.array(sorted(below), dtype=np.int64)])
        m, w = len(S), f1 - f0
        F = np.zeros((m, m))
        pos = {int(v): k for k, v in enumerate(S)}
        for k, p in enumerate(piv):
            F[k, k] = 6.0
            for q in neighbours(order[p]):
                if q >= f0:
                    j = pos[int(q)]
                    F[j, k] = -1.0
                    F[k, j] = -1.0
        for c in children[t]:
            cs, cu = upd[c]
            idx = np.searchsorted(S, cs)
            for r in range(len(idx)):  # extend-add, one row at a time
                F[idx[r], idx] += cu[r]
            upd[c] = None
        L11 = sla.cholesky(F[:w, :w], lower=True)
        if m > w:
            L21 = sla.solve_triangular(L11, F[w:, :w].T, lower=True).T
            upd[t] = (S[w:], F[w:, w:] - L21 @ L21.T)
            Lcol = np.vstack([L11, L21])
        else:
            upd[t] = (S[w:], np.zeros((0, 0)))
            Lcol = L11
        for k in range(w):
            rows = S[k:]
            cols[f0 + k] = (rows, Lcol[k:, k])
    lens = np.array([len(cols[i][0]) for i in range(n)], dtype=np.int64)
    row_ptr = np.concatenate([[0], np.cumsum(lens)])
    col = np.empty(row_ptr[-1], dtype=np.int32)
    val = np.empty(row_ptr[-1])
    for i in range(n):
        r, v = cols[i]
        col[row_ptr[i]:row_ptr[i + 1]] = r
        val[row_ptr[i]:row_ptr[i + 1]] = v
    sn = [0]
    for f0, f1, _ in nodes:
        w = f1 - f0
        k = -(-w // max_width)
        step = -(-w // k)
        for a in range(f0, f1, step):
            sn.append(min(f1, a + step))
    m = Csr(row_ptr, col, val, np.array(sn, dtype=np.int32))
    m.perm = order
    return m


def laplace3d_nd_matrix(g=40, leaf=8):
    """The 7-point 3D Laplacian (diag 6, off -1) on a g^3 grid in the nested-dissection elimination
    order of laplace3d_nd_cholesky, as CSR holding every row's entries at and right of its diagonal,
    with that dissection's fronts: (row_ptr, col, val, front_start, front_parent, order)."""
    order, nodes = _nd_tree(g, leaf)
    n = g ** 3
    inv = np.empty(n, dtype=np.int64)
    inv[order] = np.arange(n)
    z, rem = np.divmod(order, g * g)
    y, x = np.divmod(rem, g)
    rows, cols = [np.arange(n)], [np.arange(n)]
    for dz, dy, dx in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
        zz, yy, xx = z + dz, y + dy, x + dx
        ok = (zz >= 0) & (zz < g) & (yy >= 0) & (yy < g) & (xx >= 0) & (xx < g)
        i = np.nonzero(ok)[0]
        j = inv[(zz[ok] * g + yy[ok]) * g + xx[ok]]
        up = j > i
        rows.append(i[up])
        cols.append(j[up])
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    srt = np.lexsort((c, r))
    r, c = r[srt], c[srt]
    val = np.where(r == c, 6.0, -1.0)
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(row_ptr, r + 1, 1)
    row_ptr = np.cumsum(row_ptr)
    front_start = np.array([f0 for f0, _, _ in nodes] + [n], dtype=np.int32)
    front_parent = np.array([par for _, _, par in nodes], dtype=np.int32)
    return row_ptr, c.astype(np.int32), val, front_start, front_parent, order


def laplace3d_nd_cholesky_gpu(g=40, leaf=8, max_width=400, device=0):
    """The factor of laplace3d_nd_cholesky (same order, fronts and supernodes) computed by the
    library's GPU multifrontal Cholesky (sptrsv_factor_multifrontal)."""
    row_ptr, col, val, fs, fp, order = laplace3d_nd_matrix(g, leaf)
    L = _lib.lib()
    h = ctypes.c_void_p()
    rc = L.sptrsv_factor_multifrontal(int(device), len(row_ptr) - 1, row_ptr, col, val, len(fs) - 1, fs, fp,
                                      int(max_width), ctypes.byref(h))
    if rc:
        raise RuntimeError("sptrsv_factor_multifrontal: status %d" % rc)
    try:
        n, nnz, nsn = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int()
        L.sptrsv_factor_info(h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(nsn))
        rp = np.empty(n.value + 1, dtype=np.int64)
        cl = np.empty(nnz.value, dtype=np.int32)
        vl = np.empty(nnz.value, dtype=np.float64)
        sn = np.empty(nsn.value + 1, dtype=np.int32)
        L.sptrsv_factor_copy(h, rp, cl, vl, sn)
    finally:
        L.sptrsv_factor_free(h)
    m = Csr(rp, cl, vl, sn)
    m.perm = order
    return m


def supernodal_case(g=40, rhs=1, seed=3):
    """The supernodal workload: 40^3 3D Laplacian factor under nested dissection, B ~ U[-1,1]."""
    m = laplace3d_nd_cholesky(g)
    xs = uniform((int(seed) + XSTAR_SALT) % (1 << 64), m.n * rhs)
    return m, xs, spmv(m, xs, rhs)


# --------------------------------------------------------------------------------------------
# The batched uneven mix

class Mix:
    """A packed host arena of independent systems (see csrc/gen.cpp, sptrsv_gen_mix): per-system
    n, rhs, kind (0 Laplacian factor, 1 random), nnz and offsets; the concatenated local row
    pointers (int64), columns, values; x* and b = U x* (row-major n x rhs per system).  The arrays
    are views of generator-owned memory, released by close()."""

    _FIELDS = [("n", np.int32), ("rhs", np.int32), ("kind", np.int32), ("nnz", np.int64), ("rp_off", np.int64),
               ("nz_off", np.int64), ("xb_off", np.int64), ("row_ptr", np.int64), ("col", np.int32),
               ("val", np.float64), ("xstar", np.float64), ("b", np.float64), ("mean", np.float64)]

    def __init__(self, h):
        self._h = h
        G = _lib.gen()
        for k, (name, dt) in enumerate(self._FIELDS):
            p = ctypes.c_void_p()
            ln = ctypes.c_int64()
            if G.sptrsv_gen_mix_array(h, k, ctypes.byref(p), ctypes.byref(ln)):
                raise RuntimeError("mix array %s" % name)
            if ln.value == 0:
                arr = np.empty(0, dtype=dt)
            else:
                buf = (ctypes.c_char * (ln.value * np.dtype(dt).itemsize)).from_address(p.value)
                arr = np.frombuffer(buf, dtype=dt)
            setattr(self, name, arr)
        self.count = len(self.n)

    def system(self, s):
        """System s as a Csr with its x* and b (row-major n x rhs): views of the mix's memory,
        valid until close()."""
        rp = self.row_ptr[self.rp_off[s]:self.rp_off[s + 1]]
        col = self.col[self.nz_off[s]:self.nz_off[s + 1]]
        val = self.val[self.nz_off[s]:self.nz_off[s + 1]]
        xs = self.xstar[self.xb_off[s]:self.xb_off[s + 1]]
        b = self.b[self.xb_off[s]:self.xb_off[s + 1]]
        return Csr(rp, col, val), xs, b

    def close(self):
        if self._h:
            for name, _ in self._FIELDS:
                setattr(self, name, None)
            _lib.gen().sptrsv_gen_mix_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mix(count=512, seed=2, nmin=1000, nmax=200_000, mean_lo=4.0, mean_hi=16.0, rhs_max=16, threads=0):
    """The batched uneven mix: `count` systems, n log-uniform in [nmin, nmax], even-indexed ones
    2D-Laplacian Cholesky factors (grid side round(sqrt n)), odd-indexed ones random diagonally
    dominant (Poisson mean U[mean_lo, mean_hi], p_near 0.9, band 64), RHS U{1..rhs_max}.
    count 512, seed 2, n in [1k, 200k], mean in [4, 16], rhs_max 16 is the batched workload."""
    import os
    if threads <= 0:
        threads = os.cpu_count() or 1
    h = _lib.gen().sptrsv_gen_mix(int(count), int(seed), int(nmin), int(nmax), float(mean_lo), float(mean_hi),
                                  int(rhs_max), int(threads))
    if not h:
        raise ValueError("mix generator rejected its arguments")
    return Mix(h)
