// factor.cu -- the upstream step: a multifrontal supernodal Cholesky A = U^T U of a symmetric
// positive definite matrix on the GPU, producing U in the solver's CSR layout (diagonal first in
// every row) and its supernode partition.  The reference takes its factors from an external
// sparse Cholesky; this builds them from A and an elimination tree of fronts.
//
// Symbolic step (host): front t pivots rows f0 .. f1-1 and hands its update matrix to its parent.
// Its row set is S_t = [f0, f1) followed, sorted, by every row >= f1 adjacent in A to one of its
// pivots or in one of its children's update sets.  U's pattern follows: row f0 + k holds S_t[k:].
// Numeric step (GPU, fronts in the given postorder): the dense front F_t (|S_t| x |S_t|, column
// major, lower triangle) gets A's entries and its children's update matrices (extend-add), then a
// blocked right-looking Cholesky over its first w = f1 - f0 columns in 64-column panels: the
// panel's diagonal tile factored by one CTA, the rows below it solved against that tile, the
// trailing lower triangle updated by a tiled FP64 rank-64 product.  Running the trailing updates
// over the whole front leaves the Schur complement -- the update matrix for the parent -- in
// F_t[w:, w:].  Column f0 + k of L = U^T is F_t[k:, k], copied into U's row f0 + k.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>
#include "common.cuh"
#include "sptrsv_gb300.h"

namespace sptrsv {

constexpr int kFb = 64;  // panel width and update tile

// F[idx[q]] = v[q]: A's entries of one front.
__global__ void k_fr_scatter(double* __restrict__ F, const int64_t* __restrict__ idx, const double* __restrict__ v,
                             int count) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < count; q += gridDim.x * blockDim.x) F[idx[q]] = v[q];
}

// F[map[r] + map[s] m] += C[(wc + r) + (wc + s) mc] for s <= r < nu: a child's update matrix
// (the lower triangle of its front past its pivots) added into the parent front.
__global__ void k_fr_extend_add(double* __restrict__ F, int m, const double* __restrict__ C, int mc, int wc,
                                const int* __restrict__ map, int nu) {
    const long long total = (long long)nu * nu;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(e / nu), r = (int)(e - (long long)s * nu);
        if (r < s) continue;
        F[(size_t)map[r] + (size_t)map[s] * m] += C[(size_t)(wc + r) + (size_t)(wc + s) * mc];
    }
}

// Cholesky of the kb x kb diagonal tile at (k0, k0), lower, in place (one CTA of 256 threads).
// A pivot that is not positive (or not finite) sets *bad and the factor is not used.
__global__ void __launch_bounds__(256) k_fr_potrf(double* __restrict__ F, int m, int k0, int kb, int* bad) {
    __shared__ double T[kFb][kFb + 1];
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        const int r = e % kb, c = e / kb;
        T[r][c] = r >= c ? F[(size_t)(k0 + r) + (size_t)(k0 + c) * m] : 0.0;
    }
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        if (threadIdx.x == 0) {
            const double d = T[j][j];
            if (!(d > 0.0) || !isfinite(d)) atomicExch(bad, 1);
            T[j][j] = sqrt(d > 0.0 ? d : 1.0);
        }
        __syncthreads();
        const double inv = 1.0 / T[j][j];
        for (int i = j + 1 + threadIdx.x; i < kb; i += blockDim.x) T[i][j] *= inv;
        __syncthreads();
        const int rest = kb - j - 1;
        for (int e = threadIdx.x; e < rest * rest; e += blockDim.x) {
            const int i = j + 1 + e % rest, c = j + 1 + e / rest;
            if (i >= c) T[i][c] = fma(-T[i][j], T[c][j], T[i][c]);
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        const int r = e % kb, c = e / kb;
        if (r >= c) F[(size_t)(k0 + r) + (size_t)(k0 + c) * m] = T[r][c];
    }
}

// Rows r0 .. m-1 of the panel (columns k0 .. k0+kb-1): X L^T = B with L the factored tile, one
// thread per row, four partial sums per element so that the FP64 chain is a quarter as long.
__global__ void __launch_bounds__(256) k_fr_trsm(double* __restrict__ F, int m, int k0, int kb, int r0) {
    __shared__ double L[kFb][kFb + 1];
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        const int r = e % kb, c = e / kb;
        L[r][c] = r >= c ? F[(size_t)(k0 + r) + (size_t)(k0 + c) * m] : 0.0;
    }
    __syncthreads();
    const int r = r0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    double x[kFb];
    for (int j = 0; j < kb; ++j) {
        double s0 = F[(size_t)r + (size_t)(k0 + j) * m], s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int c = 0;
        for (; c + 3 < j; c += 4) {
            s0 = fma(-x[c], L[j][c], s0);
            s1 = fma(-x[c + 1], L[j][c + 1], s1);
            s2 = fma(-x[c + 2], L[j][c + 2], s2);
            s3 = fma(-x[c + 3], L[j][c + 3], s3);
        }
        for (; c < j; ++c) s0 = fma(-x[c], L[j][c], s0);
        x[j] = ((s0 + s1) + (s2 + s3)) / L[j][j];
    }
    for (int j = 0; j < kb; ++j) F[(size_t)r + (size_t)(k0 + j) * m] = x[j];
}

// The trailing lower triangle F[r0:, r0:] -= P P^T with P = F[r0:, k0:k0+kb]: one 64 x 64 output
// tile per CTA (tiles above the diagonal skip), 256 threads of 4 x 4 outputs each.
__global__ void __launch_bounds__(256) k_fr_syrk(double* __restrict__ F, int m, int k0, int kb, int r0) {
    const int ti = blockIdx.x, tj = blockIdx.y;
    if (tj > ti) return;
    extern __shared__ double fr_sm[];
    double* A = fr_sm;                  // [kFb][kFb + 1]: rows of tile ti
    double* B = fr_sm + kFb * (kFb + 1);  // [kFb][kFb + 1]: rows of tile tj
    const int rA = r0 + ti * kFb, rB = r0 + tj * kFb;
    for (int e = threadIdx.x; e < kFb * kb; e += blockDim.x) {
        const int rr = e % kFb, c = e / kFb;
        A[rr * (kFb + 1) + c] = rA + rr < m ? F[(size_t)(rA + rr) + (size_t)(k0 + c) * m] : 0.0;
        B[rr * (kFb + 1) + c] = rB + rr < m ? F[(size_t)(rB + rr) + (size_t)(k0 + c) * m] : 0.0;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4] = {};
    for (int c = 0; c < kb; ++c) {
        double a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a[u] = A[(ty * 4 + u) * (kFb + 1) + c];
            b[u] = B[(tx * 4 + u) * (kFb + 1) + c];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int row = rA + ty * 4 + u;
        if (row >= m) continue;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int colx = rB + tx * 4 + v;
            if (colx < m && colx <= row) F[(size_t)row + (size_t)colx * m] -= acc[u][v];
        }
    }
}

// U's values of one front: row f0 + k (k < w) = F[k:, k].
__global__ void k_fr_copy_rows(const double* __restrict__ F, int m, int w, const int64_t* __restrict__ rp, int f0,
                               double* __restrict__ uval) {
    const int k = blockIdx.x;
    if (k >= w) return;
    const int64_t base = rp[f0 + k];
    for (int r = k + threadIdx.x; r < m; r += blockDim.x) uval[base + (r - k)] = F[(size_t)r + (size_t)k * m];
}

struct Factor {
    int n = 0;
    std::vector<int64_t> rp;
    std::vector<int> col, snodes;
    std::vector<double> val;
};

}  // namespace sptrsv

using namespace sptrsv;

extern "C" int sptrsv_factor_multifrontal(int device, int n, const int64_t* a_rp, const int* a_col,
                                          const double* a_val, int nf, const int* front_start,
                                          const int* front_parent, int max_width, void** out) {
    if (!out) return SPTRSV_ERR_INVALID_ARG;
    *out = nullptr;
    if (n <= 0 || nf <= 0 || !a_rp || !a_col || !a_val || !front_start || !front_parent || max_width <= 0)
        return SPTRSV_ERR_INVALID_ARG;
    if (front_start[0] != 0 || front_start[nf] != n) return SPTRSV_ERR_INVALID_ARG;
    for (int t = 0; t < nf; ++t) {
        if (front_start[t + 1] <= front_start[t]) return SPTRSV_ERR_INVALID_ARG;
        const int p = front_parent[t];
        if (p != -1 && (p <= t || p >= nf)) return SPTRSV_ERR_INVALID_ARG;  // a postorder: parents come later
    }
    if (a_rp[0] != 0) return SPTRSV_ERR_ROW_PTR;
    for (int i = 0; i < n; ++i)
        if (a_rp[i + 1] < a_rp[i]) return SPTRSV_ERR_ROW_PTR;
    const int64_t annz = a_rp[n];
    for (int64_t e = 0; e < annz; ++e)
        if (a_col[e] < 0 || a_col[e] >= n) return SPTRSV_ERR_COL_RANGE;
    // ---- symbolic: row sets, index maps, U's pattern, supernodes
    std::vector<int> front_of(n);
    for (int t = 0; t < nf; ++t)
        for (int i = front_start[t]; i < front_start[t + 1]; ++i) front_of[i] = t;
    std::vector<std::vector<int>> children(nf), S(nf);
    for (int t = 0; t < nf; ++t)
        if (front_parent[t] >= 0) children[front_parent[t]].push_back(t);
    std::vector<int64_t> a_idx_off(nf + 1, 0), map_off(nf + 1, 0);
    std::vector<int64_t> a_idx;
    std::vector<double> a_v;
    std::vector<int> maps;
    std::vector<int> mark(n, -1);
    for (int t = 0; t < nf; ++t) {
        const int f0 = front_start[t], f1 = front_start[t + 1];
        std::vector<int> below;
        for (int p = f0; p < f1; ++p)
            for (int64_t e = a_rp[p]; e < a_rp[p + 1]; ++e) {
                const int q = a_col[e];
                if (q >= f1 && mark[q] != t) {
                    mark[q] = t;
                    below.push_back(q);
                }
            }
        for (int c : children[t]) {
            const int wc = front_start[c + 1] - front_start[c];
            for (size_t k = wc; k < S[c].size(); ++k) {
                const int q = S[c][k];
                if (q < f0) return SPTRSV_ERR_INVALID_ARG;  // an update row no ancestor pivots
                if (q >= f1 && mark[q] != t) {
                    mark[q] = t;
                    below.push_back(q);
                }
            }
        }
        std::sort(below.begin(), below.end());
        std::vector<int>& St = S[t];
        St.reserve((size_t)(f1 - f0) + below.size());
        for (int p = f0; p < f1; ++p) St.push_back(p);
        St.insert(St.end(), below.begin(), below.end());
        const int m = (int)St.size();
        auto pos = [&](int q) -> int {
            if (q < f1) return q - f0;
            return (f1 - f0) + (int)(std::lower_bound(below.begin(), below.end(), q) - below.begin());
        };
        // A's lower-triangle entries of the pivot columns
        for (int p = f0; p < f1; ++p)
            for (int64_t e = a_rp[p]; e < a_rp[p + 1]; ++e) {
                const int q = a_col[e];
                if (q < p) continue;
                a_idx.push_back((int64_t)pos(q) + (int64_t)(p - f0) * m);
                a_v.push_back(a_val[e]);
            }
        a_idx_off[t + 1] = (int64_t)a_idx.size();
        // the children's update rows within this front
        for (int c : children[t]) {
            const int wc = front_start[c + 1] - front_start[c];
            for (size_t k = wc; k < S[c].size(); ++k) maps.push_back(pos(S[c][k]));
        }
        map_off[t + 1] = (int64_t)maps.size();
    }
    Factor* fct = new Factor;
    fct->n = n;
    fct->rp.assign(n + 1, 0);
    for (int t = 0; t < nf; ++t) {
        const int f0 = front_start[t], w = front_start[t + 1] - f0, m = (int)S[t].size();
        for (int k = 0; k < w; ++k) fct->rp[f0 + k + 1] = m - k;
    }
    for (int i = 0; i < n; ++i) fct->rp[i + 1] += fct->rp[i];
    fct->col.resize(fct->rp[n]);
    for (int t = 0; t < nf; ++t) {
        const int f0 = front_start[t], w = front_start[t + 1] - f0;
        for (int k = 0; k < w; ++k) std::copy(S[t].begin() + k, S[t].end(), fct->col.begin() + fct->rp[f0 + k]);
    }
    fct->snodes.push_back(0);
    for (int t = 0; t < nf; ++t) {
        const int f0 = front_start[t], f1 = front_start[t + 1], w = f1 - f0;
        const int pieces = (w + max_width - 1) / max_width, step = (w + pieces - 1) / pieces;
        for (int a = f0; a < f1; a += step) fct->snodes.push_back(std::min(f1, a + step));
    }
    fct->val.resize(fct->rp[n]);
    // ---- numeric on the GPU
    int rc = 0;
    cudaStream_t st = nullptr;
    int64_t* d_aidx = nullptr;
    double* d_av = nullptr;
    int* d_maps = nullptr;
    int64_t* d_rp = nullptr;
    double* d_uval = nullptr;
    int* d_bad = nullptr;
    std::vector<double*> F(nf, nullptr);
    auto fail = [&](cudaError_t e, const char* what) {
        if (!rc) rc = set_cuda_error(e, what);
    };
    auto ck = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess) fail(e, what);
        return rc == 0;
    };
    const size_t syrk_smem = sizeof(double) * 2 * kFb * (kFb + 1);
    do {
        if (!ck(cudaSetDevice(device), "cudaSetDevice")) break;
        if (!ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream")) break;
        if (!ck(cudaFuncSetAttribute(k_fr_syrk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)syrk_smem), "attr"))
            break;
        if (!ck(cudaMallocAsync((void**)&d_aidx, sizeof(int64_t) * std::max<size_t>(1, a_idx.size()), st), "alloc")) break;
        if (!ck(cudaMallocAsync((void**)&d_av, sizeof(double) * std::max<size_t>(1, a_v.size()), st), "alloc")) break;
        if (!ck(cudaMallocAsync((void**)&d_maps, sizeof(int) * std::max<size_t>(1, maps.size()), st), "alloc")) break;
        if (!ck(cudaMallocAsync((void**)&d_rp, sizeof(int64_t) * (n + 1), st), "alloc")) break;
        if (!ck(cudaMallocAsync((void**)&d_uval, sizeof(double) * std::max<int64_t>(1, fct->rp[n]), st), "alloc")) break;
        if (!ck(cudaMallocAsync((void**)&d_bad, sizeof(int), st), "alloc")) break;
        if (!ck(cudaMemsetAsync(d_bad, 0, sizeof(int), st), "memset")) break;
        if (!a_idx.empty() &&
            (!ck(cudaMemcpyAsync(d_aidx, a_idx.data(), sizeof(int64_t) * a_idx.size(), cudaMemcpyHostToDevice, st), "h2d") ||
             !ck(cudaMemcpyAsync(d_av, a_v.data(), sizeof(double) * a_v.size(), cudaMemcpyHostToDevice, st), "h2d")))
            break;
        if (!maps.empty() &&
            !ck(cudaMemcpyAsync(d_maps, maps.data(), sizeof(int) * maps.size(), cudaMemcpyHostToDevice, st), "h2d"))
            break;
        if (!ck(cudaMemcpyAsync(d_rp, fct->rp.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st), "h2d")) break;
        for (int t = 0; t < nf && !rc; ++t) {
            const int f0 = front_start[t], w = front_start[t + 1] - f0, m = (int)S[t].size();
            if (!ck(cudaMallocAsync((void**)&F[t], sizeof(double) * (size_t)m * m, st), "front alloc")) break;
            if (!ck(cudaMemsetAsync(F[t], 0, sizeof(double) * (size_t)m * m, st), "front memset")) break;
            const int na = (int)(a_idx_off[t + 1] - a_idx_off[t]);
            if (na > 0) k_fr_scatter<<<(na + 255) / 256, 256, 0, st>>>(F[t], d_aidx + a_idx_off[t], d_av + a_idx_off[t], na);
            int64_t mo = map_off[t];
            for (int c : children[t]) {
                const int wc = front_start[c + 1] - front_start[c], mc = (int)S[c].size(), nu = mc - wc;
                if (nu > 0) {
                    const long long tot = (long long)nu * nu;
                    const int g = (int)std::min<long long>(65535, (tot + 255) / 256);
                    k_fr_extend_add<<<g, 256, 0, st>>>(F[t], m, F[c], mc, wc, d_maps + mo, nu);
                }
                mo += nu;
                if (!ck(cudaFreeAsync(F[c], st), "front free")) break;
                F[c] = nullptr;
            }
            for (int k0 = 0; k0 < w && !rc; k0 += kFb) {
                const int kb = std::min(kFb, w - k0), r0 = k0 + kb;
                k_fr_potrf<<<1, 256, 0, st>>>(F[t], m, k0, kb, d_bad);
                if (r0 < m) {
                    k_fr_trsm<<<(m - r0 + 255) / 256, 256, 0, st>>>(F[t], m, k0, kb, r0);
                    const int tiles = (m - r0 + kFb - 1) / kFb;
                    k_fr_syrk<<<dim3(tiles, tiles), 256, syrk_smem, st>>>(F[t], m, k0, kb, r0);
                }
                ck(cudaGetLastError(), "front kernels");
            }
            k_fr_copy_rows<<<w, 256, 0, st>>>(F[t], m, w, d_rp, f0, d_uval);
            ck(cudaGetLastError(), "front copy");
            if (front_parent[t] < 0) {
                ck(cudaFreeAsync(F[t], st), "front free");
                F[t] = nullptr;
            }
        }
        if (rc) break;
        int bad = 0;
        if (!ck(cudaMemcpyAsync(fct->val.data(), d_uval, sizeof(double) * fct->val.size(), cudaMemcpyDeviceToHost, st),
                "d2h") ||
            !ck(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st), "d2h") ||
            !ck(cudaStreamSynchronize(st), "sync"))
            break;
        if (bad) rc = SPTRSV_ERR_ZERO_PIVOT;  // not positive definite in this order
    } while (false);
    if (st) {
        for (double* p : F)
            if (p) cudaFreeAsync(p, st);
        for (void* p : {(void*)d_aidx, (void*)d_av, (void*)d_maps, (void*)d_rp, (void*)d_uval, (void*)d_bad})
            if (p) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    if (rc) {
        delete fct;
        return rc;
    }
    *out = fct;
    return 0;
}

extern "C" int sptrsv_factor_info(void* f, int* n, int64_t* nnz, int* nsn) {
    if (!f) return SPTRSV_ERR_INVALID_ARG;
    const Factor* F = static_cast<const Factor*>(f);
    if (n) *n = F->n;
    if (nnz) *nnz = F->rp[F->n];
    if (nsn) *nsn = (int)F->snodes.size() - 1;
    return 0;
}

extern "C" int sptrsv_factor_copy(void* f, int64_t* row_ptr, int* col, double* val, int* supernodes) {
    if (!f) return SPTRSV_ERR_INVALID_ARG;
    const Factor* F = static_cast<const Factor*>(f);
    if (row_ptr) std::memcpy(row_ptr, F->rp.data(), sizeof(int64_t) * F->rp.size());
    if (col) std::memcpy(col, F->col.data(), sizeof(int) * F->col.size());
    if (val) std::memcpy(val, F->val.data(), sizeof(double) * F->val.size());
    if (supernodes) std::memcpy(supernodes, F->snodes.data(), sizeof(int) * F->snodes.size());
    return 0;
}

extern "C" void sptrsv_factor_free(void* f) { delete static_cast<Factor*>(f); }
