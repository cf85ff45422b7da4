// supernodal.cu -- the supernodal solve (core.cpp:53-201 family) on dense supernode panels.
//
// A supernode s = rows [a, b) of U whose rows hold a dense upper triangle T_s (columns a..b-1)
// followed by one shared set R_s of columns to the right (the layout supernodal_upper and
// ccs2ccs_pad rely on, core.cpp:53-78,136-161).  The backward solve of the supernode is
//     X_s = T_s^{-1} (B_s - Rect_s X_{R_s}) = G_s [B_s ; X_{R_s}],   G_s = [T_s^{-1} | -T_s^{-1} Rect_s],
// so once G_s is formed (in FP64, at analysis: the diagonal-block factors stay FP64) every row of
// X_s is an independent dot product.  The solve is a sync-free walk over 64-row panels of the
// supernodes in reverse order (a panel waits only on rows of higher supernodes, whose panels hold
// smaller tickets):
//   * FP64: each panel's product split into column blocks taken by different CTAs, partial sums
//     added in block order by the CTA that completes the panel (panels64.cu);
//   * MIXED inner solve: one CTA per panel, BF16x3 tensor-core products (G = G_hi + G_lo and
//     V = V_hi + V_lo in bfloat16; G V ~ G_hi V_hi + G_hi V_lo + G_lo V_hi) accumulated in FP32
//     with mma.sync.m16n8k16, inside the FP64 refinement of refine.cu.
// Supernodes wider than kSnMaxW rows are split into chunks (a chunk of a supernode is again a
// supernode).  The right-hand side [B_s ; X_R] is staged in shared memory block by block; every
// wait on X_R is a bounded pending-sentinel poll.
#include <cuda_bf16.h>
#include <vector>
#include "common.cuh"
#include "kernels.cuh"
#include "handle.cuh"
#include "mma.cuh"
#include "batch.cuh"

namespace sptrsv {

constexpr int kSnMaxW = 256;   // widest supernode chunk
constexpr int kPanel = 64;     // rows per work item (4 warps x 16-row MMA tiles)
constexpr int kKc = 128;       // K rows staged per chunk
constexpr int kNc = 32;        // right-hand-side columns per pass

// --- analysis ---------------------------------------------------------------------------

// One block per supernode chunk [a, b), w = b - a.  Two layouts are accepted:
//   * exact (the layout supernodal_upper and ccs2ccs_pad rely on, core.cpp:53-78,136-161): row
//     a+t holds the w-t triangle columns a+t..b-1 first, then exactly row a's rectangle columns;
//   * skyline: every row a+t is one contiguous column range starting at its diagonal (a banded
//     factor stored with its explicit zeros); a row that ends inside the triangle leaves zeros
//     there, the rectangle is the contiguous range b..b+m-1 with m the longest row's reach past b,
//     and shorter rows read zero in it.
// Records the rectangle width and the layout (0 exact, 1 skyline).
__global__ void k_sn_check(int S, const int* __restrict__ sstart, const int* __restrict__ rp,
                           const int* __restrict__ col, int* __restrict__ m_out, int* __restrict__ kind_out,
                           Ctl* ctl) {
    for (int s = blockIdx.x; s < S; s += gridDim.x) {
        const int a = sstart[s], b = sstart[s + 1], w = b - a;
        const int m = rp[a + 1] - rp[a] - w;
        bool exact = m >= 0;
        const int* rect0 = col + rp[a] + w;
        for (int t = 0; t < w && exact; ++t) {
            const int i = a + t, base = rp[i];
            if (rp[i + 1] - base != (w - t) + m) { exact = false; break; }
            bool bad = false;
            for (int q = threadIdx.x; q < w - t; q += blockDim.x) bad |= col[base + q] != i + q;
            for (int q = threadIdx.x; q < m; q += blockDim.x) bad |= col[base + (w - t) + q] != rect0[q];
            if (__syncthreads_or(bad)) exact = false;
        }
        if (exact) {
            if (threadIdx.x == 0) { m_out[s] = m; kind_out[s] = 0; }
            continue;
        }
        bool sky = true;
        int msky = 0;
        for (int t = 0; t < w && sky; ++t) {
            const int i = a + t, base = rp[i], len = rp[i + 1] - base;
            if (len < 1) { sky = false; break; }
            msky = max(msky, len - (w - t));
            bool bad = false;
            for (int q = threadIdx.x; q < len; q += blockDim.x) bad |= col[base + q] != i + q;
            if (__syncthreads_or(bad)) sky = false;
        }
        if (threadIdx.x == 0) {
            m_out[s] = sky ? msky : 0;
            kind_out[s] = 1;
            if (!sky) record_error(ctl, SPTRSV_ERR_SUPERNODES);
        }
    }
}

__global__ void k_sn_rectcols(int S, const int* __restrict__ sstart, const int* __restrict__ rp,
                              const int* __restrict__ col, const int* __restrict__ roff,
                              const int* __restrict__ kind, int* __restrict__ rect_cols) {
    for (int s = blockIdx.x; s < S; s += gridDim.x) {
        const int a = sstart[s], w = sstart[s + 1] - a;
        const int m = roff[s + 1] - roff[s];
        if (kind[s] == 0) {
            for (int q = threadIdx.x; q < m; q += blockDim.x) rect_cols[roff[s] + q] = col[rp[a] + w + q];
        } else {
            for (int q = threadIdx.x; q < m; q += blockDim.x) rect_cols[roff[s] + q] = a + w + q;
        }
    }
}

// Column j of T_s^{-1} by back substitution, one warp per (supernode, column); written into the
// first w columns of G_s (row-major, leading dimension ld).
__global__ void __launch_bounds__(256) k_sn_tinv(int S, const int* __restrict__ sstart, const int* __restrict__ rp,
                                                 const double* __restrict__ val, const long long* __restrict__ goff,
                                                 const int* __restrict__ ld, const int* __restrict__ colbase,
                                                 int ncols, double* __restrict__ G) {
    __shared__ double xs[8][kSnMaxW];
    const int lane = threadIdx.x & 31, wv = threadIdx.x >> 5;
    for (int task = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; task < ncols; task += (gridDim.x * blockDim.x) >> 5) {
        // task -> (s, j) through the per-supernode column offsets
        int lo = 0, hi = S - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (colbase[mid] <= task) lo = mid; else hi = mid - 1;
        }
        const int s = lo, j = task - colbase[s];
        const int a = sstart[s], w = sstart[s + 1] - a;
        double* x = xs[wv];
        // T[r][c] = val[rp[a+r] + (c - r)]  (c >= r)
        if (lane == 0) x[j] = 1.0 / val[rp[a + j]];
        __syncwarp();
        for (int r = j - 1; r >= 0; --r) {
            const int base = rp[a + r] - r;
            const int lim = min(j, rp[a + r + 1] - base - 1);  // a skyline row may end inside the triangle
            double sum = 0.0;
            for (int c = r + 1 + lane; c <= lim; c += 32) sum = fma(val[base + c], x[c], sum);
            sum = warp_sum(sum);
            if (lane == 0) x[r] = -sum / val[rp[a + r]];
            __syncwarp();
        }
        double* g = G + goff[s];
        const int L = ld[s];
        for (int r = lane; r < w; r += 32) g[(size_t)r * L + j] = r <= j ? x[r] : 0.0;
        __syncwarp();
    }
}

// -T_s^{-1} Rect_s into columns w.. of G_s; one thread per output, four partial sums.
__global__ void k_sn_w(int S, const int* __restrict__ sstart, const int* __restrict__ rp,
                       const double* __restrict__ val, const long long* __restrict__ goff, const int* __restrict__ ld,
                       const int* __restrict__ mrect, const long long* __restrict__ outbase, long long nout,
                       double* __restrict__ G) {
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < nout;
         o += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = S - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (outbase[mid] <= o) lo = mid; else hi = mid - 1;
        }
        const int s = lo;
        const int a = sstart[s], w = sstart[s + 1] - a, m = mrect[s];
        const long long q = o - outbase[s];
        const int r = (int)(q / m), k = (int)(q % m);
        const double* g = G + goff[s];
        const int L = ld[s];
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        // Rect[c][k] = val[rp[a+c] + (w - c) + k] while that position is inside row a+c (in the
        // exact layout always; a skyline row shorter than the rectangle reads zero past its end)
        auto rect = [&](int c) -> double {
            const int base = rp[a + c], off = (w - c) + k;
            return off < rp[a + c + 1] - base ? val[base + off] : 0.0;
        };
        int c = r;
        for (; c + 3 < w; c += 4) {
            s0 = fma(g[(size_t)r * L + c], rect(c), s0);
            s1 = fma(g[(size_t)r * L + c + 1], rect(c + 1), s1);
            s2 = fma(g[(size_t)r * L + c + 2], rect(c + 2), s2);
            s3 = fma(g[(size_t)r * L + c + 3], rect(c + 3), s3);
        }
        for (; c < w; ++c) s0 = fma(g[(size_t)r * L + c], rect(c), s0);
        G[goff[s] + (size_t)r * L + w + k] = -((s0 + s1) + (s2 + s3));
    }
}

__global__ void k_sn_split(long long count, const double* __restrict__ G, __nv_bfloat16* __restrict__ hi,
                           __nv_bfloat16* __restrict__ lo) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < count; p += (long long)gridDim.x * blockDim.x) {
        const float f = (float)G[p];
        const __nv_bfloat16 h = __float2bfloat16_rn(f);
        hi[p] = h;
        lo[p] = __float2bfloat16_rn(f - __bfloat162float(h));
    }
}

// --- solve ------------------------------------------------------------------------------

// BF16x3 tensor-core panel product, FP32 output (the mixed path's inner solve).
__global__ void __launch_bounds__(128) k_sn_solve_bf16x3(SnArgs A, const __nv_bfloat16* __restrict__ Ghi,
                                                         const __nv_bfloat16* __restrict__ Glo, int rhs,
                                                         const float* __restrict__ b, float* x, Ctl* ctl,
                                                         int64_t budget) {
    // V chunk, split, stored [n][k] so that a B fragment register (k, k+1) is one 32-bit load
    __shared__ __align__(16) __nv_bfloat16 Vhi[kNc][kKc + 8];
    __shared__ __align__(16) __nv_bfloat16 Vlo[kNc][kKc + 8];
    __shared__ unsigned s_t;
    __shared__ int s_ok;
    const int lane = threadIdx.x & 31, wv = threadIdx.x >> 5;
    if (*(volatile const int*)&ctl->done) return;
    for (;;) {
        if (threadIdx.x == 0) s_t = aborted(ctl) ? 0xFFFFFFFFu : atomicAdd(&ctl->ticket, 1u);
        __syncthreads();
        const unsigned t = s_t;
        if (t >= (unsigned)A.nitems) break;
        const int s = A.item_s[t], p = A.item_p[t];
        const int a = A.sstart[s], w = A.sstart[s + 1] - a, m = A.mrect[s];
        const int K = w + m, L = A.ld[s];
        const int* rc = A.rect_cols + A.roff[s];
        const __nv_bfloat16* ghi = Ghi + A.goff[s];
        const __nv_bfloat16* glo = Glo + A.goff[s];
        const int r0 = p * kPanel;
        const int nrows = w - r0;           // rows of the supernode from this panel's first row
        const int row0 = r0 + 16 * wv;      // this warp's 16-row tile
        bool ok = true;
        for (int c0 = 0; c0 < rhs; c0 += kNc) {
            const int nc = min(kNc, rhs - c0);
            float acc[kNc / 8][4];
#pragma unroll
            for (int q = 0; q < kNc / 8; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
            for (int k0 = 0; k0 < K; k0 += kKc) {
                const int kc = min(kKc, K - k0);
                if (threadIdx.x == 0) s_ok = 1;
                __syncthreads();
                // eight loads per thread in flight together, then waits only on pending values
                constexpr int kStage = 8;
                const int nc8 = (nc + 7) & ~7;
                for (int base = 0; base < kKc * nc8; base += 128 * kStage) {
                    float v[kStage];
#pragma unroll
                    for (int u = 0; u < kStage; ++u) {
                        const int e = base + threadIdx.x + u * 128;
                        float val = 0.f;
                        const int j = e / kKc, kk = e % kKc, k = k0 + kk;
                        if (j < nc8 && kk < kc && j < nc)
                            val = k < w ? b[(size_t)(a + k) * rhs + c0 + j] : ld_relaxed(x + (size_t)rc[k - w] * rhs + c0 + j);
                        v[u] = val;
                    }
#pragma unroll
                    for (int u = 0; u < kStage; ++u) {
                        const int e = base + threadIdx.x + u * 128;
                        const int j = e / kKc, kk = e % kKc, k = k0 + kk;
                        if (j < nc8) {
                            float val = v[u];
                            if (kk < kc && j < nc && k >= w && Pend<float>::is(val) &&
                                !wait_ready<float>(x + (size_t)rc[k - w] * rhs + c0 + j, val, ctl, budget)) {
                                s_ok = 0;
                                val = 0.f;
                            }
                            const __nv_bfloat16 h = __float2bfloat16_rn(val);
                            Vhi[j][kk] = h;
                            Vlo[j][kk] = __float2bfloat16_rn(val - __bfloat162float(h));
                        }
                    }
                }
                __syncthreads();
                if (!s_ok) { ok = false; break; }
                if (row0 < w) {
                    for (int ks = 0; ks < kc; ks += 16) {
                        uint32_t ah[4], al[4];
                        load_a(ghi, L, row0, w, k0 + ks, ah);
                        load_a(glo, L, row0, w, k0 + ks, al);
                        const int kb = ks + (lane & 3) * 2;
#pragma unroll
                        for (int q = 0; q < kNc / 8; ++q) {
                            if (q * 8 >= nc) break;
                            const int n = q * 8 + (lane >> 2);
                            const uint32_t bh0 = *reinterpret_cast<const uint32_t*>(&Vhi[n][kb]);
                            const uint32_t bh1 = *reinterpret_cast<const uint32_t*>(&Vhi[n][kb + 8]);
                            const uint32_t bl0 = *reinterpret_cast<const uint32_t*>(&Vlo[n][kb]);
                            const uint32_t bl1 = *reinterpret_cast<const uint32_t*>(&Vlo[n][kb + 8]);
                            mma_bf16(acc[q], ah, bh0, bh1);
                            mma_bf16(acc[q], ah, bl0, bl1);
                            mma_bf16(acc[q], al, bh0, bh1);
                        }
                    }
                }
                __syncthreads();
            }
            if (!ok) break;
            if (row0 < w) {
                const int ra = row0 + (lane >> 2), rb = ra + 8;
#pragma unroll
                for (int q = 0; q < kNc / 8; ++q) {
                    const int cj = q * 8 + (lane & 3) * 2;
                    if (ra < w && cj < nc) st_relaxed(x + (size_t)(a + ra) * rhs + c0 + cj, Pend<float>::fix(acc[q][0]));
                    if (ra < w && cj + 1 < nc)
                        st_relaxed(x + (size_t)(a + ra) * rhs + c0 + cj + 1, Pend<float>::fix(acc[q][1]));
                    if (rb < w && cj < nc) st_relaxed(x + (size_t)(a + rb) * rhs + c0 + cj, Pend<float>::fix(acc[q][2]));
                    if (rb < w && cj + 1 < nc)
                        st_relaxed(x + (size_t)(a + rb) * rhs + c0 + cj + 1, Pend<float>::fix(acc[q][3]));
                }
            }
        }
        (void)nrows;
        if (__syncthreads_or(!ok)) break;
    }
}

// --- host side --------------------------------------------------------------------------

int Handle::set_supernodes(int sn, const int* snodes_host) {
    if (!analysed) return SPTRSV_ERR_NO_ANALYSIS;
    auto_supernodes = false;
    if (sn < 1 || !snodes_host) return SPTRSV_ERR_INVALID_ARG;
    // validate the partition and split wide supernodes (metadata only, O(sn))
    if (snodes_host[0] != 0 || snodes_host[sn] != n) return SPTRSV_ERR_SUPERNODES;
    std::vector<int> ss{0};
    for (int q = 0; q < sn; ++q) {
        const int a = snodes_host[q], b = snodes_host[q + 1];
        if (b <= a) return SPTRSV_ERR_SUPERNODES;
        const int parts = (b - a + kSnMaxW - 1) / kSnMaxW;
        const int step = (b - a + parts - 1) / parts;
        for (int x0 = a + step; x0 < b; x0 += step) ss.push_back(x0);
        ss.push_back(b);
    }
    const int S = (int)ss.size() - 1;
    int rc;
    if ((rc = sn_start.ensure(sizeof(int) * (S + 1))) || (rc = sn_m.ensure(sizeof(int) * 2 * S))) return rc;
    CUDA_TRY(cudaMemcpyAsync(sn_start.p, ss.data(), sizeof(int) * (S + 1), cudaMemcpyHostToDevice, st));
    if ((rc = reset_ctl())) return rc;
    k_sn_check<<<std::min(S, sm_count * 8), 128, 0, st>>>(S, sn_start.as<int>(), rp, col, sn_m.as<int>(),
                                                         sn_m.as<int>() + S, ctl);
    ++launches;
    CUDA_TRY(cudaGetLastError());
    Ctl c{};
    if ((rc = read_ctl(&c))) return rc;
    if (c.status) return c.status;
    std::vector<int> m(S);
    CUDA_TRY(cudaMemcpy(m.data(), sn_m.p, sizeof(int) * S, cudaMemcpyDeviceToHost));
    // per-chunk offsets (host bookkeeping over S entries)
    std::vector<int> roffh(S + 1, 0), ldh(S), colbase(S + 1, 0);
    std::vector<long long> goffh(S + 1, 0), outbase(S + 1, 0);
    std::vector<int> item_s, item_p;
    for (int s = 0; s < S; ++s) {
        const int w = ss[s + 1] - ss[s];
        roffh[s + 1] = roffh[s] + m[s];
        ldh[s] = (w + m[s] + 15) & ~15;
        const int wpad = (w + 15) & ~15;
        goffh[s + 1] = goffh[s] + (long long)wpad * ldh[s];
        colbase[s + 1] = colbase[s] + w;
        outbase[s + 1] = outbase[s] + (long long)w * m[s];
    }
    for (int s = S - 1; s >= 0; --s) {
        const int w = ss[s + 1] - ss[s];
        for (int p = 0; p * kPanel < w; ++p) { item_s.push_back(s); item_p.push_back(p); }
    }
    const long long gtot = goffh[S];
    if ((rc = sn_roff.ensure(sizeof(int) * (S + 1))) || (rc = sn_rect.ensure(sizeof(int) * ((size_t)roffh[S] + 1))) ||
        (rc = sn_goff.ensure(sizeof(long long) * (S + 1))) || (rc = sn_ld.ensure(sizeof(int) * S)) ||
        (rc = sn_colbase.ensure(sizeof(int) * (S + 1))) || (rc = sn_outbase.ensure(sizeof(long long) * (S + 1))) ||
        (rc = sn_items.ensure(sizeof(int) * 2 * item_s.size())) || (rc = sn_G.ensure(sizeof(double) * (size_t)gtot)) ||
        (rc = sn_Ghi.ensure(2 * (size_t)gtot)) || (rc = sn_Glo.ensure(2 * (size_t)gtot)))
        return rc;
    CUDA_TRY(cudaMemcpyAsync(sn_roff.p, roffh.data(), sizeof(int) * (S + 1), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(sn_goff.p, goffh.data(), sizeof(long long) * (S + 1), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(sn_ld.p, ldh.data(), sizeof(int) * S, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(sn_colbase.p, colbase.data(), sizeof(int) * (S + 1), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(sn_outbase.p, outbase.data(), sizeof(long long) * (S + 1), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(sn_items.p, item_s.data(), sizeof(int) * item_s.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(sn_items.as<int>() + item_s.size(), item_p.data(), sizeof(int) * item_p.size(),
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(sn_G.p, 0, sizeof(double) * (size_t)gtot, st));
    k_sn_rectcols<<<std::min(S, sm_count * 8), 128, 0, st>>>(S, sn_start.as<int>(), rp, col, sn_roff.as<int>(),
                                                            sn_m.as<int>() + S, sn_rect.as<int>());
    k_sn_tinv<<<sm_count * 8, 256, 0, st>>>(S, sn_start.as<int>(), rp, val, sn_goff.as<long long>(), sn_ld.as<int>(),
                                            sn_colbase.as<int>(), colbase[S], sn_G.as<double>());
    launches += 2;
    if (outbase[S] > 0) {
        k_sn_w<<<sm_count * 16, 256, 0, st>>>(S, sn_start.as<int>(), rp, val, sn_goff.as<long long>(), sn_ld.as<int>(),
                                              sn_m.as<int>(), sn_outbase.as<long long>(), outbase[S],
                                              sn_G.as<double>());
        ++launches;
    }
    k_sn_split<<<sm_count * 16, 256, 0, st>>>(gtot, sn_G.as<double>(), sn_Ghi.as<__nv_bfloat16>(),
                                              sn_Glo.as<__nv_bfloat16>());
    ++launches;
    CUDA_TRY(cudaGetLastError());
    // FP64 panel records: every 64-row panel of every chunk, its G split into column blocks
    // (panels64.cu).  Items run chunk by chunk from the last; within a chunk, every panel's own
    // right-hand-side blocks first (no waits), then the solved-row blocks farthest first.
    std::vector<BChunk> pan;
    std::vector<int2> pit;
    long long prows = 0;
    for (int s = S - 1; s >= 0; --s) {
        const int w = ss[s + 1] - ss[s], K = w + m[s], nb = p64_nblk(w, K), no = p64_nown(w);
        const int first = (int)pan.size();
        for (int r0 = 0; r0 < w; r0 += kP64) {
            BChunk c{};
            c.sys = 0;
            c.a = ss[s];
            c.w = w;
            c.m = m[s];
            c.ld = ldh[s];
            c.g64 = sn_G.as<double>() + goffh[s];
            c.rect = sn_rect.as<int>() + roffh[s];
            c.nblk = nb;
            c.r0 = r0;
            c.pw = std::min(kP64, w - r0);
            c.poff = prows;
            c.cbase = (int)pan.size();
            prows += (long long)nb * c.pw;
            pan.push_back(c);
        }
        const int np = (int)pan.size() - first;
        for (int q = 0; q < no; ++q)
            for (int p = 0; p < np; ++p) pit.push_back(make_int2(first + p, q));
        for (int q = nb - 1; q >= no; --q)
            for (int p = 0; p < np; ++p) pit.push_back(make_int2(first + p, q));
    }
    // tensor-core schedule: every panel's G records (digit slices, panels_tc.cu), built below
    std::vector<int2> recs;
    sn_tc = false;
    if (panels_mode() == 1 && build_tc) {
        size_t tot = 0;
        std::vector<size_t> toff(pan.size());
        for (size_t p = 0; p < pan.size(); ++p) {
            toff[p] = tot;
            tot += (tc_panel_bytes(pan[p].w, pan[p].w + pan[p].m) + 127) & ~(size_t)127;
            for (int q = 0; q < pan[p].nblk; ++q) recs.push_back(make_int2((int)p, q));
        }
        if ((rc = sn_gtc.ensure(tot)) || (rc = sn_tcrec.ensure(sizeof(int2) * recs.size()))) return rc;
        for (size_t p = 0; p < pan.size(); ++p) pan[p].gtc = sn_gtc.as<unsigned char>() + toff[p];
    }
    // double-FP32 schedule: G as scaled FP32 pairs (laid out like sn_G) and the row exponents,
    // indexed by the matrix row, converted below
    const bool df = panels_mode() == 2 && build_tc;
    if (df) {
        if ((rc = sn_ghl.ensure(sizeof(float2) * (size_t)std::max(1LL, gtot))) ||
            (rc = sn_gexp.ensure(sizeof(int) * (size_t)std::max(1, n))))
            return rc;
        for (BChunk& c : pan) {
            c.ghl = sn_ghl.as<float2>() + (c.g64 - sn_G.as<double>());
            c.gexp = sn_gexp.as<int>() + c.a;
        }
    }
    if ((rc = sn_pan.ensure(sizeof(BChunk) * pan.size())) || (rc = sn_pitems.ensure(sizeof(int2) * pit.size())))
        return rc;
    CUDA_TRY(cudaMemcpyAsync(sn_pan.p, pan.data(), sizeof(BChunk) * pan.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(sn_pitems.p, pit.data(), sizeof(int2) * pit.size(), cudaMemcpyHostToDevice, st));
    if (!recs.empty()) {
        CUDA_TRY(cudaMemcpyAsync(sn_tcrec.p, recs.data(), sizeof(int2) * recs.size(), cudaMemcpyHostToDevice, st));
        if ((rc = launch_tc_split(sn_pan.as<BChunk>(), sn_tcrec.as<int2>(), (int)recs.size(), sm_count, st, &launches)))
            return rc;
        sn_tc = true;
    }
    if (df && (rc = launch_g_df(sn_pan.as<BChunk>(), (int)pan.size(), st, &launches))) return rc;
    CUDA_TRY(cudaStreamSynchronize(st));
    sn_npan = (int)pan.size();
    sn_npitems = (unsigned)pit.size();
    sn_prows = prows;
    sn_count = S;
    sn_nitems = (int)item_s.size();
    have_supernodes = true;
    drop_graphs();
    return 0;
}

SnArgs Handle::sn_args() const {
    SnArgs A;
    A.nitems = sn_nitems;
    A.item_s = sn_items.as<int>();
    A.item_p = sn_items.as<int>() + sn_nitems;
    A.sstart = sn_start.as<int>();
    A.mrect = sn_m.as<int>();
    A.roff = sn_roff.as<int>();
    A.rect_cols = sn_rect.as<int>();
    A.goff = sn_goff.as<long long>();
    A.ld = sn_ld.as<int>();
    return A;
}

int launch_sn_solve(const Handle& h, bool mixed, const void* b, void* x, int rhs, int64_t budget, int64_t* launches) {
    if (!mixed) {
        // the partial sums (sn_prows x rhs doubles) and the counters (one per panel and RHS group)
        // are sized by Handle::prepare
        const int ncnt = h.sn_npan * p64_groups(rhs);
        if (h.sn_ppart.cap < sizeof(double) * (size_t)h.sn_prows * rhs || h.sn_pcnt.cap < sizeof(int) * (size_t)ncnt)
            return SPTRSV_ERR_INVALID_ARG;
        if (h.sn_tc)
            return launch_panels_tc(nullptr, rhs, (const double*)b, (double*)x, h.ctl, &h.ctl->ticket, budget,
                                    h.sn_pitems.as<int2>(), h.sn_npitems, h.sn_pan.as<BChunk>(),
                                    h.sn_ppart.as<double>(), h.sn_pcnt.as<int>(), h.sn_npan * tc_groups_host(rhs),
                                    h.sm_count, h.st, launches);
        return launch_panels64(nullptr, rhs, (const double*)b, (double*)x, h.ctl, &h.ctl->ticket, budget,
                               h.sn_pitems.as<int2>(), h.sn_npitems, h.sn_pan.as<BChunk>(), h.sn_ppart.as<double>(),
                               h.sn_pcnt.as<int>(), ncnt, 64, h.sm_count, h.st, launches);
    }
    const SnArgs A = h.sn_args();
    {
        int per_sm = 0;
        CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sn_solve_bf16x3, 128, 0));
        int grid = std::max(1, std::min(per_sm * h.sm_count, A.nitems));
        k_sn_solve_bf16x3<<<grid, 128, 0, h.st>>>(A, h.sn_Ghi.as<__nv_bfloat16>(), h.sn_Glo.as<__nv_bfloat16>(), rhs,
                                                 (const float*)b, (float*)x, h.ctl, budget);
    }
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

}  // namespace sptrsv
