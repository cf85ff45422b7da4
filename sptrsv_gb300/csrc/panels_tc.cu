// panels_tc.cu -- FP64-accurate panel products on the tensor cores (tcgen05, TMEM accumulators):
// the same work items, partial sums and publication protocol as the FP64 panel kernel
// (panels64.cu), with G x [b ; x_R] formed from BF16 digit slices instead of FP64 FMAs.
//
// Split product (Ozaki, Ogita, Oishi and Rump 2012, fixed-point digits): every row of a panel block
// of G and every right-hand-side column of the matching block of [b ; x_R] is written as eight
// signed 7-bit digits against a power-of-two scale (tc.cuh), so G_blk V = 2^(e_r + f_j) sum over
// digit pairs (p, q) of D_pq 2^(-7(p+q)), with D_pq = G_p V_q an integer matrix product.  Pairs with
// p + q <= 9 are formed (the rest lie below FP64 rounding of the dot product): 36 products.  The
// BF16 digits are exact, the tensor cores multiply them exactly and every FP32 accumulator sums at
// most eight 64-term digit products, below 2^23: exact.  The eight accumulators (one per digit
// diagonal) are combined in FP64, so the product's error is that of an FP64 dot product.
//
// Tensor-core use: the G record of a (panel, block) holds the eight digit slices of its 64 rows as
// K-major tiles one after another, so the A operand of an M = 128 MMA starting at slice p is
// [G_p ; G_(p+1)]: one MMA forms D_pq in TMEM lanes 0..63 and D_(p+1)q in lanes 64..127.  With p odd
// the accumulator of diagonal k = p + q therefore holds diagonal k in its top half and part of
// diagonal k + 1 in its bottom half, and every pair (p, q) with p + q <= 9 is formed exactly once
// (plus a few of diagonal 10): 20 MMAs of M 128 x N x K 16 per 16 columns of the block.
//
// G records are built once per partition (k_tc_split); the right-hand-side block is gathered,
// waited on and split by the CTA for every item.  One thread issues the MMAs; all four warps read
// TMEM (warp w: lanes 32w .. 32w+31) and combine.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include "common.cuh"
#include "batch.cuh"
#include "tc.cuh"

namespace sptrsv {

constexpr int kTcN = 16;                   // right-hand-side columns per item (the MMA's N, at most)
constexpr int kTcAcc = 8;                  // accumulators: top diagonal k = 2 .. 9
constexpr int kTcCols = kTcAcc * kTcN;     // TMEM columns per CTA
constexpr int kTcRows = 64;                // rows per panel
constexpr size_t kTcTileMax = (size_t)kTcRows * kP64 * 2;           // one digit slice, K = 64
constexpr size_t kTcRecMax = tc::kDigits * kTcTileMax + 64 * 4;   // slices + row exponents
constexpr size_t kTcVTile = (size_t)kTcN * kP64 * 2;
constexpr size_t kTcSmem = kTcRecMax + tc::kDigits * kTcVTile + (size_t)kTcRows * kTcN * 8 + 128;

__host__ __device__ __forceinline__ int tc_kpad(int kc) { return (kc + 15) & ~15; }
__host__ __device__ __forceinline__ size_t tc_rec_bytes(int kc) {
    return (size_t)tc::kDigits * kTcRows * tc_kpad(kc) * 2 + 64 * 4;
}
// Bytes of a panel's G records, and the offset of block `blk`'s record within them.
__host__ __device__ __forceinline__ size_t tc_block_offset(int w, int K, int blk) {
    size_t off = 0;
    for (int q = 0; q < blk; ++q) {
        int k0, kc;
        p64_block(w, K, q, k0, kc);
        off += tc_rec_bytes(kc);
    }
    return off;
}
size_t tc_panel_bytes(int w, int K) { return tc_block_offset(w, K, p64_nblk(w, K)); }
// Right-hand-side columns per item and items per (panel, block).
__host__ __device__ __forceinline__ int tc_group_width(int rhs) { return rhs < kTcN ? rhs : kTcN; }
__host__ __device__ __forceinline__ int tc_groups(int rhs) { return (rhs + kTcN - 1) / kTcN; }
int tc_groups_host(int rhs) { return tc_groups(rhs); }
static int g_panels_mode = -1;
int panels_mode() {
    if (g_panels_mode < 0) {
        const char* e = getenv("SPTRSV_PANELS");
        g_panels_mode = (e && strcmp(e, "tc") == 0) ? 1 : (e && strcmp(e, "df") == 0) ? 2 : 0;
    }
    return g_panels_mode;
}

// G records of every (panel, block) in recs: digit slices in K-major tile layout, row exponents.
__global__ void __launch_bounds__(256) k_tc_split(const BChunk* __restrict__ panels, const int2* __restrict__ recs,
                                                  int nrec) {
    __shared__ int s_exp[kTcRows];
    for (int q = blockIdx.x; q < nrec; q += gridDim.x) {
        const int2 pr = recs[q];
        const BChunk C = panels[pr.x];
        const int K = C.w + C.m;
        int k0, kc;
        p64_block(C.w, K, pr.y, k0, kc);
        const int kcp = tc_kpad(kc);
        unsigned char* rec = C.gtc + tc_block_offset(C.w, K, pr.y);
        const size_t tile = (size_t)kTcRows * kcp * 2;
        if (threadIdx.x < kTcRows) s_exp[threadIdx.x] = tc::kExpZero;
        __syncthreads();
        for (int e = threadIdx.x; e < C.pw * kc; e += blockDim.x) {
            const int r = e / kc, kk = e - r * kc;
            atomicMax(&s_exp[r], tc::exp_bound(C.g64[(size_t)(C.r0 + r) * C.ld + k0 + kk]));
        }
        __syncthreads();
        for (int e = threadIdx.x; e < kTcRows * kcp; e += blockDim.x) {
            const int r = e / kcp, kk = e - r * kcp;
            float d[tc::kDigits];
            if (r < C.pw && kk < kc) {
                tc::digits(C.g64[(size_t)(C.r0 + r) * C.ld + k0 + kk], s_exp[r], d);
            } else {
#pragma unroll
                for (int p = 0; p < tc::kDigits; ++p) d[p] = 0.f;
            }
            const int o = tc::tile_off(r, kk, kcp);
#pragma unroll
            for (int p = 0; p < tc::kDigits; ++p) *(__nv_bfloat16*)(rec + p * tile + o) = __float2bfloat16(d[p]);
        }
        if (threadIdx.x < kTcRows) reinterpret_cast<int*>(rec + tc::kDigits * tile)[threadIdx.x] = s_exp[threadIdx.x];
        __syncthreads();
    }
}

// Work items as in k_panels64 (see panels64.cu), with tc_groups(rhs) groups of up to kTcN columns.
__global__ void __launch_bounds__(128, 2) k_panels_tc(const BSys* __restrict__ sys, int rhs, int ncg,
                                                     const double* __restrict__ bbase, double* xbase, Ctl* ctl,
                                                     unsigned* ticket, int64_t budget, const int2* __restrict__ items,
                                                     unsigned ntickets, const BChunk* __restrict__ panels,
                                                     double* __restrict__ part, int* __restrict__ cnt) {
    extern __shared__ __align__(128) unsigned char tc_smem[];
    unsigned char* sG = tc_smem;                                    // the item's G record
    unsigned char* sV = tc_smem + kTcRecMax;                        // right-hand-side digit tiles
    double* red = reinterpret_cast<double*>(sV + tc::kDigits * kTcVTile);  // bottom-half sums
    __shared__ __align__(8) uint64_t barG, barM;
    __shared__ uint32_t s_tmem;
    __shared__ int s_vexp[kTcN];
    __shared__ unsigned s_t;
    __shared__ int s_ok, s_last;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tc::tmem_alloc(&s_tmem, kTcCols);
    if (tid == 0) {
        tc::mbar_init(&barG, 1);
        tc::mbar_init(&barM, 1);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = s_tmem;
    unsigned phase = 0;  // of both mbarriers: each completes once per tensor-core item
    for (;;) {
        if (tid == 0) s_t = aborted(ctl) ? 0xFFFFFFFFu : atomicAdd(ticket, 1u);
        __syncthreads();
        const unsigned t = s_t;
        __syncthreads();
        if (t >= ntickets) break;
        int2 it;
        int cg;
        if (sys) {
            it = items[t];
            cg = it.y >> 16;
            it.y &= 0xFFFF;
        } else {
            it = items[t / ncg];
            cg = (int)(t % ncg);
        }
        const BChunk C = panels[it.x];
        const int m = sys ? sys[C.sys].rhs : rhs;
        const long long xb0 = sys ? sys[C.sys].xb0 : 0, poff = sys ? C.poff : C.poff * m;
        const int cidx = sys ? C.cbase + cg : C.cbase * ncg + cg;
        const int gw = tc_group_width(m), c0 = cg * gw, nc = min(gw, m - c0);
        constexpr int N = kTcN;  // an M = 128 MMA takes N in multiples of 16; unused columns are zero
        const int a = C.a, w = C.w, K = C.w + C.m, blk = it.y, r0 = C.r0, pw = C.pw;
        int k0, kc;
        p64_block(w, K, blk, k0, kc);
        const int kcp = tc_kpad(kc);
        const unsigned rec_bytes = (unsigned)tc_rec_bytes(kc);
        const double* b = bbase + xb0;
        double* x = xbase + xb0;
        double* pb = part + poff + (long long)blk * pw * m;
        const int no = p64_nown(w), nn = p64_nnear(w, K);
        if (blk >= no && blk < no + nn) {
            // a narrow block next to the dependency chain (the nearest solved rows): FP64 FMAs, as
            // in the FP64 panel kernel -- no digit split, TMEM round trip or record copy on the chain
            double* Gs = reinterpret_cast<double*>(sG);  // pw x kc
            double* Vs = red;                             // kc x nc
            for (int e = tid; e < pw * kc; e += 128) {
                const int r = e / kc, kk = e - r * kc;
                tc::cp_async8(&Gs[e], C.g64 + (size_t)(r0 + r) * C.ld + k0 + kk);
            }
            if (tid == 0) s_ok = 1;
            __syncthreads();
            for (int e = tid; e < kc * nc; e += 128) {
                const int kk = e / nc, j = e - kk * nc, k = k0 + kk;
                double val = k < w ? b[(size_t)(a + k) * m + c0 + j] : ld_relaxed(x + (size_t)C.rect[k - w] * m + c0 + j);
                if (k >= w && Pend<double>::is(val) &&
                    !wait_ready<double>(x + (size_t)C.rect[k - w] * m + c0 + j, val, ctl, budget)) {
                    s_ok = 0;
                    val = 0.0;
                }
                Vs[e] = val;
            }
            tc::cp_async_wait_all();
            if (__syncthreads_or(!s_ok)) break;
            for (int o = tid; o < pw * nc; o += 128) {
                const int r = o / nc, j = o - r * nc;
                double s0 = 0.0, s1 = 0.0;
                int kk = 0;
                for (; kk + 1 < kc; kk += 2) {
                    s0 = fma(Gs[r * kc + kk], Vs[kk * nc + j], s0);
                    s1 = fma(Gs[r * kc + kk + 1], Vs[(kk + 1) * nc + j], s1);
                }
                if (kk < kc) s0 = fma(Gs[r * kc + kk], Vs[kk * nc + j], s0);
                pb[(size_t)r * m + c0 + j] = s0 + s1;
            }
        } else {
            // 1. the G record (digit slices + row exponents), one bulk copy
            if (tid == 0) {
                tc::mbar_expect_tx(&barG, rec_bytes);
                tc::bulk_g2s(sG, C.gtc + tc_block_offset(w, K, blk), rec_bytes, &barG);
                s_ok = 1;
            }
            if (tid < kTcN) s_vexp[tid] = tc::kExpZero;
            __syncthreads();
            // 2. the right-hand-side block (kc x nc), waiting on unsolved rows; column scales; digits
            constexpr int kPer = (kP64 * kTcN + 127) / 128;
            double v[kPer];
#pragma unroll
            for (int u = 0; u < kPer; ++u) {
                const int e = tid + u * 128;
                double val = 0.0;
                if (e < kc * nc) {
                    const int kk = e / nc, j = e - kk * nc, k = k0 + kk;
                    val = k < w ? b[(size_t)(a + k) * m + c0 + j] : ld_relaxed(x + (size_t)C.rect[k - w] * m + c0 + j);
                }
                v[u] = val;
            }
#pragma unroll
            for (int u = 0; u < kPer; ++u) {
                const int e = tid + u * 128;
                if (e < kc * nc) {
                    const int kk = e / nc, j = e - kk * nc, k = k0 + kk;
                    if (k >= w && Pend<double>::is(v[u]) &&
                        !wait_ready<double>(x + (size_t)C.rect[k - w] * m + c0 + j, v[u], ctl, budget)) {
                        s_ok = 0;
                        v[u] = 0.0;
                    }
                    atomicMax(&s_vexp[j], tc::exp_bound(v[u]));
                }
            }
            __syncthreads();
            const size_t vtile = (size_t)N * kcp * 2;
#pragma unroll
            for (int u = 0; u < kPer; ++u) {
                const int e = tid + u * 128;
                if (e < kc * nc) {
                    const int kk = e / nc, j = e - kk * nc;
                    float d[tc::kDigits];
                    tc::digits(v[u], s_vexp[j], d);
                    const int o = tc::tile_off(j, kk, kcp);
#pragma unroll
                    for (int p = 0; p < tc::kDigits; ++p) *(__nv_bfloat16*)(sV + p * vtile + o) = __float2bfloat16(d[p]);
                }
            }
            // zero digits of the padding (columns nc .. N, rows kc .. kcp)
            for (int e = tid; e < N * kcp; e += 128) {
                const int j = e / kcp, kk = e - j * kcp;
                if (j >= nc || kk >= kc) {
                    const int o = tc::tile_off(j, kk, kcp);
#pragma unroll
                    for (int p = 0; p < tc::kDigits; ++p) *(__nv_bfloat16*)(sV + p * vtile + o) = __float2bfloat16(0.f);
                }
            }
            tc::fence_async_smem();
            const bool ok = !__syncthreads_or(!s_ok);
            if (!ok) {
                if (tid == 0) tc::mbar_drain(&barG, phase, budget);  // the copy this CTA started ends first
                break;
            }
            // 3. the MMAs: accumulator k - 2 of the 20 stacked pairs (p odd, q = k - p), once every thread
            //    has seen the G record land (its row exponents are read below)
            {
                const bool got = tc::mbar_wait(&barG, phase, ctl, budget);
                if (!got) {
                    tc::mbar_drain(&barG, phase, budget);
                    s_ok = 0;
                }
            }
            if (__syncthreads_or(!s_ok)) break;
            if (tid == 0) {
                {
                    tc::fence_after();
                    const uint32_t sbo = (uint32_t)kcp * 16;
                    const uint32_t tileA = (uint32_t)kTcRows * kcp * 2;
                    const uint32_t id = tc::idesc_bf16_f32(128, N);
                    const uint32_t gA = tc::smem(sG), gB = tc::smem(sV);
                    for (int k = 2; k <= 9; ++k) {
                        uint32_t acc = 0;
                        for (int p = 1; p <= 7; p += 2) {
                            const int q = k - p;
                            if (q < 1 || q > tc::kDigits) continue;
                            for (int ks = 0; ks < kcp / 16; ++ks) {
                                const uint64_t da = tc::desc(gA + (p - 1) * tileA + ks * 256, 128, sbo);
                                const uint64_t db = tc::desc(gB + (q - 1) * (uint32_t)vtile + ks * 256, 128, sbo);
                                tc::mma_bf16(tmem + (uint32_t)(k - 2) * kTcN, da, db, id, acc);
                                acc = 1;
                            }
                        }
                    }
                    tc::mma_commit(&barM);
                }
            }
            {
                // every thread waits for the MMAs (the wait has its own bound; a timeout is recorded)
                const bool got = tc::mbar_wait(&barM, phase, ctl, budget);
                if (!got) tc::mbar_drain(&barM, phase, budget);
                if (!got) s_ok = 0;
            }
            tc::fence_after();
            // 4. combine the accumulators in FP64: lane R = 32 warp + lane of TMEM, R < 64 the top half
            const int R = 32 * warp + lane;
            const bool top = R < kTcRows;
            const int r = top ? R : R - kTcRows;
            double accd[kTcN];
#pragma unroll
            for (int j = 0; j < kTcN; ++j) accd[j] = 0.0;
            for (int k = 9; k >= 2; --k) {
                float f[16];
                tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(k - 2) * kTcN, f);
                const double sc = ldexp(1.0, -tc::kDigitBits * (top ? k : k + 1));
#pragma unroll
                for (int j = 0; j < kTcN; ++j) accd[j] = fma((double)f[j], sc, accd[j]);
            }
            tc::fence_before();
            if (!top) {
#pragma unroll
                for (int j = 0; j < kTcN; ++j) red[r * kTcN + j] = accd[j];
            }
            if (__syncthreads_or(!s_ok)) break;
            if (top && r < pw) {
                const int er = reinterpret_cast<const int*>(sG + (size_t)tc::kDigits * kTcRows * kcp * 2)[r];
#pragma unroll
                for (int j = 0; j < kTcN; ++j) {
                    if (j < nc) {
                        const int fj = s_vexp[j];
                        const double vsum = accd[j] + red[r * kTcN + j];
                        pb[(size_t)r * m + c0 + j] =
                            (er == tc::kExpZero || fj == tc::kExpZero) ? 0.0 : ldexp(vsum, er + fj);
                    }
                }
            }
            phase ^= 1u;
        }
        __threadfence();  // this thread's partial sums visible before the count moves
        __syncthreads();
        // the last block of the (panel, group) sums the partials in block order and publishes
        if (tid == 0) {
            __threadfence();
            s_last = atomicAdd(&cnt[cidx], 1) == C.nblk - 1;
            if (s_last) __threadfence();
        }
        __syncthreads();
        if (s_last) {
            const double* p0 = part + poff;
            const long long bs = (long long)pw * m;
            for (int o = tid; o < pw * nc; o += blockDim.x) {
                const int rr = o / nc, j = o - rr * nc;
                const double* pr = p0 + (size_t)rr * m + c0 + j;
                double s = 0.0;
                for (int q = 0; q < C.nblk; ++q) s += __ldcg(pr + q * bs);
                st_relaxed(x + (size_t)(a + r0 + rr) * m + c0 + j, Pend<double>::fix(s));
            }
        }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTcCols);
}

int launch_panels_tc(const BSys* sys, int rhs, const double* b, double* x, Ctl* ctl, unsigned* ticket, int64_t budget,
                     const int2* items, unsigned nitems, const BChunk* panels, double* part, int* cnt, int ncnt,
                     int sm_count, cudaStream_t st, int64_t* launches) {
    if (!nitems) return 0;
    const int ncg = sys ? 0 : tc_groups(rhs);
    const unsigned ntickets = sys ? nitems : nitems * (unsigned)ncg;
    static bool configured[64] = {};
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return SPTRSV_ERR_INVALID_ARG;
    if (!configured[dev]) {
        CUDA_TRY(cudaFuncSetAttribute(k_panels_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
        configured[dev] = true;
    }
    CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)ncnt, st));
    const int grid = (int)std::max<long long>(1, std::min<long long>(2ll * sm_count, ntickets));
    k_panels_tc<<<grid, 128, kTcSmem, st>>>(sys, rhs, ncg, b, x, ctl, ticket, budget, items, ntickets, panels, part,
                                             cnt);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_tc_split(const BChunk* panels, const int2* recs, int nrec, int sm_count, cudaStream_t st,
                    int64_t* launches) {
    if (nrec <= 0) return 0;
    k_tc_split<<<std::min(nrec, sm_count * 8), 256, 0, st>>>(panels, recs, nrec);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

}  // namespace sptrsv

extern "C" int sptrsv_set_panels_mode(int mode) {
    if (mode != 0 && mode != 1 && mode != 2) return SPTRSV_ERR_INVALID_ARG;
    const int prev = sptrsv::panels_mode();
    sptrsv::g_panels_mode = mode;
    return prev;
}
