// panels64.cu -- exact FP64 products over dense panels, each panel's product split into column
// blocks taken by different CTAs (used by the batched path and the single-system supernodal path).
#include <algorithm>
#include "common.cuh"
#include "batch.cuh"

namespace sptrsv {

// 8-byte global -> shared copies that complete asynchronously (no register staging), so a tile's
// loads are all in flight together and overlap the waits on the right-hand side.
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Double-FP32 ("df") products: FP32 pipes run 64 times the FP64 rate on this part.  Each G entry is
// stored as an unevaluated FP32 pair hi + lo (48 significant bits) of g 2^-e_r, e_r the row's
// exponent bound; each right-hand-side value likewise against its column's bound for the item.
// A product term a b adds hi_a hi_b exactly split (p + e, with e from an FMA: Dekker's product)
// plus the cross terms hi_a lo_b + lo_a hi_b into e, and p into a compensated running sum (Knuth's
// TwoSum, the Dot2 scheme of Ogita, Rump and Oishi 2005): the sum is as accurate as one computed
// with 48-bit products in twice the working precision, then rounded -- FP64 quality for these
// dot products, since FP64 summation itself loses up to K 2^-53 of sum |a b|.  __fmul_rn and
// __fadd_rn keep the compiler from contracting the error-free transformations into FMAs.
__device__ __forceinline__ int df_exp_bound(double g) {
    // smallest e with |g| < 2^e (g finite); -2000 for g == 0
    const unsigned long long b = (unsigned long long)__double_as_longlong(g) & 0x7FFFFFFFFFFFFFFFull;
    if (b == 0) return -2000;
    const int E = (int)(b >> 52);
    if (E == 0) return -1074 + 64 - __clzll((long long)b);  // subnormal: bits above the lowest
    return E - 1022;
}
__device__ __forceinline__ float2 df_split(double g) {
    const float hi = __double2float_rn(g);
    return make_float2(hi, __double2float_rn(g - (double)hi));
}
__device__ __forceinline__ void df_term(float2 a, float2 b, float& s, float& c) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    const float t = __fadd_rn(s, p);
    const float z = __fadd_rn(t, -s);
    const float q = __fadd_rn(__fadd_rn(s, -__fadd_rn(t, -z)), __fadd_rn(p, -z));
    s = t;
    c = __fadd_rn(c, __fadd_rn(q, e));
}

// Work item (panel, block, RHS group): the block's columns of G times the matching rows of
// [b ; x_R] for one group of right-hand-side columns (waiting on solved rows), written to the
// panel's partial-sum slot for that block.  The CTA that completes the last block of a (panel,
// group) sums the partials in block order (deterministic) and publishes those rows and columns of
// x.  Splitting the RHS columns over items keeps the FP64 work on the dependency chain (the nearest
// block's product and the final sum, each on one SM) short.  Blocks of a panel depend only on
// rows of later chunks, whose items hold smaller tickets, so the ticket order guarantees progress.
//
// Batched (sys != nullptr): items[t] = {panel, block | group << 16}, one per ticket; the panel's
// poff and cbase are absolute.  One system (sys == nullptr, `rhs` columns at offset 0): ticket t is
// group t % ncg of item t / ncg, and poff and cbase count per column and per group.
// One thread's double-FP32 outputs: row r, columns jb + 2u (u < J), over the item's kc columns of G.
template <int J>
__device__ __forceinline__ void df_row(const float2* G2, const float2* V2, int r, int jb, int kc, int nc, int er,
                                       const int* vexp, double* pb, int m, int c0) {
    float sa[J], ca[J];
#pragma unroll
    for (int u = 0; u < J; ++u) sa[u] = ca[u] = 0.f;
    for (int kk = 0; kk < kc; ++kk) {
        const float2 g = G2[r * (kP64 + 1) + kk];
#pragma unroll
        for (int u = 0; u < J; ++u) df_term(g, V2[kk * (kP64Nc + 1) + jb + 2 * u], sa[u], ca[u]);
    }
#pragma unroll
    for (int u = 0; u < J; ++u) {
        const int j = jb + 2 * u;
        if (j < nc) {
            const int f = vexp[j];
            pb[(size_t)r * m + c0 + j] = (er == -2000 || f == -2000) ? 0.0 : ldexp((double)sa[u] + (double)ca[u], er + f);
        }
    }
}

__global__ void __launch_bounds__(128, 8) k_panels64(const BSys* __restrict__ sys, int rhs, int ncg,
                                                  const double* __restrict__ bbase, double* xbase, Ctl* ctl,
                                                  unsigned* ticket, int64_t budget, const int2* __restrict__ items,
                                                  unsigned ntickets, const BChunk* __restrict__ panels,
                                                  double* __restrict__ part, int* __restrict__ cnt) {
    __shared__ double Gs[kP64][kP64 + 1];
    __shared__ double Vs[kP64][kP64Nc + 1];
    __shared__ unsigned s_t;
    __shared__ int s_ok, s_last;
    __shared__ int s_vexp[kP64Nc];  // double-FP32 panels: the item's column exponent bounds
    for (;;) {
        if (threadIdx.x == 0) s_t = aborted(ctl) ? 0xFFFFFFFFu : atomicAdd(ticket, 1u);
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
        const bool df = C.ghl != nullptr;  // double-FP32 products for this panel
        const int gw = p64_group_width(m), c0 = cg * gw, nc = min(gw, m - c0);
        const int a = C.a, w = C.w, K = C.w + C.m, L = C.ld, blk = it.y, r0 = C.r0, pw = C.pw;
        int k0, kc;
        p64_block(w, K, blk, k0, kc);
        const double* b = bbase + xb0;
        double* x = xbase + xb0;
        double* pb = part + poff + (long long)blk * pw * m;
        // the block of G (the panel's rows, columns k0 .. k0+kc), copied asynchronously while the
        // right-hand side below is gathered and waited on
        for (int e = threadIdx.x; e < pw * kc; e += blockDim.x) {
            const int r = e / kc, kk = e - r * kc;
            const size_t g = (size_t)(r0 + r) * L + k0 + kk;
            cp_async8(&Gs[r][kk], df ? (const void*)(C.ghl + g) : (const void*)(C.g64 + g));
        }
        if (threadIdx.x == 0) s_ok = 1;
        if (threadIdx.x < kP64Nc) s_vexp[threadIdx.x] = -2000;
        __syncthreads();
        // eight loads per thread in flight together, then waits only on pending values
        constexpr int kStage = 8;
        for (int base = 0; base < kc * nc; base += 128 * kStage) {
            double v[kStage];
#pragma unroll
            for (int u = 0; u < kStage; ++u) {
                const int e = base + threadIdx.x + u * 128;
                double val = 0.0;
                if (e < kc * nc) {
                    const int kk = e / nc, j = e - kk * nc, k = k0 + kk;
                    val = k < w ? b[(size_t)(a + k) * m + c0 + j] : ld_relaxed(x + (size_t)C.rect[k - w] * m + c0 + j);
                }
                v[u] = val;
            }
#pragma unroll
            for (int u = 0; u < kStage; ++u) {
                const int e = base + threadIdx.x + u * 128;
                if (e < kc * nc) {
                    const int kk = e / nc, j = e - kk * nc, k = k0 + kk;
                    double val = v[u];
                    if (k >= w && Pend<double>::is(val) &&
                        !wait_ready<double>(x + (size_t)C.rect[k - w] * m + c0 + j, val, ctl, budget)) {
                        s_ok = 0;
                        val = 0.0;
                    }
                    Vs[kk][j] = val;
                    if (df) atomicMax(&s_vexp[j], df_exp_bound(val));
                }
            }
        }
        cp_async_wait_all();
        __syncthreads();
        const bool ok = s_ok;
        if (ok && df) {
            // the right-hand side scaled by its columns' bounds and split, in place (8 bytes each)
            float2* V2 = reinterpret_cast<float2*>(&Vs[0][0]);
            for (int e = threadIdx.x; e < kc * nc; e += blockDim.x) {
                const int kk = e / nc, j = e - kk * nc;
                const int f = s_vexp[j];
                const double v = Vs[kk][j];
                V2[kk * (kP64Nc + 1) + j] = df_split(f == -2000 ? 0.0 : ldexp(v, -f));
            }
            __syncthreads();
            // thread: row r of the panel, columns jb, jb + 2, ...; one G load serves its columns
            const float2* G2 = reinterpret_cast<const float2*>(&Gs[0][0]);
            const int r = threadIdx.x & (kP64 - 1), jb = threadIdx.x >> 6;
            if (r < pw) {
                const int er = C.gexp[r0 + r];
                if (nc <= 2) df_row<1>(G2, V2, r, jb, kc, nc, er, s_vexp, pb, m, c0);
                else if (nc <= 4) df_row<2>(G2, V2, r, jb, kc, nc, er, s_vexp, pb, m, c0);
                else if (nc <= 8) df_row<4>(G2, V2, r, jb, kc, nc, er, s_vexp, pb, m, c0);
                else df_row<kP64Nc / 2>(G2, V2, r, jb, kc, nc, er, s_vexp, pb, m, c0);
            }
        } else if (ok) {
            for (int o = threadIdx.x; o < pw * nc; o += blockDim.x) {
                const int r = o / nc, j = o - r * nc;
                double s0 = 0.0, s1 = 0.0;
                int kk = 0;
                for (; kk + 1 < kc; kk += 2) {
                    s0 = fma(Gs[r][kk], Vs[kk][j], s0);
                    s1 = fma(Gs[r][kk + 1], Vs[kk + 1][j], s1);
                }
                if (kk < kc) s0 = fma(Gs[r][kk], Vs[kk][j], s0);
                pb[(size_t)r * m + c0 + j] = s0 + s1;
            }
        }
        __threadfence();  // this thread's partial sums visible before the count moves
        if (__syncthreads_or(!ok)) break;
        // the last block of the (panel, group) sums the partials in block order and publishes
        if (threadIdx.x == 0) {
            __threadfence();
            s_last = atomicAdd(&cnt[cidx], 1) == C.nblk - 1;
            if (s_last) __threadfence();
        }
        __syncthreads();
        if (s_last) {
            const double* p0 = part + poff;
            const long long bs = (long long)pw * m;
            for (int o = threadIdx.x; o < pw * nc; o += blockDim.x) {
                const int r = o / nc, j = o - r * nc;
                const double* pr = p0 + (size_t)r * m + c0 + j;
                // eight partials loaded together, then added in block order
                double v = 0.0;
                int q = 0;
                for (; q + 8 <= C.nblk; q += 8) {
                    double t[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) t[u] = __ldcg(pr + (q + u) * bs);
#pragma unroll
                    for (int u = 0; u < 8; ++u) v += t[u];
                }
                for (; q < C.nblk; ++q) v += __ldcg(pr + q * bs);
                st_relaxed(x + (size_t)(a + r0 + r) * m + c0 + j, Pend<double>::fix(v));
            }
        }
    }
}

// Double-FP32 G of every panel: row r's exponent bound e_r (over all its columns), then hi + lo of
// g 2^-e_r for each of its K = w + m entries, laid out like g64.
__global__ void __launch_bounds__(256) k_g_df(const BChunk* __restrict__ panels, int npanels) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int q = blockIdx.x; q < npanels; q += gridDim.x) {
        const BChunk C = panels[q];
        const int K = C.w + C.m;
        for (int r = warp; r < C.pw; r += 8) {
            const size_t row = (size_t)(C.r0 + r) * C.ld;
            int e = -2000;
            for (int k = lane; k < K; k += 32) e = max(e, df_exp_bound(C.g64[row + k]));
            for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
            float2* out = const_cast<float2*>(C.ghl) + row;
            for (int k = lane; k < K; k += 32) out[k] = df_split(e == -2000 ? 0.0 : ldexp(C.g64[row + k], -e));
            if (lane == 0) const_cast<int*>(C.gexp)[C.r0 + r] = e;
        }
    }
}

int launch_g_df(const BChunk* panels, int npanels, cudaStream_t st, int64_t* launches) {
    if (npanels <= 0) return 0;
    k_g_df<<<std::min(npanels, 65535), 256, 0, st>>>(panels, npanels);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_panels64(const BSys* sys, int rhs, const double* b, double* x, Ctl* ctl, unsigned* ticket, int64_t budget,
                    const int2* items, unsigned nitems, const BChunk* panels, double* part, int* cnt, int ncnt,
                    int ctas_per_sm, int sm_count, cudaStream_t st, int64_t* launches) {
    if (!nitems) return 0;
    const int ncg = sys ? 0 : p64_groups(rhs);
    const unsigned ntickets = sys ? nitems : nitems * (unsigned)ncg;
    CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)ncnt, st));
    int per_sm = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_panels64, 128, 0));
    per_sm = std::max(1, std::min(per_sm, ctas_per_sm));
    const int grid = (int)std::max<long long>(1, std::min<long long>((long long)per_sm * sm_count, ntickets));
    k_panels64<<<grid, 128, 0, st>>>(sys, rhs, ncg, b, x, ctl, ticket, budget, items, ntickets, panels, part, cnt);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

}  // namespace sptrsv
