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
__global__ void __launch_bounds__(128, 8) k_panels64(const BSys* __restrict__ sys, int rhs, int ncg,
                                                  const double* __restrict__ bbase, double* xbase, Ctl* ctl,
                                                  unsigned* ticket, int64_t budget, const int2* __restrict__ items,
                                                  unsigned ntickets, const BChunk* __restrict__ panels,
                                                  double* __restrict__ part, int* __restrict__ cnt) {
    __shared__ double Gs[kP64][kP64 + 1];
    __shared__ double Vs[kP64][kP64Nc + 1];
    __shared__ unsigned s_t;
    __shared__ int s_ok, s_last;
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
            cp_async8(&Gs[r][kk], C.g64 + (size_t)(r0 + r) * L + k0 + kk);
        }
        if (threadIdx.x == 0) s_ok = 1;
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
                }
            }
        }
        cp_async_wait_all();
        __syncthreads();
        const bool ok = s_ok;
        if (ok) {
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
