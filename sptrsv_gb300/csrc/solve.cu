// solve.cu -- the direct solve kernels (FP64, and FP32 for the mixed path's inner solve).
//
// Sync-free CSR pull (SYNCFREE_WARP, SYNCFREE_THREAD).  Rows are claimed through an atomic
// ticket in reverse order (n-1 first).  A waiting row only ever waits on rows with smaller
// tickets, which were claimed by warps that are already running, so the spins cannot wait
// on a row no warp holds: the grid needs no co-residency guarantee, and no global barrier
// is used.  x is its own completion flag (see common.cuh).
//   - warp kernel, rhs = 1: 32/LPR rows per warp, LPR lanes per row stride the row with
//     coalesced loads; group-masked shuffle reduction; each lane waits only for its own
//     dependencies.
//   - warp kernel, rhs > 1: one row per warp; lanes = (entry slot, RHS column) pairs with
//     the RHS tile R across lanes (X row-major, so a tile is contiguous in memory).
//   - thread kernel: one lane per row (kernel_full3.cl:14-56 family); each lane walks its
//     row from the right (largest column = earliest solved) and waits entry by entry.
// CSC push (SYNCFREE_CSC, kernel_full.cl:54-228 family): warp per column in reverse; wait
//   until the column's row has received all its contributions (in_degree == 1); compute x_j
//   with the precomputed reciprocal (kernel_full.cl:83,98); push x_j * U_ij into left_sum[i]
//   with FP64 atomics and release-decrement in_degree[i].
// Level-set (LEVELSET, core.cpp:336-370 on the GPU): one persistent cooperative grid walks
//   the levels in order; warps take a level's rows round-robin; a bounded grid barrier
//   separates levels.
#include <cooperative_groups.h>
#include "common.cuh"
#include "kernels.cuh"

namespace sptrsv {

template <typename T>
__global__ void k_fill_pending(T* x, size_t count) {
    const T v = Pend<T>::value();
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x)
        x[k] = v;
}

__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }

template <typename T, int LPR>
__global__ void __launch_bounds__(256) k_pull_warp_v(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                     const T* __restrict__ val, const T* __restrict__ invd,
                                                     const T* __restrict__ b, T* x, Ctl* ctl, int64_t budget) {
    constexpr int RPW = 32 / LPR;
    const int lane = threadIdx.x & 31;
    const int g = lane / LPR, gl = lane % LPR;
    const unsigned gmask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << (g * LPR));
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&ctl->ticket, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if ((long long)t * RPW >= n || aborted(ctl)) break;
        const long long r = (long long)t * RPW + g;
        bool ok = true;
        if (r < n) {
            const int i = n - 1 - (int)r;
            const int s = rp[i], e = rp[i + 1];
            T sum = T(0);
            for (int k = s + 1 + gl; k < e; k += LPR) {
                T xv;
                if (!wait_ready<T>(x + col[k], xv, ctl, budget)) { ok = false; break; }
                sum = fma_t(val[k], xv, sum);
            }
#pragma unroll
            for (int o = LPR / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(gmask, sum, o);
            ok = __all_sync(gmask, ok);
            if (gl == 0 && ok) st_relaxed(x + i, Pend<T>::fix((b[i] - sum) * invd[i]));
        }
        if (__any_sync(0xffffffffu, !ok)) break;
    }
}

template <typename T, int R>
__global__ void __launch_bounds__(256) k_pull_warp_m(int n, int rhs, const int* __restrict__ rp,
                                                     const int* __restrict__ col, const T* __restrict__ val,
                                                     const T* __restrict__ invd, const T* __restrict__ b, T* x,
                                                     Ctl* ctl, int64_t budget) {
    constexpr int Q = 32 / R;
    const int lane = threadIdx.x & 31;
    const int c = lane % R, q = lane / R;
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&ctl->ticket, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= (unsigned)n || aborted(ctl)) break;
        const int i = n - 1 - (int)t;
        const int s = rp[i], e = rp[i + 1];
        const T di = invd[i];
        bool ok = true;
        for (int c0 = 0; c0 < rhs; c0 += R) {
            const int cc = c0 + c;
            T sum = T(0);
            if (cc < rhs && ok) {
                for (int k = s + 1 + q; k < e; k += Q) {
                    T xv;
                    if (!wait_ready<T>(x + (size_t)col[k] * rhs + cc, xv, ctl, budget)) { ok = false; break; }
                    sum = fma_t(val[k], xv, sum);
                }
            }
#pragma unroll
            for (int o = 16; o >= R; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
            ok = __all_sync(0xffffffffu, ok);
            if (q == 0 && cc < rhs && ok) {
                const size_t p = (size_t)i * rhs + cc;
                st_relaxed(x + p, Pend<T>::fix((b[p] - sum) * di));
            }
        }
        if (!ok) break;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_pull_thread(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                     const T* __restrict__ val, const T* __restrict__ invd,
                                                     const T* __restrict__ b, T* x, Ctl* ctl, int64_t budget) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&ctl->ticket, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if ((long long)t * 32 >= n || aborted(ctl)) break;
        const long long r = (long long)t * 32 + lane;
        bool ok = true;
        if (r < n) {
            const int i = n - 1 - (int)r;
            const int s = rp[i], e = rp[i + 1];
            T sum = T(0);
            for (int k = e - 1; k > s; --k) {
                T xv;
                if (!wait_ready<T>(x + col[k], xv, ctl, budget)) { ok = false; break; }
                sum = fma_t(val[k], xv, sum);
            }
            if (ok) st_relaxed(x + i, Pend<T>::fix((b[i] - sum) * invd[i]));
        }
        if (__any_sync(0xffffffffu, !ok)) break;
    }
}

// Block sync-free (SYNCFREE_BLOCK): a CTA claims a block of kBsfRows consecutive rows (blocks in
// decreasing order through the ticket) and solves it with one thread per row, each walking its
// row from the right.  The block's own x values live in shared memory, so a dependency inside
// the block is a shared-memory poll (~90 ns on this GPU) instead of an L2 round trip (~375 ns);
// dependencies on higher blocks use the self-flagging global x.  Forward progress: a block only
// waits on higher blocks (claimed earlier by running CTAs) and on higher rows of its own block
// (threads of the same CTA, which never wait on lower rows).  The final update is a single FMA
// with b_i * invd_i precomputed, which shortens the FP64 chain after the last dependency.
constexpr int kBsfRows = 512;

template <typename T>
__global__ void __launch_bounds__(kBsfRows) k_bsf(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                  const T* __restrict__ val, const T* __restrict__ invd,
                                                  const T* __restrict__ b, T* x, Ctl* ctl, int64_t budget) {
    __shared__ T xs[kBsfRows];
    __shared__ unsigned s_ticket;
    const int nblk = (n + kBsfRows - 1) / kBsfRows;
    for (;;) {
        // thread 0 decides for the whole CTA (a uniform exit keeps the barriers matched)
        if (threadIdx.x == 0) s_ticket = aborted(ctl) ? 0xFFFFFFFFu : atomicAdd(&ctl->ticket, 1u);
        __syncthreads();
        const unsigned t = s_ticket;
        if (t >= (unsigned)nblk) break;
        const int blk = nblk - 1 - (int)t;
        const int lo = blk * kBsfRows, hi = min(n, lo + kBsfRows);
        xs[threadIdx.x] = Pend<T>::value();
        __syncthreads();
        const int i = hi - 1 - (int)threadIdx.x;  // thread 0 takes the block's highest row
        bool ok = true, done = i < lo;
        int k = 0, s = 0;
        T sum = T(0), di = T(0), bd = T(0);
        if (!done) {
            s = rp[i];
            k = rp[i + 1] - 1;
            di = invd[i];
            bd = b[i] * di;
            // phase 1: entries in higher blocks (rightmost in the row) through the global x
            for (; k > s; --k) {
                const int c = col[k];
                if (c < hi) break;
                T xv;
                if (!wait_ready<T>(x + c, xv, ctl, budget)) { ok = false; break; }
                sum = fma_t(val[k], xv, sum);
            }
        }
        // phase 2: entries inside the block, in warp lockstep: every lane consumes whatever is
        // ready, then the warp polls again together (no lane spins alone in divergent code)
        const uint64_t t0 = gtimer();
        unsigned iter = 0;
        if (!ok) done = true;
        while (!__all_sync(0xffffffffu, done)) {
            if (!done) {
                for (; k > s; --k) {
                    const T xv = ((volatile T*)xs)[col[k] - lo];
                    if (Pend<T>::is(xv)) break;
                    sum = fma_t(val[k], xv, sum);
                }
                if (k == s) {
                    const T xi = Pend<T>::fix(fma_t(-sum, di, bd));
                    ((volatile T*)xs)[i - lo] = xi;
                    st_relaxed(x + i, xi);
                    done = true;
                }
            }
            if ((++iter & 255u) == 0) {
                if (aborted(ctl)) { ok = false; done = true; }
                else if ((int64_t)(gtimer() - t0) > budget) {
                    record_error(ctl, SPTRSV_ERR_TIMEOUT);
                    ok = false;
                    done = true;
                }
            }
        }
        if (__syncthreads_or(!ok)) break;
    }
}

__global__ void __launch_bounds__(256) k_push_csc(int n, int rhs, const int* __restrict__ cp,
                                                  const int* __restrict__ crow, const double* __restrict__ cval,
                                                  const double* __restrict__ invd, const double* __restrict__ b,
                                                  double* x, int* indeg, double* left, Ctl* ctl, int64_t budget) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&ctl->ticket, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= (unsigned)n || aborted(ctl)) break;
        const int j = n - 1 - (int)t;
        int ok = 1;
        if (lane == 0) ok = wait_equal(indeg + j, 1, ctl, budget) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) break;
        (void)ld_acquire(indeg + j);  // each lane synchronises with the producers
        const int s = cp[j], e = cp[j + 1] - 1;  // e: the diagonal, last in the column
        const double coef = invd[j];
        if (rhs == 1) {
            double xj = 0.0;
            if (lane == 0) {
                xj = (b[j] - ld_relaxed(left + j)) * coef;
                x[j] = xj;
            }
            xj = __shfl_sync(0xffffffffu, xj, 0);
            for (int k = s + lane; k < e; k += 32) {
                const int i = crow[k];
                atomicAdd(left + i, xj * cval[k]);
                red_release_add(indeg + i, -1);
            }
        } else {
            for (int c = lane; c < rhs; c += 32) {
                const size_t p = (size_t)j * rhs + c;
                x[p] = (b[p] - ld_relaxed(left + p)) * coef;
            }
            for (int k = s; k < e; ++k) {
                const int i = crow[k];
                const double v = cval[k];
                for (int c = lane; c < rhs; c += 32) atomicAdd(left + (size_t)i * rhs + c, x[(size_t)j * rhs + c] * v);
                __syncwarp();
                if (lane == 0) {
                    __threadfence();
                    atomicSub(indeg + i, 1);
                }
            }
        }
    }
}

template <typename T>
__device__ __forceinline__ T ldcg(const T* p) { return __ldcg(p); }

constexpr int kLevelsetThreads = 1024;  // one CTA per SM: a grid barrier takes one arrival per SM

template <typename T>
__global__ void __launch_bounds__(kLevelsetThreads, 1) k_levelset(int n, int rhs, const int* __restrict__ rp, const int* __restrict__ col,
                                                  const T* __restrict__ val, const T* __restrict__ invd,
                                                  const T* __restrict__ b, T* x, int max_level,
                                                  const int* __restrict__ lptr, const int* __restrict__ lrows,
                                                  Ctl* ctl, int64_t budget) {
    if (*(volatile const int*)&ctl->done) return;  // refinement already converged (grid-uniform)
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    if (rhs == 1) {
        // The matrix data of this warp's first row of a level (row index, row pointers, the first
        // kPre x 32 entries, b_i and 1/U_ii) is loaded before the barrier that opens the level, so
        // after the barrier a row waits only for its loads of x.
        constexpr int kPre = 2;
        int i = -1, s = 0, e = 0;
        int pc[kPre];
        T pv[kPre], pb = T(0), pd = T(0);
        auto fetch = [&](int l) {
            i = -1;
            const int k = lptr[l] + gw;
            if (k >= lptr[l + 1]) return;
            i = lrows[k];
            s = rp[i] + 1;
            e = rp[i + 1];
#pragma unroll
            for (int u = 0; u < kPre; ++u) {
                const int q = s + lane + 32 * u;
                pc[u] = q < e ? col[q] : 0;
                pv[u] = q < e ? val[q] : T(0);
            }
            pb = b[i];
            pd = invd[i];
        };
        fetch(1);
        // x of earlier levels: through L2 (written by other SMs), or through L1 when the grid is one
        // CTA (its own stores, ordered by the CTA barrier)
        const bool one = gridDim.x == 1;
        auto ldx = [&](int c) -> T { return one ? x[c] : ldcg(x + c); };
        for (int l = 1; l <= max_level; ++l) {
            if (i >= 0) {
                T sum = T(0);
#pragma unroll
                for (int u = 0; u < kPre; ++u)
                    if (s + lane + 32 * u < e) sum = fma_t(pv[u], ldx(pc[u]), sum);
                for (int q = s + 32 * kPre + lane; q < e; q += 32) sum = fma_t(val[q], ldx(col[q]), sum);
                sum = warp_sum(sum);
                if (lane == 0) x[i] = (pb - sum) * pd;
                // more rows of this level for this warp (levels wider than the grid's warps)
                for (int k = lptr[l] + gw + nw; k < lptr[l + 1]; k += nw) {
                    const int r = lrows[k];
                    T t = T(0);
                    for (int q = rp[r] + 1 + lane; q < rp[r + 1]; q += 32) t = fma_t(val[q], ldx(col[q]), t);
                    t = warp_sum(t);
                    if (lane == 0) x[r] = (b[r] - t) * invd[r];
                }
            }
            if (l < max_level) {
                fetch(l + 1);
                if (!grid_barrier(ctl, gridDim.x, budget)) return;
            }
        }
        return;
    }
    for (int l = 1; l <= max_level; ++l) {
        const int beg = lptr[l], end = lptr[l + 1];
        for (int k = beg + gw; k < end; k += nw) {
            const int i = lrows[k];
            const int s = rp[i], e = rp[i + 1];
            const T di = invd[i];
            for (int c = lane; c < rhs; c += 32) {
                T sum = T(0);
                for (int q = s + 1; q < e; ++q) sum = fma_t(val[q], ldcg(x + (size_t)col[q] * rhs + c), sum);
                const size_t p = (size_t)i * rhs + c;
                x[p] = (b[p] - sum) * di;
            }
        }
        if (l < max_level && !grid_barrier(ctl, gridDim.x, budget)) return;
    }
}

__global__ void k_to_row_major(const double* __restrict__ src, double* __restrict__ dst, int n, int rhs) {
    const size_t total = (size_t)n * rhs;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total; p += (size_t)gridDim.x * blockDim.x) {
        const size_t i = p / rhs, c = p % rhs;
        dst[p] = src[i + c * (size_t)n];
    }
}
__global__ void k_to_col_major(const double* __restrict__ src, double* __restrict__ dst, int n, int rhs) {
    const size_t total = (size_t)n * rhs;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total; p += (size_t)gridDim.x * blockDim.x) {
        const size_t i = p % n, c = p / n;
        dst[p] = src[i * rhs + c];
    }
}

// ---------------------------------------------------------------------------------------
static int grid_for(const void* fn, int block, int sm_count, int warps) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
    int full = per_sm * sm_count;
    if (warps > 0) {
        int want = (warps * 32 + block - 1) / block;
        if (want < full) full = want < 1 ? 1 : want;
    }
    return full;
}

int launch_fill_pending(bool f32, void* x, size_t count, cudaStream_t st, int64_t* launches) {
    if (count == 0) return 0;
    const int blocks = (int)std::min<size_t>((count + 255) / 256, 4096);
    if (f32) k_fill_pending<float><<<blocks, 256, 0, st>>>((float*)x, count);
    else k_fill_pending<double><<<blocks, 256, 0, st>>>((double*)x, count);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

template <typename T>
static int pull_warp_t(const SolveArgs& a, int rows_per_warp, int rhs_tile) {
    const T* val = (const T*)a.val;
    const T* invd = (const T*)a.invd;
    const T* b = (const T*)a.b;
    T* x = (T*)a.x;
    const void* fn;
    if (a.rhs == 1) {
        switch (rows_per_warp) {
            case 2: fn = (const void*)k_pull_warp_v<T, 16>; break;
            case 4: fn = (const void*)k_pull_warp_v<T, 8>; break;
            case 8: fn = (const void*)k_pull_warp_v<T, 4>; break;
            case 16: fn = (const void*)k_pull_warp_v<T, 2>; break;
            default: fn = (const void*)k_pull_warp_v<T, 32>; break;
        }
        const int grid = grid_for(fn, 256, a.sm_count, a.warps);
        void* args[] = {(void*)&a.n, (void*)&a.rp, (void*)&a.col, (void*)&val, (void*)&invd, (void*)&b, (void*)&x,
                        (void*)&a.ctl, (void*)&a.budget};
        CUDA_TRY(cudaLaunchKernel(fn, grid, 256, args, 0, a.st));
    } else {
        int R = rhs_tile > 0 ? rhs_tile : a.rhs;
        int p2 = 1;
        while (p2 < R && p2 < 32) p2 <<= 1;
        switch (p2) {
            case 1: fn = (const void*)k_pull_warp_m<T, 1>; break;
            case 2: fn = (const void*)k_pull_warp_m<T, 2>; break;
            case 4: fn = (const void*)k_pull_warp_m<T, 4>; break;
            case 8: fn = (const void*)k_pull_warp_m<T, 8>; break;
            case 16: fn = (const void*)k_pull_warp_m<T, 16>; break;
            default: fn = (const void*)k_pull_warp_m<T, 32>; break;
        }
        const int grid = grid_for(fn, 256, a.sm_count, a.warps);
        void* args[] = {(void*)&a.n, (void*)&a.rhs, (void*)&a.rp, (void*)&a.col, (void*)&val, (void*)&invd,
                        (void*)&b, (void*)&x, (void*)&a.ctl, (void*)&a.budget};
        CUDA_TRY(cudaLaunchKernel(fn, grid, 256, args, 0, a.st));
    }
    ++*a.launches;
    return 0;
}

int launch_pull_warp(bool f32, const SolveArgs& a, int rows_per_warp, int rhs_tile) {
    return f32 ? pull_warp_t<float>(a, rows_per_warp, rhs_tile) : pull_warp_t<double>(a, rows_per_warp, rhs_tile);
}

template <typename T>
static int pull_thread_t(const SolveArgs& a) {
    const void* fn = (const void*)k_pull_thread<T>;
    const int grid = grid_for(fn, 256, a.sm_count, a.warps);
    const T* val = (const T*)a.val;
    const T* invd = (const T*)a.invd;
    const T* b = (const T*)a.b;
    T* x = (T*)a.x;
    void* args[] = {(void*)&a.n, (void*)&a.rp, (void*)&a.col, (void*)&val, (void*)&invd, (void*)&b, (void*)&x,
                    (void*)&a.ctl, (void*)&a.budget};
    CUDA_TRY(cudaLaunchKernel(fn, grid, 256, args, 0, a.st));
    ++*a.launches;
    return 0;
}

int launch_pull_thread(bool f32, const SolveArgs& a) {
    if (a.rhs != 1) return SPTRSV_ERR_UNSUPPORTED;
    return f32 ? pull_thread_t<float>(a) : pull_thread_t<double>(a);
}

template <typename T>
static int bsf_t(const SolveArgs& a) {
    const void* fn = (const void*)k_bsf<T>;
    const int nblk = (a.n + kBsfRows - 1) / kBsfRows;
    int grid = grid_for(fn, kBsfRows, a.sm_count, a.warps);
    if (grid > nblk) grid = nblk;
    const T* val = (const T*)a.val;
    const T* invd = (const T*)a.invd;
    const T* b = (const T*)a.b;
    T* x = (T*)a.x;
    void* args[] = {(void*)&a.n, (void*)&a.rp, (void*)&a.col, (void*)&val, (void*)&invd, (void*)&b, (void*)&x,
                    (void*)&a.ctl, (void*)&a.budget};
    CUDA_TRY(cudaLaunchKernel(fn, grid, kBsfRows, args, 0, a.st));
    ++*a.launches;
    return 0;
}

int launch_bsf(bool f32, const SolveArgs& a) {
    if (a.rhs != 1) return SPTRSV_ERR_UNSUPPORTED;
    return f32 ? bsf_t<float>(a) : bsf_t<double>(a);
}

int launch_push_csc(const SolveArgs& a, const int* cp, const int* crow, const double* cval, int* indeg_work,
                    double* left_sum) {
    const void* fn = (const void*)k_push_csc;
    const int grid = grid_for(fn, 256, a.sm_count, a.warps);
    const double* invd = (const double*)a.invd;
    const double* b = (const double*)a.b;
    double* x = (double*)a.x;
    void* args[] = {(void*)&a.n, (void*)&a.rhs, (void*)&cp, (void*)&crow, (void*)&cval, (void*)&invd, (void*)&b,
                    (void*)&x, (void*)&indeg_work, (void*)&left_sum, (void*)&a.ctl, (void*)&a.budget};
    CUDA_TRY(cudaLaunchKernel(fn, grid, 256, args, 0, a.st));
    ++*a.launches;
    return 0;
}

template <typename T>
static int levelset_t(const SolveArgs& a, int max_level, const int* lptr, const int* lrows) {
    const void* fn = (const void*)k_levelset<T>;
    int per_sm = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kLevelsetThreads, 0));
    if (per_sm < 1) return SPTRSV_ERR_UNSUPPORTED;
    int grid = a.sm_count;  // one CTA per SM (co-resident: per_sm >= 1)
    if (a.warps > 0) grid = std::max(1, std::min(grid, (a.warps * 32 + kLevelsetThreads - 1) / kLevelsetThreads));
    const T* val = (const T*)a.val;
    const T* invd = (const T*)a.invd;
    const T* b = (const T*)a.b;
    T* x = (T*)a.x;
    void* args[] = {(void*)&a.n, (void*)&a.rhs, (void*)&a.rp, (void*)&a.col, (void*)&val, (void*)&invd, (void*)&b,
                    (void*)&x, (void*)&max_level, (void*)&lptr, (void*)&lrows, (void*)&a.ctl, (void*)&a.budget};
    CUDA_TRY(cudaLaunchCooperativeKernel(fn, grid, kLevelsetThreads, args, 0, a.st));
    ++*a.launches;
    return 0;
}

int launch_levelset(bool f32, const SolveArgs& a, int max_level, const int* lptr, const int* lrows) {
    return f32 ? levelset_t<float>(a, max_level, lptr, lrows) : levelset_t<double>(a, max_level, lptr, lrows);
}

int launch_transpose(bool to_row_major, const double* src, double* dst, int n, int rhs, cudaStream_t st,
                     int64_t* launches) {
    const size_t total = (size_t)n * rhs;
    if (total == 0) return 0;
    const int blocks = (int)std::min<size_t>((total + 255) / 256, 8192);
    if (to_row_major) k_to_row_major<<<blocks, 256, 0, st>>>(src, dst, n, rhs);
    else k_to_col_major<<<blocks, 256, 0, st>>>(src, dst, n, rhs);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

}  // namespace sptrsv
