// refine.cu -- FP32 bulk solves with FP64 iterative refinement.
//
// One refinement step, all on the device (no host round trip, so the whole solve is one
// CUDA graph launch):
//   r   = b - U x               FP64 SpMV over the FP64 values (k_residual_*); ||r_c||^2 per
//                               column for the convergence test; r is also stored in FP32 as
//                               the inner right-hand side, and d0 = D^-1 r seeds the sweeps;
//   test                        rel = max_c ||r_c|| / ||b_c||; once rel <= tol the `done` flag
//                               is raised (flat graphs: every later kernel returns at once;
//                               conditional graphs: the outer WHILE node stops);
//   d  ~= U^{-1} r              FP32 inner solve, either
//                                 JACOBI: d <- D^-1 (r - N d) sweeps over an interleaved
//                                 (column, FP32 value) copy of the off-diagonals, until the
//                                 largest change is below max(10^-e, 0.1 tol / rel) of the
//                                 largest |d| (the inner WHILE node) -- fully parallel; it
//                                 converges for any triangular U because N is nilpotent, and
//                                 fast when U is diagonally dominant -- or
//                                 an exact FP32 sync-free / level-set solve (solve.cu);
//   x  += d                     FP64 update.
// x starts at 0, so the first residual is b itself.
//
// Short rows: the FP64 residual uses warp tiles of 32 consecutive rows (the warp copies the
// tile's entries into shared memory with coalesced loads, then each lane sums its own row in
// order: deterministic; tiles with more than kTileMax entries read straight from global memory);
// the default Jacobi sweep gives each lane a row of the paired layout (16-byte loads of two
// entries).  Long-row matrices use the warp-per-row kernels (LPR lanes per row).
#include "common.cuh"
#include "kernels.cuh"

namespace sptrsv {

constexpr int kTileMax = 512;   // staged entries per warp
constexpr int kJacWarps = 8;    // warps per block, Jacobi tile kernel (4 KiB stage per warp)
constexpr int kResWarps = 4;    // warps per block, residual tile kernel (6 KiB stage per warp)

__device__ __forceinline__ bool is_done(const Ctl* ctl) { return *(volatile const int*)&ctl->done != 0; }

// ||b_c||^2 for row-major b (rhs <= 1024).
__global__ void k_colnorm2(int n, int rhs, const double* __restrict__ b, double* __restrict__ out) {
    extern __shared__ double acc[];
    for (int c = threadIdx.x; c < rhs; c += blockDim.x) acc[c] = 0.0;
    __syncthreads();
    const int per_pass = (blockDim.x / rhs) > 0 ? (blockDim.x / rhs) : 0;
    if (rhs == 1) {
        double s = 0.0;
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
            const double v = b[i];
            s += v * v;
        }
        s = warp_sum(s);
        if ((threadIdx.x & 31) == 0) atomicAdd(&acc[0], s);
    } else if (per_pass > 0 && (int)threadIdx.x < per_pass * rhs) {
        const int c = threadIdx.x % rhs, r0 = threadIdx.x / rhs;
        double s = 0.0;
        for (long long i = (long long)blockIdx.x * per_pass + r0; i < n; i += (long long)gridDim.x * per_pass) {
            const double v = b[i * rhs + c];
            s += v * v;
        }
        atomicAdd(&acc[c], s);
    } else if (per_pass == 0) {
        for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < (long long)n * rhs;
             p += (long long)gridDim.x * blockDim.x) {
            const double v = b[p];
            atomicAdd(&acc[p % rhs], v * v);
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < rhs; c += blockDim.x) atomicAdd(out + c, acc[c]);
}

// Interleaved FP32 off-diagonals: entry k of row i (k > rp[i]) goes to slot k - i - 1, so the
// off-diagonals of row i occupy [rp[i] - i, rp[i+1] - i - 1).
__global__ void k_build_offdiag(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                const double* __restrict__ val, int2* __restrict__ off) {
    const int lane = threadIdx.x & 31;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += (gridDim.x * blockDim.x) >> 5)
        for (int k = rp[i] + 1 + lane; k < rp[i + 1]; k += 32)
            off[k - i - 1] = make_int2(col[k], __float_as_int((float)val[k]));
}

// roff[i] = first off-diagonal slot of row i = rp[i] - i, padded past n with its end value.
__global__ void k_build_roff(int n, int pad, const int* __restrict__ rp, int* __restrict__ roff) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n + pad; i += gridDim.x * blockDim.x)
        roff[i] = (i <= n) ? rp[i] - i : rp[n] - n;
}

__global__ void k_pair_len(int n, const int* __restrict__ rp, int* __restrict__ len2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int len = rp[i + 1] - rp[i] - 1;
        len2[i] = len + (len & 1);
    }
}

__global__ void k_pad_roff(int n, int pad, int* __restrict__ roff) {
    const int total = roff[n];
    for (int i = n + 1 + blockIdx.x * blockDim.x + threadIdx.x; i <= n + pad; i += gridDim.x * blockDim.x)
        roff[i] = total;
}

__global__ void k_build_offdiag_pairs(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                      const double* __restrict__ val, const int* __restrict__ roff,
                                      int2* __restrict__ off) {
    const int lane = threadIdx.x & 31;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += (gridDim.x * blockDim.x) >> 5) {
        const int b = rp[i] + 1, len = rp[i + 1] - b, o = roff[i];
        for (int k = lane; k < len; k += 32) off[o + k] = make_int2(col[b + k], __float_as_int((float)val[b + k]));
        if (lane == 0 && (len & 1)) off[o + len] = make_int2(i, __float_as_int(0.f));
    }
}

// Group-jagged layout (32-row groups, jagged diagonals inside each group).  Group g holds rows
// 32g .. 32g+31; they are ranked by off-diagonal count, longest first (ties by row), and
// jmeta[32g + R] = (local row << 27) | count of the rank-R row.  Entry t of the rank-R row lives at
// jbase[g] + sum_{t' < t} c_g(t') + R, where c_g(t') = rows of the group with more than t' entries:
// the entries of one diagonal t are contiguous, so a warp whose lane R walks the rank-R row loads
// each diagonal with one coalesced request, and no slot is padding.  Rows past n count 0 entries.
// jbase[ngroups] = total entries, jbase[ngroups + 1] = 1 if some row has >= 2^27 entries.
constexpr int kJdsLenBits = 27;
constexpr int kJdsLenMask = (1 << kJdsLenBits) - 1;

__global__ void k_jds_sizes(int n, int ngroups, const int* __restrict__ rp, int* __restrict__ gsize,
                            int* __restrict__ overflow) {
    const int lane = threadIdx.x & 31;
    for (int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < ngroups; g += (gridDim.x * blockDim.x) >> 5) {
        const int i = 32 * g + lane;
        const int len = (i < n) ? rp[i + 1] - rp[i] - 1 : 0;
        if (len > kJdsLenMask) atomicOr(overflow, 1);
        const int s = __reduce_add_sync(0xffffffffu, len);
        if (lane == 0) gsize[g] = s;
    }
}

__global__ void k_jds_fill(int n, int ngroups, const int* __restrict__ rp, const int* __restrict__ col,
                           const double* __restrict__ val, const int* __restrict__ jbase, int* __restrict__ jmeta,
                           int2* __restrict__ jent) {
    const int lane = threadIdx.x & 31;
    for (int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < ngroups; g += (gridDim.x * blockDim.x) >> 5) {
        const int i = 32 * g + lane;
        const int first = (i < n) ? rp[i] + 1 : 0;
        const int len = (i < n) ? rp[i + 1] - first : 0;
        int rank = 0;
        for (int j = 0; j < 32; ++j) {
            const int lj = __shfl_sync(0xffffffffu, len, j);
            rank += (lj > len) || (lj == len && j < lane);
        }
        jmeta[32 * g + rank] = (lane << kJdsLenBits) | len;
        const int maxlen = __reduce_max_sync(0xffffffffu, len);
        int pos = jbase[g] + rank;
        for (int t = 0; t < maxlen; ++t) {
            const unsigned act = __ballot_sync(0xffffffffu, len > t);
            if (t < len) jent[pos] = make_int2(col[first + t], __float_as_int((float)val[first + t]));
            pos += __popc(act);
        }
    }
}

// Jacobi seed d0 = D^-1 r from the FP32 residual and FP32 reciprocal (FP32 pipe; the FP64 pipe
// is the residual kernels' bottleneck on this GPU), or the pending fill for an exact inner solve.
__device__ __forceinline__ void seed_out(int seed, float* d0, size_t p, float r32, float invd32) {
    if (seed == 1) d0[p] = r32 * invd32;
    else if (seed == 2) d0[p] = __uint_as_float(kPend32);
}

// r = b when x = 0 (the first correction of a solve): the matrix is not read.
__device__ __forceinline__ void residual_of_b(int n, const double* __restrict__ b, const float* __restrict__ invd,
                                              float* __restrict__ r32, float* __restrict__ d0, int seed,
                                              double* __restrict__ rn2, double* s_acc) {
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double r = b[i];
        const float rf = (float)r;
        r32[i] = rf;
        seed_out(seed, d0, i, rf, invd[i]);
        acc = fma(r, r, acc);
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) atomicAdd(s_acc, acc);
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(rn2, *s_acc);
}

// r = b - U x (rhs == 1), warp tiles of 32 rows staged in shared memory.
__global__ void __launch_bounds__(kResWarps * 32) k_residual_tile(int n, const int* __restrict__ rp,
                                                                  const int* __restrict__ col,
                                                                  const double* __restrict__ val,
                                                                  const float* __restrict__ invd,
                                                                  const double* __restrict__ b,
                                                                  const double* __restrict__ x,
                                                                  double* __restrict__ x_out, float* __restrict__ r32,
                                                                  float* __restrict__ d0, int seed,
                                                                  double* __restrict__ rn2, const Ctl* ctl) {
    __shared__ int s_col[kResWarps][kTileMax];
    __shared__ double s_val[kResWarps][kTileMax];
    __shared__ double s_acc;
    if (is_done(ctl)) return;
    if (threadIdx.x == 0) s_acc = 0.0;
    __syncthreads();
    if (*(volatile const int*)&ctl->x_zero) {
        residual_of_b(n, b, invd, r32, d0, seed, rn2, &s_acc);
        return;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int* sc = s_col[w];
    double* sv = s_val[w];
    double acc = 0.0;
    for (int t = blockIdx.x * kResWarps + w; t * 32 < n; t += gridDim.x * kResWarps) {
        const int r0 = t * 32, i = r0 + lane;
        const int s = rp[min(i, n)];
        int e = __shfl_down_sync(0xffffffffu, s, 1);
        if (lane == 31) e = rp[min(r0 + 32, n)];
        const int E0 = __shfl_sync(0xffffffffu, s, 0), E1 = __shfl_sync(0xffffffffu, e, 31);
        double sum = 0.0;
        if (E1 - E0 <= kTileMax) {
            for (int q = lane; q < E1 - E0; q += 32) {
                sc[q] = __ldg(col + E0 + q);
                sv[q] = __ldg(val + E0 + q);
            }
            __syncwarp();
            if (i < n) {
#pragma unroll 4
                for (int k = s - E0; k < e - E0; ++k) sum = fma(sv[k], __ldg(x + sc[k]), sum);
            }
            __syncwarp();
        } else if (i < n) {
            for (int k = s; k < e; ++k) sum = fma(__ldg(val + k), __ldg(x + __ldg(col + k)), sum);
        }
        if (i < n) {
            const double r = b[i] - sum;
            const float rf = (float)r;
            r32[i] = rf;
            seed_out(seed, d0, i, rf, invd[i]);
            acc = fma(r, r, acc);
            if (x_out) x_out[i] = x[i];
        }
    }
    acc = warp_sum(acc);
    if (lane == 0) atomicAdd(&s_acc, acc);
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(rn2, s_acc);
}

// r = b - U x (rhs == 1), LPR lanes per row (long rows).
template <int LPR>
__global__ void __launch_bounds__(256) k_residual_v(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                    const double* __restrict__ val, const float* __restrict__ invd,
                                                    const double* __restrict__ b, const double* __restrict__ x,
                                                    double* __restrict__ x_out, float* __restrict__ r32,
                                                    float* __restrict__ d0, int seed, double* __restrict__ rn2,
                                                    const Ctl* ctl) {
    if (is_done(ctl)) return;
    if (*(volatile const int*)&ctl->x_zero) x_out = nullptr;  // x is still the zero start vector
    __shared__ double s_acc;
    if (threadIdx.x == 0) s_acc = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int gl = lane % LPR;
    const unsigned gmask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << ((lane / LPR) * LPR));
    const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / LPR;
    const long long gstride = ((long long)gridDim.x * blockDim.x) / LPR;
    double acc = 0.0;
    for (long long i = gid; i < n; i += gstride) {
        const int s = rp[i], e = rp[i + 1];
        double sum = 0.0;
        for (int k = s + gl; k < e; k += LPR) sum = fma(val[k], x[col[k]], sum);
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(gmask, sum, o);
        if (gl == 0) {
            const double r = b[i] - sum;
            const float rf = (float)r;
            r32[i] = rf;
            seed_out(seed, d0, i, rf, invd[i]);
            acc = fma(r, r, acc);
            if (x_out) x_out[i] = x[i];
        }
    }
    acc = warp_sum(acc);
    if (lane == 0) atomicAdd(&s_acc, acc);
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(rn2, s_acc);
}

// rhs > 1: warp per row, lanes over RHS columns, entries sequential.
__global__ void __launch_bounds__(256) k_residual_m(int n, int rhs, const int* __restrict__ rp,
                                                    const int* __restrict__ col, const double* __restrict__ val,
                                                    const float* __restrict__ invd, const double* __restrict__ b,
                                                    const double* __restrict__ x, float* __restrict__ r32,
                                                    float* __restrict__ d0, int seed, double* __restrict__ rn2,
                                                    const Ctl* ctl) {
    if (is_done(ctl)) return;
    extern __shared__ double s_accm[];
    for (int c = threadIdx.x; c < rhs; c += blockDim.x) s_accm[c] = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long ws = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = w; i < n; i += ws) {
        const int s = rp[i], e = rp[i + 1];
        const float di = invd[i];
        for (int c = lane; c < rhs; c += 32) {
            double sum = 0.0;
            for (int k = s; k < e; ++k) sum = fma(val[k], x[(size_t)col[k] * rhs + c], sum);
            const size_t p = (size_t)i * rhs + c;
            const double r = b[p] - sum;
            const float rf = (float)r;
            r32[p] = rf;
            seed_out(seed, d0, p, rf, di);
            atomicAdd(&s_accm[c], r * r);
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < rhs; c += blockDim.x) atomicAdd(rn2 + c, s_accm[c]);
}

__device__ __forceinline__ double rel_of(int rhs, double* rn2, const double* bn2) {
    double rel = 0.0;
    for (int c = 0; c < rhs; ++c) {
        const double r = rn2[c], bb = bn2[c];
        const double q = (bb > 0.0) ? sqrt(r / bb) : (r > 0.0 ? INFINITY : 0.0);
        rel = fmax(rel, q);
        rn2[c] = 0.0;
    }
    return rel;
}

// Flat graphs: the convergence test of step `step`.
__global__ void k_check(int rhs, double* rn2, const double* bn2, Ctl* ctl, double tol, int step, int reset_ticket) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    ctl->x_zero = 0;
    if (ctl->done) return;
    const double rel = rel_of(rhs, rn2, bn2);
    ctl->rel_res = rel;
    ctl->steps = step;
    if (rel <= tol) ctl->done = 1;
    if (reset_ticket) ctl->ticket = 0u;
}

// Conditional graphs: the test at the top of every outer iteration.  Continues (and arms the
// inner loop) while rel > tol and fewer than max_refine corrections were applied.
// Relative accuracy asked of a correction: a tenth of what would just reach the tolerance.
constexpr double kInnerTarget = 0.1;

__global__ void k_check_outer(int rhs, double* rn2, const double* bn2, Ctl* ctl, double tol, int max_refine,
                              cudaGraphConditionalHandle h_outer, cudaGraphConditionalHandle h_inner) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double rel = rel_of(rhs, rn2, bn2);
    ctl->rel_res = rel;
    const int step = ctl->steps;
    const bool stop = rel <= tol || step >= max_refine;
    ctl->x_zero = 0;
    if (rel <= tol) ctl->done = 1;
    ctl->inner_count = 0;
    ctl->dmax_bits = 0u;
    ctl->dchg_bits = 0u;
    if (stop) {
        cudaGraphSetConditional(h_outer, 0);
        cudaGraphSetConditional(h_inner, 0);
    } else {
        ctl->steps = step + 1;
        // inexact correction: x + d has residual ~ rel * (relative error of d), so the next inner
        // solve only needs kInnerTarget * tol / rel (never tighter than its own floor, below)
        ctl->inner_eps = (float)fmin(1.0, kInnerTarget * tol / rel);
        cudaGraphSetConditional(h_inner, 1);
    }
}

// Conditional graphs: after each pair of sweeps.  Stops the inner loop once the largest
// change is at most max(eps, ctl->inner_eps) times the largest |d|, or after max_sweeps sweeps:
// eps is the FP32 floor of the sweeps, ctl->inner_eps what the outer residual still asks for.
__global__ void k_check_inner(Ctl* ctl, float eps_floor, int max_sweeps, cudaGraphConditionalHandle h_inner) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const float eps = fmaxf(eps_floor, ctl->inner_eps);
    const float dmax = __uint_as_float(ctl->dmax_bits), dchg = __uint_as_float(ctl->dchg_bits);
    const int cnt = ctl->inner_count + 2;
    ctl->inner_count = cnt;
    ctl->inner_total += 2;
    ctl->dmax_bits = 0u;
    ctl->dchg_bits = 0u;
    if (!(dchg > eps * dmax) || cnt >= max_sweeps) cudaGraphSetConditional(h_inner, 0);
}

__device__ __forceinline__ void reduce_stats(float dmax, float dchg, Ctl* ctl, unsigned* s_max) {
    for (int o = 16; o > 0; o >>= 1) {
        dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        dchg = fmaxf(dchg, __shfl_xor_sync(0xffffffffu, dchg, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&s_max[0], __float_as_uint(dmax));
        atomicMax(&s_max[1], __float_as_uint(dchg));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicMax(&ctl->dmax_bits, s_max[0]);
        atomicMax(&ctl->dchg_bits, s_max[1]);
    }
}

// One FP32 Jacobi sweep over warp tiles: dst = D^-1 (r - N src), or x += that when `last`.
// stats: accumulate max|d| and max|d - src| (non-negative floats order like their bits).
template <int TMAX, int MINB>
__global__ void __launch_bounds__(kJacWarps * 32, MINB) k_jacobi_tile(int n, const int* __restrict__ rp,
                                                                const int2* __restrict__ off,
                                                                const float* __restrict__ invd,
                                                                const float* __restrict__ r,
                                                                const float* __restrict__ src, float* __restrict__ dst,
                                                                double* __restrict__ x, int last, int stats, Ctl* ctl) {
    __shared__ __align__(16) int2 stage[kJacWarps][TMAX];
    __shared__ unsigned s_max[2];
    if (is_done(ctl)) return;
    if (threadIdx.x < 2) s_max[threadIdx.x] = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int2* sb = stage[w];
    float dmax = 0.f, dchg = 0.f;
    for (int t = blockIdx.x * kJacWarps + w; t * 32 < n; t += gridDim.x * kJacWarps) {
        const int r0 = t * 32, i = r0 + lane;
        const int ii = min(i, n);
        const int s = rp[ii] - ii;  // first off-diagonal slot of row i
        int e = __shfl_down_sync(0xffffffffu, s, 1);
        if (lane == 31) {
            const int j = min(r0 + 32, n);
            e = rp[j] - j;
        }
        const int E0 = __shfl_sync(0xffffffffu, s, 0), E1 = __shfl_sync(0xffffffffu, e, 31);
        float sum = 0.f;
        const int a0 = E0 & ~1;  // 16-byte aligned start (pairs of int2)
        if (E1 - a0 <= TMAX) {
            const int npair = (E1 - a0 + 1) >> 1;
            const int4* v4 = reinterpret_cast<const int4*>(off + a0);
            int4* s4 = reinterpret_cast<int4*>(sb);
            for (int q = lane; q < npair; q += 32) s4[q] = __ldg(v4 + q);
            __syncwarp();
            if (i < n) {
#pragma unroll 4
                for (int k = s - a0; k < e - a0; ++k) {
                    const int2 p = sb[k];
                    sum = fmaf(__int_as_float(p.y), __ldg(src + p.x), sum);
                }
            }
            __syncwarp();
        } else if (i < n) {
            for (int k = s; k < e; ++k) {
                const int2 p = __ldg(off + k);
                sum = fmaf(__int_as_float(p.y), __ldg(src + p.x), sum);
            }
        }
        if (i < n) {
            const float d = (r[i] - sum) * invd[i];
            if (stats) {
                dmax = fmaxf(dmax, fabsf(d));
                dchg = fmaxf(dchg, fabsf(d - src[i]));
            }
            if (last) x[i] += (double)d;
            else dst[i] = d;
        }
    }
    if (stats) reduce_stats(dmax, dchg, ctl, s_max);
}

// Lane-per-row sweep reading the interleaved off-diagonals straight from global memory (L1 keeps
// the lines a warp's 32 neighbouring rows share); bounded to 32 registers for full occupancy.
__global__ void __launch_bounds__(256, 8) k_jacobi_direct(int n, const int* __restrict__ roff,
                                                         const int2* __restrict__ off,
                                                         const float* __restrict__ invd,
                                                         const float* __restrict__ r, const float* __restrict__ src,
                                                         float* __restrict__ dst, double* __restrict__ x, int last,
                                                         int stats, Ctl* ctl) {
    __shared__ unsigned s_max[2];
    if (is_done(ctl)) return;
    if (threadIdx.x < 2) s_max[threadIdx.x] = 0u;
    __syncthreads();
    float dmax = 0.f, dchg = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int s = __ldg(roff + i), e = __ldg(roff + i + 1);
        float sum = 0.f;
#pragma unroll 4
        for (int k = s; k < e; ++k) {
            const int2 p = __ldg(off + k);
            sum = fmaf(__int_as_float(p.y), __ldg(src + p.x), sum);
        }
        const float d = (r[i] - sum) * invd[i];
        if (stats) {
            dmax = fmaxf(dmax, fabsf(d));
            dchg = fmaxf(dchg, fabsf(d - src[i]));
        }
        if (last) x[i] += (double)d;
        else dst[i] = d;
    }
    if (stats) reduce_stats(dmax, dchg, ctl, s_max);
}

// Lane-per-row sweep with explicit load batching: the next row's offsets are fetched while the
// current row is summed, and each batch of B entries issues all B entry loads, then all B
// gathers, then the B FMAs (in entry order, so the sum is the same as the sequential loop's).
template <int B, int MINB>
__global__ void __launch_bounds__(256, MINB) k_jacobi_batched(int n, const int* __restrict__ roff,
                                                             const int2* __restrict__ off,
                                                             const float* __restrict__ invd,
                                                             const float* __restrict__ r,
                                                             const float* __restrict__ src, float* __restrict__ dst,
                                                             double* __restrict__ x, int last, int stats, Ctl* ctl) {
    __shared__ unsigned s_max[2];
    if (is_done(ctl)) return;
    if (threadIdx.x < 2) s_max[threadIdx.x] = 0u;
    __syncthreads();
    float dmax = 0.f, dchg = 0.f;
    const int stride = gridDim.x * blockDim.x;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int s = 0, e = 0;
    if (i < n) { s = __ldg(roff + i); e = __ldg(roff + i + 1); }
    while (i < n) {
        const int inext = i + stride;
        int sn = 0, en = 0;
        if (inext < n) { sn = __ldg(roff + inext); en = __ldg(roff + inext + 1); }
        const float ri = r[i], di = invd[i];
        float sum = 0.f;
        for (int k0 = s; k0 < e; k0 += B) {
            int2 p[B];
            float g[B];
#pragma unroll
            for (int j = 0; j < B; ++j) p[j] = (k0 + j < e) ? __ldg(off + k0 + j) : make_int2(i, 0);
#pragma unroll
            for (int j = 0; j < B; ++j) g[j] = (k0 + j < e) ? __ldg(src + p[j].x) : 0.f;
#pragma unroll
            for (int j = 0; j < B; ++j) sum = fmaf(__int_as_float(p[j].y), g[j], sum);
        }
        const float d = (ri - sum) * di;
        if (stats) {
            dmax = fmaxf(dmax, fabsf(d));
            dchg = fmaxf(dchg, fabsf(d - src[i]));
        }
        if (last) x[i] += (double)d;
        else dst[i] = d;
        i = inext;
        s = sn;
        e = en;
    }
    if (stats) reduce_stats(dmax, dchg, ctl, s_max);
}

// The lane-per-row sweep over the paired layout: every row's slots start on a 16-byte boundary and
// come in pairs, so one 16-byte load brings two entries (half the load instructions, and the L1
// wavefronts, of 8-byte entry loads).  B entries (B/2 pair loads, then B gathers, then B FMAs in
// entry order) per batch; the next row's offsets are fetched while the current row is summed.  The
// pad entry of an odd row adds 0 * d_i.
template <int B, int MINB>
__global__ void __launch_bounds__(256, MINB) k_jacobi_pairs(int n, const int* __restrict__ roff,
                                                           const int4* __restrict__ off2,
                                                           const float* __restrict__ invd,
                                                           const float* __restrict__ r,
                                                           const float* __restrict__ src, float* __restrict__ dst,
                                                           double* __restrict__ x, int last, int stats, Ctl* ctl) {
    static_assert(B % 2 == 0, "entries come in pairs");
    __shared__ unsigned s_max[2];
    if (is_done(ctl)) return;
    if (threadIdx.x < 2) s_max[threadIdx.x] = 0u;
    __syncthreads();
    float dmax = 0.f, dchg = 0.f;
    const int stride = gridDim.x * blockDim.x;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int s = 0, e = 0;
    if (i < n) { s = __ldg(roff + i); e = __ldg(roff + i + 1); }
    while (i < n) {
        const int inext = i + stride;
        int sn = 0, en = 0;
        if (inext < n) { sn = __ldg(roff + inext); en = __ldg(roff + inext + 1); }
        const float ri = r[i], di = invd[i];
        float sum = 0.f;
        for (int k0 = s; k0 < e; k0 += B) {
            int4 p[B / 2];
            float g[B];
#pragma unroll
            for (int j = 0; j < B / 2; ++j) p[j] = (k0 + 2 * j < e) ? __ldg(off2 + (k0 >> 1) + j) : make_int4(i, 0, i, 0);
#pragma unroll
            for (int j = 0; j < B / 2; ++j) {
                g[2 * j] = (k0 + 2 * j < e) ? __ldg(src + p[j].x) : 0.f;
                g[2 * j + 1] = (k0 + 2 * j < e) ? __ldg(src + p[j].z) : 0.f;
            }
#pragma unroll
            for (int j = 0; j < B / 2; ++j) {
                sum = fmaf(__int_as_float(p[j].y), g[2 * j], sum);
                sum = fmaf(__int_as_float(p[j].w), g[2 * j + 1], sum);
            }
        }
        const float d = (ri - sum) * di;
        if (stats) {
            dmax = fmaxf(dmax, fabsf(d));
            dchg = fmaxf(dchg, fabsf(d - src[i]));
        }
        if (last) x[i] += (double)d;
        else dst[i] = d;
        i = inext;
        s = sn;
        e = en;
    }
    if (stats) reduce_stats(dmax, dchg, ctl, s_max);
}

// The sweep over the group-jagged layout: a warp per 32-row group, lane R on the rank-R row.  One
// diagonal of the group is one contiguous run of entries, so every entry load of the warp is a
// single coalesced request (the lane-per-row layouts touch one cache line per lane instead).  B
// diagonals per batch: B loads, B gathers, B FMAs in entry order; the group's next metadata is
// fetched while the current group is summed.  Measured on GB300 against the paired lane-per-row
// sweep: L1 throughput 51 % instead of 76 %, 5 % fewer DRAM bytes, the same time (the sweep is
// bound by load latency, not by L1 wavefronts); issuing the next batch's loads ahead of the current
// gathers (register pipelining, also unrolled by two) made it slower.
template <int B, int MINB>
__global__ void __launch_bounds__(256, MINB) k_jacobi_jds(int n, int ngroups, const int* __restrict__ jmeta,
                                                         const int* __restrict__ jbase,
                                                         const int2* __restrict__ jent,
                                                         const float* __restrict__ invd,
                                                         const float* __restrict__ r,
                                                         const float* __restrict__ src, float* __restrict__ dst,
                                                         double* __restrict__ x, int last, int stats, Ctl* ctl) {
    __shared__ unsigned s_max[2];
    if (is_done(ctl)) return;
    if (threadIdx.x < 2) s_max[threadIdx.x] = 0u;
    __syncthreads();
    float dmax = 0.f, dchg = 0.f;
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int meta = 0, base = 0;
    if (g < ngroups) { meta = __ldg(jmeta + 32 * g + lane); base = __ldg(jbase + g); }
    while (g < ngroups) {
        const int gn = g + nwarps;
        int meta_n = 0, base_n = 0;
        if (gn < ngroups) { meta_n = __ldg(jmeta + 32 * gn + lane); base_n = __ldg(jbase + gn); }
        const int len = meta & kJdsLenMask;
        const int row = 32 * g + (int)((unsigned)meta >> kJdsLenBits);
        const bool valid = row < n;
        const int maxlen = __reduce_max_sync(0xffffffffu, len);
        float ri = 0.f, di = 0.f;
        if (valid) { ri = r[row]; di = invd[row]; }
        float sum = 0.f;
        int pos = base + lane;
        for (int t0 = 0; t0 < maxlen; t0 += B) {
            int2 e[B];
            float gv[B];
#pragma unroll
            for (int j = 0; j < B; ++j) {
                const unsigned act = __ballot_sync(0xffffffffu, len > t0 + j);
                e[j] = (t0 + j < len) ? __ldg(jent + pos) : make_int2(0, 0);
                pos += __popc(act);
            }
#pragma unroll
            for (int j = 0; j < B; ++j) gv[j] = (t0 + j < len) ? __ldg(src + e[j].x) : 0.f;
#pragma unroll
            for (int j = 0; j < B; ++j) sum = fmaf(__int_as_float(e[j].y), gv[j], sum);
        }
        if (valid) {
            const float d = (ri - sum) * di;
            if (stats) {
                dmax = fmaxf(dmax, fabsf(d));
                dchg = fmaxf(dchg, fabsf(d - src[row]));
            }
            if (last) x[row] += (double)d;
            else dst[row] = d;
        }
        g = gn;
        meta = meta_n;
        base = base_n;
    }
    if (stats) reduce_stats(dmax, dchg, ctl, s_max);
}

// Same, two rows per thread per iteration (i and i + half the grid): two independent load chains
// in flight per thread.
__global__ void __launch_bounds__(256, 8) k_jacobi_direct2(int n, const int* __restrict__ roff,
                                                          const int2* __restrict__ off,
                                                          const float* __restrict__ invd,
                                                          const float* __restrict__ r, const float* __restrict__ src,
                                                          float* __restrict__ dst, double* __restrict__ x, int last,
                                                          int stats, Ctl* ctl) {
    __shared__ unsigned s_max[2];
    if (is_done(ctl)) return;
    if (threadIdx.x < 2) s_max[threadIdx.x] = 0u;
    __syncthreads();
    float dmax = 0.f, dchg = 0.f;
    const int stride = gridDim.x * blockDim.x;
    for (int i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += 2 * stride) {
        const int i1 = i0 + stride;
        const bool has1 = i1 < n;
        const int s0 = __ldg(roff + i0), e0 = __ldg(roff + i0 + 1);
        const int s1 = has1 ? __ldg(roff + i1) : 0, e1 = has1 ? __ldg(roff + i1 + 1) : 0;
        float sum0 = 0.f, sum1 = 0.f;
        const int l0 = e0 - s0, l1 = e1 - s1;
        const int lmax = l0 > l1 ? l0 : l1;
#pragma unroll 2
        for (int q = 0; q < lmax; ++q) {
            if (q < l0) {
                const int2 p = __ldg(off + s0 + q);
                sum0 = fmaf(__int_as_float(p.y), __ldg(src + p.x), sum0);
            }
            if (q < l1) {
                const int2 p = __ldg(off + s1 + q);
                sum1 = fmaf(__int_as_float(p.y), __ldg(src + p.x), sum1);
            }
        }
        const float d0 = (r[i0] - sum0) * invd[i0];
        if (stats) {
            dmax = fmaxf(dmax, fabsf(d0));
            dchg = fmaxf(dchg, fabsf(d0 - src[i0]));
        }
        if (last) x[i0] += (double)d0;
        else dst[i0] = d0;
        if (has1) {
            const float d1 = (r[i1] - sum1) * invd[i1];
            if (stats) {
                dmax = fmaxf(dmax, fabsf(d1));
                dchg = fmaxf(dchg, fabsf(d1 - src[i1]));
            }
            if (last) x[i1] += (double)d1;
            else dst[i1] = d1;
        }
    }
    if (stats) reduce_stats(dmax, dchg, ctl, s_max);
}

// ---------------------------------------------------------------------------------------
// SELL-32-256 copy of the off-diagonals for the sweeps: rows are sorted by off-diagonal count
// (descending, stable) inside windows of 256 rows and grouped into slices of 32; a slice stores
// entry k of its 32 rows contiguously (column-major inside the slice) and is padded to its
// longest row with (column = the row itself, value 0).  A warp sweeps a slice with every load
// coalesced (256 bytes per instruction) and no divergence.
constexpr int kSellWin = 256;

// One block of 256 threads per window: bitonic sort of (count, row) by count descending, row
// ascending (stable order), then slice lengths.
__global__ void __launch_bounds__(kSellWin) k_sell_sort(int n, const int* __restrict__ rp, int* __restrict__ perm,
                                                        int* __restrict__ slen) {
    __shared__ int key[kSellWin], idx[kSellWin];
    const int w = blockIdx.x, t = threadIdx.x;
    const int row = w * kSellWin + t;
    key[t] = row < n ? rp[row + 1] - rp[row] - 1 : -1;  // padding rows sort last
    idx[t] = row;
    __syncthreads();
    for (int k = 2; k <= kSellWin; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            const int p = t ^ j;
            if (p > t) {
                const bool up = (t & k) == 0;  // this pair sorts "descending by key, ascending by row"
                const int ka = key[t], kb = key[p], ia = idx[t], ib = idx[p];
                const bool a_first = ka > kb || (ka == kb && ia < ib);
                if (a_first != up) {
                    key[t] = kb; key[p] = ka;
                    idx[t] = ib; idx[p] = ia;
                }
            }
            __syncthreads();
        }
    }
    perm[row] = idx[t] < n ? idx[t] : -1;
    if ((t & 31) == 0) slen[row >> 5] = key[t] > 0 ? key[t] : 0;  // first row of a slice is its longest
}

__global__ void k_sell_sizes(int nslices, const int* __restrict__ slen, int* __restrict__ sz) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nslices; s += gridDim.x * blockDim.x) sz[s] = 32 * slen[s];
}

__global__ void k_sell_fill(int nslices, const int* __restrict__ rp, const int* __restrict__ col,
                            const double* __restrict__ val, const int* __restrict__ perm, const int* __restrict__ slen,
                            const int* __restrict__ sptr, int2* __restrict__ sell) {
    const int lane = threadIdx.x & 31;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += (gridDim.x * blockDim.x) >> 5) {
        const int row = perm[32 * s + lane];
        const int len = slen[s];
        const int base = sptr[s];
        const int b = row >= 0 ? rp[row] + 1 : 0, e = row >= 0 ? rp[row + 1] : 0;
        for (int k = 0; k < len; ++k) {
            int2 v = make_int2(row >= 0 ? row : 0, 0);  // padding: 0 * x[row]
            if (b + k < e) v = make_int2(col[b + k], __float_as_int((float)val[b + k]));
            sell[base + 32 * k + lane] = v;
        }
    }
}

__global__ void __launch_bounds__(256, 8) k_jacobi_sell(int nslices, const int* __restrict__ perm,
                                                       const int* __restrict__ slen, const int* __restrict__ sptr,
                                                       const int2* __restrict__ sell,
                                                       const float* __restrict__ invd, const float* __restrict__ r,
                                                       const float* __restrict__ src, float* __restrict__ dst,
                                                       double* __restrict__ x, int last, int stats, Ctl* ctl) {
    __shared__ unsigned s_max[2];
    if (is_done(ctl)) return;
    if (threadIdx.x < 2) s_max[threadIdx.x] = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    float dmax = 0.f, dchg = 0.f;
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nslices; s += (gridDim.x * blockDim.x) >> 5) {
        const int row = __ldg(perm + 32 * s + lane);
        const int len = __ldg(slen + s);
        const int2* p = sell + __ldg(sptr + s) + lane;
        float sum = 0.f;
#pragma unroll 4
        for (int k = 0; k < len; ++k) {
            const int2 v = __ldg(p + 32 * k);
            sum = fmaf(__int_as_float(v.y), __ldg(src + v.x), sum);
        }
        if (row >= 0) {
            const float d = (r[row] - sum) * invd[row];
            if (stats) {
                dmax = fmaxf(dmax, fabsf(d));
                dchg = fmaxf(dchg, fabsf(d - src[row]));
            }
            if (last) x[row] += (double)d;
            else dst[row] = d;
        }
    }
    if (stats) reduce_stats(dmax, dchg, ctl, s_max);
}

// SELL build, first half: window sorts, slice lengths and slice offsets; returns the entry count.
int sell_prepare(int n, const int* rp, int* perm, int* slen, int* sptr, int* part, int sm_count, cudaStream_t st,
                 int64_t* launches, int* total) {
    const int nwin = (n + kSellWin - 1) / kSellWin;
    const int nslices = nwin * (kSellWin / 32);
    k_sell_sort<<<nwin, kSellWin, 0, st>>>(n, rp, perm, slen);
    k_sell_sizes<<<sm_count * 4, 256, 0, st>>>(nslices, slen, sptr);
    *launches += 2;
    int rc = scan_exclusive(sptr, sptr, nslices, part, st, launches);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(total, sptr + nslices, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return 0;
}

// SELL build, second half: the slices' column-major entries (`sell` holds `total` entries).
int sell_fill(int n, const int* rp, const int* col, const double* val, const int* perm, const int* slen,
              const int* sptr, int2* sell, int sm_count, cudaStream_t st, int64_t* launches) {
    const int nslices = ((n + kSellWin - 1) / kSellWin) * (kSellWin / 32);
    k_sell_fill<<<sm_count * 8, 256, 0, st>>>(nslices, rp, col, val, perm, slen, sptr, sell);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}
int sell_slices(int n) { return ((n + kSellWin - 1) / kSellWin) * (kSellWin / 32); }

// ---------------------------------------------------------------------------------------
// Bulk-copy pipelined sweep.  Each warp walks its tiles (32 rows each) with a kStages-deep
// pipeline: lane 0 issues cp.async.bulk copies of the next tiles' row offsets and interleaved
// off-diagonals into the warp's shared-memory stages (completion counted in bytes on an
// mbarrier), while the lanes compute on the current tile.  No registers hold in-flight data,
// so every SM keeps tens of KB of matrix traffic in flight.  Copies start on 16-byte
// boundaries (even int2 index, 32-row aligned offset rows) and move multiples of 16 bytes;
// `off` and `roff` carry padding so the rounded-up ranges stay inside their allocations.
// Tiles larger than a stage are read straight from global memory.  Every mbarrier wait is
// bounded by the spin budget.
constexpr int kStages = 4;
constexpr int kTmaWarps = 4;
constexpr int kStageEntries = 384;  // int2 entries per stage (3 KiB)

struct __align__(128) TmaStage {
    int2 off[kStageEntries];
    int roff[36];  // 36 ints = 144 bytes: the tile's 33 row offsets, rounded up to 16 bytes
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for phase `parity` of *bar; false on timeout or abort (error recorded)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, Ctl* ctl, int64_t budget) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (aborted(ctl)) return false;
        if ((int64_t)(gtimer() - t0) > budget) { record_error(ctl, SPTRSV_ERR_TIMEOUT); return false; }
    }
}

__global__ void __launch_bounds__(kTmaWarps * 32) k_jacobi_tma(int n, const int* __restrict__ roff,
                                                              const int2* __restrict__ off,
                                                              const float* __restrict__ invd,
                                                              const float* __restrict__ r,
                                                              const float* __restrict__ src, float* __restrict__ dst,
                                                              double* __restrict__ x, int last, int stats, Ctl* ctl,
                                                              int64_t budget) {
    extern __shared__ __align__(128) unsigned char tma_smem[];
    TmaStage(*stages)[kStages] = reinterpret_cast<TmaStage(*)[kStages]>(tma_smem);
    __shared__ __align__(8) uint64_t bars[kTmaWarps][kStages];
    __shared__ unsigned s_max[2];
    if (is_done(ctl)) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x < 2) s_max[threadIdx.x] = 0u;
    if (lane == 0)
        for (int q = 0; q < kStages; ++q) mbar_init(&bars[w][q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();
    const int ntiles = (n + 31) >> 5;
    const int nw = gridDim.x * kTmaWarps;
    const int first = blockIdx.x * kTmaWarps + w;
    TmaStage* st = stages[w];
    uint64_t* bar = bars[w];
    // issue tile j (the j-th tile of this warp) into stage j % kStages; returns its mode:
    // 1 staged, 2 direct (too large for a stage), 0 none (past the end)
    // lane 0 keeps the row-offset bounds of the next tile to issue in registers, loaded one
    // iteration before they are needed, so the issue never waits on a global load
    int nx_e0 = 0, nx_e1 = 0;
    auto fetch = [&](int j) {
        const int t = first + j * nw;
        if (t < ntiles) { nx_e0 = __ldg(roff + 32 * t); nx_e1 = __ldg(roff + 32 * t + 32); }
    };
    auto issue = [&](int j) -> int {
        const int t = first + j * nw;
        if (t >= ntiles) return 0;
        const int e0 = nx_e0, e1 = nx_e1;
        fetch(j + 1);
        const int a0 = e0 & ~1, a1 = (e1 + 1) & ~1;
        TmaStage& S = st[j % kStages];
        uint64_t* b = &bar[j % kStages];
        if (a1 - a0 > kStageEntries) return 2;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const unsigned bytes = (unsigned)(a1 - a0) * 8u;
        mbar_expect_tx(b, bytes + 144u);
        bulk_g2s(S.roff, roff + 32 * t, 144u, b);
        if (bytes) bulk_g2s(S.off, off + a0, bytes, b);
        return 1;
    };
    // per-stage mode (2 bits each: 0 none, 1 staged, 2 direct) and mbarrier phase bits
    unsigned modes = 0u, phases = 0u, pending = 0u;
    auto set_mode = [&](int q, int md) {
        modes = (modes & ~(3u << (2 * q))) | ((unsigned)md << (2 * q));
        if (md == 1) pending |= 1u << q;
    };
    // prologue: fill the pipeline (lane 0 issues, the mode is broadcast)
    if (lane == 0) fetch(0);
    for (int j = 0; j < kStages - 1; ++j) {
        int md = 0;
        if (lane == 0) md = issue(j);
        set_mode(j % kStages, __shfl_sync(0xffffffffu, md, 0));
    }
    float dmax = 0.f, dchg = 0.f;
    bool ok = true;
    for (int j = 0;; ++j) {
        const int t = first + j * nw;
        if (t >= ntiles) break;
        {   // keep kStages - 1 tiles in flight ahead of the one being computed
            int md = 0;
            if (lane == 0) md = issue(j + kStages - 1);
            set_mode((j + kStages - 1) % kStages, __shfl_sync(0xffffffffu, md, 0));
        }
        const int q = j % kStages;
        const int r0 = t * 32, i = r0 + lane;
        float sum = 0.f;
        const int mq = (modes >> (2 * q)) & 3u;
        if (mq == 1) {
            ok = mbar_wait(&bar[q], (phases >> q) & 1u, ctl, budget);
            phases ^= 1u << q;
            pending &= ~(1u << q);
            if (!__all_sync(0xffffffffu, ok)) break;
            const TmaStage& S = st[q];
            const int a0 = S.roff[0] & ~1;
            if (i < n) {
                const int s = S.roff[lane] - a0, e = S.roff[lane + 1] - a0;
#pragma unroll 4
                for (int k = s; k < e; ++k) {
                    const int2 p = S.off[k];
                    sum = fmaf(__int_as_float(p.y), __ldg(src + p.x), sum);
                }
            }
        } else if (i < n) {
            const int s = roff[i], e = roff[i + 1];
            for (int k = s; k < e; ++k) {
                const int2 p = __ldg(off + k);
                sum = fmaf(__int_as_float(p.y), __ldg(src + p.x), sum);
            }
        }
        __syncwarp();  // every lane is done with stage q before it is refilled
        if (i < n) {
            const float d = (r[i] - sum) * invd[i];
            if (stats) {
                dmax = fmaxf(dmax, fabsf(d));
                dchg = fmaxf(dchg, fabsf(d - src[i]));
            }
            if (last) x[i] += (double)d;
            else dst[i] = d;
        }
    }
    // drain: copies issued but not consumed (only after an aborted wait) complete before the
    // block exits, each wait again bounded by the budget
    for (int q = 0; q < kStages; ++q)
        if (pending & (1u << q)) (void)mbar_wait(&bar[q], (phases >> q) & 1u, ctl, budget);
    if (stats) reduce_stats(dmax, dchg, ctl, s_max);
}

// Same sweep, LPR lanes per row over the CSR FP32 values (long rows).
template <int LPR>
__global__ void __launch_bounds__(256) k_jacobi_v(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                  const float* __restrict__ val, const float* __restrict__ invd,
                                                  const float* __restrict__ r, const float* __restrict__ src,
                                                  float* __restrict__ dst, double* __restrict__ x, int last,
                                                  int stats, Ctl* ctl) {
    __shared__ unsigned s_max[2];
    if (is_done(ctl)) return;
    if (threadIdx.x < 2) s_max[threadIdx.x] = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int gl = lane % LPR;
    const unsigned gmask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << ((lane / LPR) * LPR));
    const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / LPR;
    const long long gstride = ((long long)gridDim.x * blockDim.x) / LPR;
    float dmax = 0.f, dchg = 0.f;
    for (long long i = gid; i < n; i += gstride) {
        const int s = rp[i], e = rp[i + 1];
        float sum = 0.f;
        for (int k = s + 1 + gl; k < e; k += LPR) sum = fmaf(val[k], src[col[k]], sum);
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(gmask, sum, o);
        if (gl == 0) {
            const float d = (r[i] - sum) * invd[i];
            if (stats) {
                dmax = fmaxf(dmax, fabsf(d));
                dchg = fmaxf(dchg, fabsf(d - src[i]));
            }
            if (last) x[i] += (double)d;
            else dst[i] = d;
        }
    }
    if (stats) reduce_stats(dmax, dchg, ctl, s_max);
}

__global__ void __launch_bounds__(256) k_jacobi_m(int n, int rhs, const int* __restrict__ rp,
                                                  const int* __restrict__ col, const float* __restrict__ val,
                                                  const float* __restrict__ invd, const float* __restrict__ r,
                                                  const float* __restrict__ src, float* __restrict__ dst,
                                                  double* __restrict__ x, int last, int stats, Ctl* ctl) {
    __shared__ unsigned s_max[2];
    if (is_done(ctl)) return;
    if (threadIdx.x < 2) s_max[threadIdx.x] = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long ws = ((long long)gridDim.x * blockDim.x) >> 5;
    float dmax = 0.f, dchg = 0.f;
    for (long long i = w; i < n; i += ws) {
        const int s = rp[i], e = rp[i + 1];
        const float di = invd[i];
        for (int c = lane; c < rhs; c += 32) {
            float sum = 0.f;
            for (int k = s + 1; k < e; ++k) sum = fmaf(val[k], src[(size_t)col[k] * rhs + c], sum);
            const size_t p = (size_t)i * rhs + c;
            const float d = (r[p] - sum) * di;
            if (stats) {
                dmax = fmaxf(dmax, fabsf(d));
                dchg = fmaxf(dchg, fabsf(d - src[p]));
            }
            if (last) x[p] += (double)d;
            else dst[p] = d;
        }
    }
    if (stats) reduce_stats(dmax, dchg, ctl, s_max);
}

__global__ void k_axpy_f32(size_t count, const float* __restrict__ d, double* __restrict__ x, const Ctl* ctl) {
    if (is_done(ctl)) return;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < count; p += (size_t)gridDim.x * blockDim.x)
        x[p] += (double)d[p];
}

// Exact inner solves skip themselves once the refinement has converged.
__global__ void k_gate_ticket(Ctl* ctl) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && ctl->done) ctl->ticket = 0xF0000000u;  // no row left to claim
}

// ---------------------------------------------------------------------------------------
static int lpr_for(int n, int nnz) {
    const double mean = n > 0 ? (double)nnz / n : 1.0;
    if (mean <= 6.0) return 4;
    if (mean <= 12.0) return 8;
    if (mean <= 24.0) return 16;
    return 32;
}
// warp tiles pay off while a 32-row tile usually fits the stage
static bool short_rows(const RefineArgs& a) { return a.rhs == 1 && (double)a.nnz / a.n <= 14.0; }
static bool use_tiles(const RefineArgs& a) { return short_rows(a) && a.off; }

static int stream_grid(int sm_count) { return sm_count * 8; }

// One resident wave: blocks per SM from the occupancy calculator, times the SM count, so that a
// grid-stride kernel never leaves a partial second wave.
static int resident_grid(const void* fn, int block, int sm_count) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
    return per_sm * sm_count;
}

static size_t tma_smem_bytes() { return sizeof(TmaStage) * kStages * kTmaWarps; }

int launch_pair_offsets(int n, const int* rp, int* len2, int* roff, int roff_pad, int* part, int sm_count,
                        cudaStream_t st, int64_t* launches) {
    k_pair_len<<<sm_count * 4, 256, 0, st>>>(n, rp, len2);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    int rc = scan_exclusive(len2, roff, n, part, st, launches);
    if (rc) return rc;
    k_pad_roff<<<1, 64, 0, st>>>(n, roff_pad, roff);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_build_offdiag_pairs(int n, const int* rp, const int* col, const double* val, const int* roff, int2* off,
                               int sm_count, cudaStream_t st, int64_t* launches) {
    k_build_offdiag_pairs<<<sm_count * 8, 256, 0, st>>>(n, rp, col, val, roff, off);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_jds_sizes(int n, const int* rp, int* gsize, int* overflow, int sm_count, cudaStream_t st,
                     int64_t* launches) {
    const int ngroups = (n + 31) / 32;
    k_jds_sizes<<<sm_count * 8, 256, 0, st>>>(n, ngroups, rp, gsize, overflow);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_jds_fill(int n, const int* rp, const int* col, const double* val, const int* jbase, int* jmeta, int2* jent,
                    int sm_count, cudaStream_t st, int64_t* launches) {
    const int ngroups = (n + 31) / 32;
    k_jds_fill<<<sm_count * 8, 256, 0, st>>>(n, ngroups, rp, col, val, jbase, jmeta, jent);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_build_offdiag(int n, const int* rp, const int* col, const double* val, int2* off, int* roff,
                         int roff_pad, int sm_count, cudaStream_t st, int64_t* launches) {
    k_build_offdiag<<<sm_count * 8, 256, 0, st>>>(n, rp, col, val, off);
    k_build_roff<<<sm_count * 4, 256, 0, st>>>(n, roff_pad, rp, roff);
    *launches += 2;
    CUDA_TRY(cudaGetLastError());
    // opt in to the sweep kernel's dynamic shared memory here, outside any stream capture
    CUDA_TRY(cudaFuncSetAttribute(k_jacobi_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tma_smem_bytes()));
    return 0;
}

__global__ void k_mark_x_zero(Ctl* ctl) {
    if (threadIdx.x == 0 && blockIdx.x == 0) ctl->x_zero = 1;
}

// x = 0, ||b_c||^2; the device-looped graphs also mark x as zero so that their first residual
// is taken from b without reading the matrix.
int launch_refine_init(const RefineArgs& a, bool mark_zero) {
    CUDA_TRY(cudaMemsetAsync(a.x, 0, sizeof(double) * (size_t)a.n * a.rhs, a.st));
    if (mark_zero) {
        k_mark_x_zero<<<1, 32, 0, a.st>>>(a.ctl);
        ++*a.launches;
    }
    CUDA_TRY(cudaMemsetAsync(a.rn2, 0, sizeof(double) * a.rhs, a.st));
    CUDA_TRY(cudaMemsetAsync(a.bn2, 0, sizeof(double) * a.rhs, a.st));
    k_colnorm2<<<stream_grid(a.sm_count), 256, sizeof(double) * a.rhs, a.st>>>(a.n, a.rhs, a.b, a.bn2);
    ++*a.launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

// seed: 0 none, 1 Jacobi d0 = D^{-1} r into d32[0], 2 pending fill of d32[0].
int launch_residual(const RefineArgs& a, bool jacobi_seed, int final_check) {
    const int seed = final_check ? 0 : (jacobi_seed ? 1 : 2);
    const int grid = stream_grid(a.sm_count);
    if (short_rows(a)) {
        static int grid_rt = 0;
        if (!grid_rt) grid_rt = resident_grid((const void*)k_residual_tile, kResWarps * 32, a.sm_count);
        k_residual_tile<<<grid_rt, kResWarps * 32, 0, a.st>>>(a.n, a.rp, a.col, a.val, a.invd32, a.b, a.x,
                                                                      a.x_out, a.r32, a.d32[0], seed, a.rn2, a.ctl);
    } else if (a.rhs == 1) {
        switch (lpr_for(a.n, a.nnz)) {
            case 4: k_residual_v<4><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val, a.invd32, a.b, a.x, a.x_out, a.r32, a.d32[0], seed, a.rn2, a.ctl); break;
            case 8: k_residual_v<8><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val, a.invd32, a.b, a.x, a.x_out, a.r32, a.d32[0], seed, a.rn2, a.ctl); break;
            case 16: k_residual_v<16><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val, a.invd32, a.b, a.x, a.x_out, a.r32, a.d32[0], seed, a.rn2, a.ctl); break;
            default: k_residual_v<32><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val, a.invd32, a.b, a.x, a.x_out, a.r32, a.d32[0], seed, a.rn2, a.ctl); break;
        }
    } else {
        k_residual_m<<<grid, 256, sizeof(double) * a.rhs, a.st>>>(a.n, a.rhs, a.rp, a.col, a.val, a.invd32, a.b, a.x,
                                                                  a.r32, a.d32[0], seed, a.rn2, a.ctl);
    }
    ++*a.launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_check(const RefineArgs& a, int step, bool reset_ticket) {
    k_check<<<1, 32, 0, a.st>>>(a.rhs, a.rn2, a.bn2, a.ctl, a.tol, step, reset_ticket ? 1 : 0);
    ++*a.launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_check_outer(const RefineArgs& a, int max_refine, cudaGraphConditionalHandle ho,
                       cudaGraphConditionalHandle hi) {
    k_check_outer<<<1, 32, 0, a.st>>>(a.rhs, a.rn2, a.bn2, a.ctl, a.tol, max_refine, ho, hi);
    ++*a.launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_check_inner(const RefineArgs& a, float eps, int max_sweeps, cudaGraphConditionalHandle hi) {
    k_check_inner<<<1, 32, 0, a.st>>>(a.ctl, eps, max_sweeps, hi);
    ++*a.launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_jacobi_sweep(const RefineArgs& a, int src, bool last, bool stats) {
    const int grid = stream_grid(a.sm_count);
    const float* s = a.d32[src];
    float* d = a.d32[src ^ 1];
    const int st_flag = stats ? 1 : 0;
    if (use_tiles(a) && a.jmeta) {
        static int grid_j6 = 0;
        if (!grid_j6) grid_j6 = resident_grid((const void*)k_jacobi_jds<6, 6>, 256, a.sm_count);
        k_jacobi_jds<6, 6><<<grid_j6, 256, 0, a.st>>>(a.n, (a.n + 31) / 32, a.jmeta, a.jbase, a.off, a.invd32, a.r32, s,
                                                     d, a.x, last, st_flag, a.ctl);
    } else if (use_tiles(a) && a.roff && a.pairs) {
        static int grid_p8 = 0;
        if (!grid_p8) grid_p8 = resident_grid((const void*)k_jacobi_pairs<8, 6>, 256, a.sm_count);
        k_jacobi_pairs<8, 6><<<grid_p8, 256, 0, a.st>>>(a.n, a.roff, reinterpret_cast<const int4*>(a.off), a.invd32,
                                                       a.r32, s, d, a.x, last, st_flag, a.ctl);
    } else if (use_tiles(a) && a.roff && (a.sweep_kernel == 7)) {
        static int grid_b4 = 0;
        if (!grid_b4) grid_b4 = resident_grid((const void*)k_jacobi_batched<4, 8>, 256, a.sm_count);
        k_jacobi_batched<4, 8><<<grid_b4, 256, 0, a.st>>>(a.n, a.roff, a.off, a.invd32, a.r32, s, d, a.x, last,
                                                         st_flag, a.ctl);
    } else if (use_tiles(a) && a.roff && (a.sweep_kernel == 8 || a.sweep_kernel == 0)) {
        static int grid_b8 = 0;
        if (!grid_b8) grid_b8 = resident_grid((const void*)k_jacobi_batched<8, 6>, 256, a.sm_count);
        k_jacobi_batched<8, 6><<<grid_b8, 256, 0, a.st>>>(a.n, a.roff, a.off, a.invd32, a.r32, s, d, a.x, last,
                                                         st_flag, a.ctl);
    } else if (a.rhs == 1 && a.sell && a.sweep_kernel == 6) {
        static int grid_s = 0;
        if (!grid_s) grid_s = resident_grid((const void*)k_jacobi_sell, 256, a.sm_count);
        k_jacobi_sell<<<grid_s, 256, 0, a.st>>>(a.nslices, a.sell_perm, a.sell_len, a.sell_ptr, a.sell, a.invd32, a.r32,
                                                s, d, a.x, last, st_flag, a.ctl);
    } else if (use_tiles(a) && a.roff && a.sweep_kernel == 4) {
        static int grid_d2 = 0;
        if (!grid_d2) grid_d2 = resident_grid((const void*)k_jacobi_direct2, 256, a.sm_count);
        k_jacobi_direct2<<<grid_d2, 256, 0, a.st>>>(a.n, a.roff, a.off, a.invd32, a.r32, s, d, a.x, last, st_flag,
                                                   a.ctl);
    } else if (use_tiles(a) && a.roff && a.sweep_kernel == 2) {
        static int grid_d = 0;
        if (!grid_d) grid_d = resident_grid((const void*)k_jacobi_direct, 256, a.sm_count);
        k_jacobi_direct<<<grid_d, 256, 0, a.st>>>(a.n, a.roff, a.off, a.invd32, a.r32, s, d, a.x, last, st_flag, a.ctl);
    } else if (use_tiles(a) && a.sweep_kernel == 3) {
        static int grid_t8 = 0;
        if (!grid_t8) grid_t8 = resident_grid((const void*)k_jacobi_tile<384, 8>, kJacWarps * 32, a.sm_count);
        k_jacobi_tile<384, 8><<<grid_t8, kJacWarps * 32, 0, a.st>>>(a.n, a.rp, a.off, a.invd32, a.r32, s, d, a.x,
                                                                   last, st_flag, a.ctl);
    } else if (use_tiles(a) && a.roff && a.sweep_kernel == 5) {
        static int grid_tma = 0;
        if (!grid_tma) {
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_jacobi_tma, kTmaWarps * 32,
                                                              tma_smem_bytes()) != cudaSuccess || per_sm < 1)
                per_sm = 1;
            grid_tma = per_sm * a.sm_count;
        }
        k_jacobi_tma<<<grid_tma, kTmaWarps * 32, tma_smem_bytes(), a.st>>>(a.n, a.roff, a.off, a.invd32, a.r32, s, d,
                                                                         a.x, last, st_flag, a.ctl, a.budget);
    } else if (use_tiles(a)) {
        static int grid_jt = 0;
        if (!grid_jt) grid_jt = resident_grid((const void*)k_jacobi_tile<kTileMax, 1>, kJacWarps * 32, a.sm_count);
        k_jacobi_tile<kTileMax, 1><<<grid_jt, kJacWarps * 32, 0, a.st>>>(a.n, a.rp, a.off, a.invd32, a.r32, s, d, a.x, last,
                                                                  st_flag, a.ctl);
    } else if (a.rhs == 1) {
        switch (lpr_for(a.n, a.nnz)) {
            case 4: k_jacobi_v<4><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val32, a.invd32, a.r32, s, d, a.x, last, st_flag, a.ctl); break;
            case 8: k_jacobi_v<8><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val32, a.invd32, a.r32, s, d, a.x, last, st_flag, a.ctl); break;
            case 16: k_jacobi_v<16><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val32, a.invd32, a.r32, s, d, a.x, last, st_flag, a.ctl); break;
            default: k_jacobi_v<32><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val32, a.invd32, a.r32, s, d, a.x, last, st_flag, a.ctl); break;
        }
    } else {
        k_jacobi_m<<<grid, 256, 0, a.st>>>(a.n, a.rhs, a.rp, a.col, a.val32, a.invd32, a.r32, s, d, a.x, last,
                                           st_flag, a.ctl);
    }
    ++*a.launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_axpy_pending(const RefineArgs& a, int src) {
    const size_t count = (size_t)a.n * a.rhs;
    const int blocks = (int)std::min<size_t>((count + 255) / 256, (size_t)a.sm_count * 8);
    k_axpy_f32<<<blocks, 256, 0, a.st>>>(count, a.d32[src], a.x, a.ctl);
    ++*a.launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

int launch_exact_inner(const RefineArgs& a, int schedule, int rows_per_warp, int dst, int max_level,
                       const int* lptr, const int* lrows, int warps) {
    SolveArgs s{};
    s.n = a.n;
    s.rp = a.rp;
    s.col = a.col;
    s.val = a.val32;
    s.invd = a.invd32;
    s.b = a.r32;
    s.x = a.d32[dst];
    s.rhs = a.rhs;
    s.ctl = a.ctl;
    s.budget = a.budget;
    s.sm_count = a.sm_count;
    s.warps = warps;
    s.nnz = a.nnz;
    s.st = a.st;
    s.launches = a.launches;
    if (schedule == SPTRSV_SCHED_LEVELSET) return launch_levelset(true, s, max_level, lptr, lrows);
    k_gate_ticket<<<1, 32, 0, a.st>>>(a.ctl);
    ++*a.launches;
    if (schedule == SPTRSV_SCHED_SYNCFREE_THREAD && a.rhs == 1) return launch_pull_thread(true, s);
    if (schedule == SPTRSV_SCHED_SYNCFREE_BLOCK && a.rhs == 1) return launch_bsf(true, s);
    if (schedule == SPTRSV_SCHED_SYNCFREE_WINDOW && a.rhs == 1) return launch_window(true, s);
    return launch_pull_warp(true, s, rows_per_warp, 0);
}

}  // namespace sptrsv
