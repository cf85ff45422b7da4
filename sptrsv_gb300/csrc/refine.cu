// refine.cu -- FP32 bulk solves with FP64 iterative refinement.
//
// One refinement step, all on the device (no host round trip, so the whole sequence can be
// captured in a CUDA graph):
//   r   = b - U x               FP64 SpMV over the FP64 values (k_residual); ||r_c||^2 per
//                               column is accumulated for the convergence test; r is also
//                               stored in FP32 as the inner right-hand side;
//   test                        k_check: rel = max_c ||r_c|| / ||b_c||; once rel <= tol the
//                               `done` flag is raised and every later kernel returns at once;
//   d  ~= U^{-1} r              FP32 inner solve, either
//                                 JACOBI: d <- D^{-1} (r - N d), `inner_sweeps` sweeps over
//                                 the FP32 values (fully parallel; converges for any
//                                 triangular U because N is nilpotent, fast when U is
//                                 diagonally dominant), or
//                                 an exact FP32 sync-free / level-set solve (solve.cu);
//   x  += d                     FP64 update (fused into the last Jacobi sweep).
// x starts at 0, so the first residual is b itself.
#include "common.cuh"
#include "kernels.cuh"

namespace sptrsv {

__device__ __forceinline__ bool is_done(const Ctl* ctl) { return *(volatile const int*)&ctl->done != 0; }

// ||b_c||^2 for row-major b (rhs <= 1024).
__global__ void k_colnorm2(int n, int rhs, const double* __restrict__ b, double* __restrict__ out) {
    extern __shared__ double acc[];
    for (int c = threadIdx.x; c < rhs; c += blockDim.x) acc[c] = 0.0;
    __syncthreads();
    const int per_pass = (blockDim.x / rhs) > 0 ? (blockDim.x / rhs) : 0;
    if (per_pass > 0 && (int)threadIdx.x < per_pass * rhs) {
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

// r = b - U x; r32 = (float)r; seed: d0 = D^{-1} r (Jacobi) or d0 = pending (exact inner).
// rhs == 1: LPR lanes per row.
template <int LPR>
__global__ void __launch_bounds__(256) k_residual_v(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                    const double* __restrict__ val, const double* __restrict__ invd,
                                                    const double* __restrict__ b, const double* __restrict__ x,
                                                    float* __restrict__ r32, float* __restrict__ d0, int seed,
                                                    double* __restrict__ rn2, const Ctl* ctl) {
    if (is_done(ctl)) return;
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
            r32[i] = (float)r;
            if (seed == 1) d0[i] = (float)(r * invd[i]);
            else if (seed == 2) d0[i] = __uint_as_float(kPend32);
            acc += r * r;
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) atomicAdd(&s_acc, acc);
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(rn2, s_acc);
}

// rhs > 1: warp per row, lanes over RHS columns, entries sequential.
__global__ void __launch_bounds__(256) k_residual_m(int n, int rhs, const int* __restrict__ rp,
                                                    const int* __restrict__ col, const double* __restrict__ val,
                                                    const double* __restrict__ invd, const double* __restrict__ b,
                                                    const double* __restrict__ x, float* __restrict__ r32,
                                                    float* __restrict__ d0, int seed, double* __restrict__ rn2,
                                                    const Ctl* ctl) {
    if (is_done(ctl)) return;
    extern __shared__ double s_acc[];
    for (int c = threadIdx.x; c < rhs; c += blockDim.x) s_acc[c] = 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long ws = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = w; i < n; i += ws) {
        const int s = rp[i], e = rp[i + 1];
        const double di = invd[i];
        for (int c = lane; c < rhs; c += 32) {
            double sum = 0.0;
            for (int k = s; k < e; ++k) sum = fma(val[k], x[(size_t)col[k] * rhs + c], sum);
            const size_t p = (size_t)i * rhs + c;
            const double r = b[p] - sum;
            r32[p] = (float)r;
            if (seed == 1) d0[p] = (float)(r * di);
            else if (seed == 2) d0[p] = __uint_as_float(kPend32);
            atomicAdd(&s_acc[c], r * r);
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < rhs; c += blockDim.x) atomicAdd(rn2 + c, s_acc[c]);
}

__global__ void k_check(int rhs, double* rn2, const double* bn2, Ctl* ctl, double tol, int step, int reset_ticket) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (ctl->done) return;
    double rel = 0.0;
    for (int c = 0; c < rhs; ++c) {
        const double r = rn2[c], bb = bn2[c];
        const double q = (bb > 0.0) ? sqrt(r / bb) : (r > 0.0 ? INFINITY : 0.0);
        rel = fmax(rel, q);
        rn2[c] = 0.0;
    }
    ctl->rel_res = rel;
    ctl->steps = step;
    if (rel <= tol) ctl->done = 1;
    if (reset_ticket) ctl->ticket = 0u;
}

// One Jacobi sweep: dst = D^{-1} (r - N src); last: x += D^{-1} (r - N src) instead.
template <int LPR>
__global__ void __launch_bounds__(256) k_jacobi_v(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                  const float* __restrict__ val, const float* __restrict__ invd,
                                                  const float* __restrict__ r, const float* __restrict__ src,
                                                  float* __restrict__ dst, double* __restrict__ x, int last,
                                                  const Ctl* ctl) {
    if (is_done(ctl)) return;
    const int lane = threadIdx.x & 31;
    const int gl = lane % LPR;
    const unsigned gmask = (LPR == 32) ? 0xffffffffu : (((1u << LPR) - 1u) << ((lane / LPR) * LPR));
    const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / LPR;
    const long long gstride = ((long long)gridDim.x * blockDim.x) / LPR;
    for (long long i = gid; i < n; i += gstride) {
        const int s = rp[i], e = rp[i + 1];
        float sum = 0.f;
        for (int k = s + 1 + gl; k < e; k += LPR) sum = fmaf(val[k], src[col[k]], sum);
#pragma unroll
        for (int o = LPR / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(gmask, sum, o);
        if (gl == 0) {
            const float d = (r[i] - sum) * invd[i];
            if (last) x[i] += (double)d;
            else dst[i] = d;
        }
    }
}

__global__ void __launch_bounds__(256) k_jacobi_m(int n, int rhs, const int* __restrict__ rp,
                                                  const int* __restrict__ col, const float* __restrict__ val,
                                                  const float* __restrict__ invd, const float* __restrict__ r,
                                                  const float* __restrict__ src, float* __restrict__ dst,
                                                  double* __restrict__ x, int last, const Ctl* ctl) {
    if (is_done(ctl)) return;
    const int lane = threadIdx.x & 31;
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long ws = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = w; i < n; i += ws) {
        const int s = rp[i], e = rp[i + 1];
        const float di = invd[i];
        for (int c = lane; c < rhs; c += 32) {
            float sum = 0.f;
            for (int k = s + 1; k < e; ++k) sum = fmaf(val[k], src[(size_t)col[k] * rhs + c], sum);
            const size_t p = (size_t)i * rhs + c;
            const float d = (r[p] - sum) * di;
            if (last) x[p] += (double)d;
            else dst[p] = d;
        }
    }
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

static int stream_grid(int sm_count) { return sm_count * 8; }

int launch_refine_init(const RefineArgs& a) {
    CUDA_TRY(cudaMemsetAsync(a.x, 0, sizeof(double) * (size_t)a.n * a.rhs, a.st));
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
    if (a.rhs == 1) {
        switch (lpr_for(a.n, a.nnz)) {
            case 4: k_residual_v<4><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val, a.invd, a.b, a.x, a.r32, a.d32[0], seed, a.rn2, a.ctl); break;
            case 8: k_residual_v<8><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val, a.invd, a.b, a.x, a.r32, a.d32[0], seed, a.rn2, a.ctl); break;
            case 16: k_residual_v<16><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val, a.invd, a.b, a.x, a.r32, a.d32[0], seed, a.rn2, a.ctl); break;
            default: k_residual_v<32><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val, a.invd, a.b, a.x, a.r32, a.d32[0], seed, a.rn2, a.ctl); break;
        }
    } else {
        k_residual_m<<<grid, 256, sizeof(double) * a.rhs, a.st>>>(a.n, a.rhs, a.rp, a.col, a.val, a.invd, a.b, a.x,
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

int launch_jacobi_sweep(const RefineArgs& a, int src, bool last) {
    const int grid = stream_grid(a.sm_count);
    const float* s = a.d32[src];
    float* d = a.d32[src ^ 1];
    if (a.rhs == 1) {
        switch (lpr_for(a.n, a.nnz)) {
            case 4: k_jacobi_v<4><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val32, a.invd32, a.r32, s, d, a.x, last, a.ctl); break;
            case 8: k_jacobi_v<8><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val32, a.invd32, a.r32, s, d, a.x, last, a.ctl); break;
            case 16: k_jacobi_v<16><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val32, a.invd32, a.r32, s, d, a.x, last, a.ctl); break;
            default: k_jacobi_v<32><<<grid, 256, 0, a.st>>>(a.n, a.rp, a.col, a.val32, a.invd32, a.r32, s, d, a.x, last, a.ctl); break;
        }
    } else {
        k_jacobi_m<<<grid, 256, 0, a.st>>>(a.n, a.rhs, a.rp, a.col, a.val32, a.invd32, a.r32, s, d, a.x, last, a.ctl);
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
                       const int* lptr, const int* lrows) {
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
    s.warps = 0;
    s.st = a.st;
    s.launches = a.launches;
    if (schedule == SPTRSV_SCHED_LEVELSET) return launch_levelset(true, s, max_level, lptr, lrows);
    k_gate_ticket<<<1, 32, 0, a.st>>>(a.ctl);
    ++*a.launches;
    if (schedule == SPTRSV_SCHED_SYNCFREE_THREAD && a.rhs == 1) return launch_pull_thread(true, s);
    return launch_pull_warp(true, s, rows_per_warp, 0);
}

}  // namespace sptrsv
