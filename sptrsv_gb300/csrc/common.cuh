// common.cuh -- device helpers shared by every kernel of the solver.
//
// Completion signalling: the solution vector is its own flag array.  Before a sync-free
// solve every x entry is set to a signalling-NaN bit pattern (the "pending" sentinel); a
// row publishes its result with one aligned store of the final value, and a consumer polls
// the value itself with an L1-bypassing relaxed load until it differs from the sentinel.
// A single aligned 8- or 4-byte access is single-copy atomic, so no fence or separate flag
// is needed, which removes one memory round trip from every dependency hop.  GPU arithmetic
// never produces this pattern (its NaN results are canonical); a computed value that equals
// it is replaced by the canonical NaN before it is stored.
//
// Every spin is bounded: it gives up after `budget_ns` of %globaltimer time, records
// SPTRSV_ERR_TIMEOUT in the control block, raises the abort flag that every other waiter
// polls, and returns false.  No kernel traps, asserts or waits unboundedly.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/sptrsv_gb300.h"

namespace sptrsv {

constexpr uint64_t kPend64 = 0xFFF4535054525356ull;  // signalling NaN, payload "SPTRSV"
constexpr uint32_t kPend32 = 0xFFA5A5A5u;            // signalling NaN (FP32)
constexpr int64_t kDefaultBudgetNs = 2000000000ll;   // 2 s per wait

// Per-handle control block in device memory (zeroed before each solve).
struct Ctl {
    unsigned int ticket;   // next row ticket (rows are claimed in reverse order)
    int status;            // first error (0 = ok)
    int abort;             // set when any waiter gives up
    int done;              // MIXED: residual reached the tolerance
    unsigned long long bar_count;  // grid barrier arrivals (monotonic within a solve)
    int steps;             // MIXED: refinement steps taken
    int max_level;         // analysis: largest level
    double rnorm2;         // MIXED: ||r||^2 of the last residual
    double bnorm2;         // MIXED: ||b||^2
    double rel_res;        // MIXED: last relative residual
    unsigned int ticket2;  // second ticket (analysis kernels)
    unsigned int dmax_bits;  // MIXED + JACOBI: max |d| of the last checked sweep (float bits)
    unsigned int dchg_bits;  // MIXED + JACOBI: max |d_new - d_old| of the last checked sweep
    int inner_count;       // MIXED + JACOBI: sweeps of the current inner solve
    int inner_total;       // MIXED + JACOBI: sweeps over the whole solve
    int x_zero;            // MIXED: x is still the zero start vector (the residual is b)
    float inner_eps;       // MIXED + JACOBI: change test of the next inner solve, from the last residual
};

template <typename T> struct Pend;
template <> struct Pend<double> {
    static __device__ __forceinline__ double value() { return __longlong_as_double((long long)kPend64); }
    static __device__ __forceinline__ bool is(double v) { return (uint64_t)__double_as_longlong(v) == kPend64; }
    static __device__ __forceinline__ double fix(double v) {
        return is(v) ? __longlong_as_double(0x7FFFFFFFFFFFFFFFll) : v;
    }
};
template <> struct Pend<float> {
    static __device__ __forceinline__ float value() { return __uint_as_float(kPend32); }
    static __device__ __forceinline__ bool is(float v) { return __float_as_uint(v) == kPend32; }
    static __device__ __forceinline__ float fix(float v) { return is(v) ? __uint_as_float(0x7FFFFFFFu) : v; }
};

__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Coherent (L1-bypassing) loads and stores at GPU scope.
__device__ __forceinline__ double ld_relaxed(const double* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return __longlong_as_double((long long)v);
}
__device__ __forceinline__ float ld_relaxed(const float* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return __uint_as_float(v);
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(double* p, double v) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"((uint64_t)__double_as_longlong(v)) : "memory");
}
__device__ __forceinline__ void st_relaxed(float* p, float v) {
    asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(__float_as_uint(v)) : "memory");
}
__device__ __forceinline__ void st_relaxed(int* p, int v) {
    asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_release_add(int* p, int v) {
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void record_error(Ctl* ctl, int code) {
    atomicCAS(&ctl->status, 0, code);
    atomicExch(&ctl->abort, 1);
}
__device__ __forceinline__ bool aborted(const Ctl* ctl) { return ld_relaxed(&ctl->abort) != 0; }

// Wait until *p is no longer the pending sentinel.  Returns false on timeout or abort.
template <typename T>
__device__ __forceinline__ bool wait_ready(const T* p, T& out, Ctl* ctl, int64_t budget_ns) {
    T v = ld_relaxed(p);
    if (!Pend<T>::is(v)) { out = v; return true; }
    const uint64_t t0 = gtimer();
    unsigned ns = 20;
    for (;;) {
        __nanosleep(ns);
        v = ld_relaxed(p);
        if (!Pend<T>::is(v)) { out = v; return true; }
        if (aborted(ctl)) return false;
        if ((int64_t)(gtimer() - t0) > budget_ns) { record_error(ctl, SPTRSV_ERR_TIMEOUT); return false; }
        if (ns < 200) ns += ns;
    }
}

// Wait until *p == want (acquire).  Returns false on timeout or abort.
__device__ __forceinline__ bool wait_equal(const int* p, int want, Ctl* ctl, int64_t budget_ns) {
    if (ld_acquire(p) == want) return true;
    const uint64_t t0 = gtimer();
    unsigned ns = 20;
    for (;;) {
        __nanosleep(ns);
        if (ld_acquire(p) == want) return true;
        if (aborted(ctl)) return false;
        if ((int64_t)(gtimer() - t0) > budget_ns) { record_error(ctl, SPTRSV_ERR_TIMEOUT); return false; }
        if (ns < 200) ns += ns;
    }
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v, unsigned mask = 0xffffffffu) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
    return v;
}

// Grid-wide barrier for a cooperative launch, bounded: returns false on timeout/abort.
// Arrivals count up in ctl->bar_count and the count is never reset inside a solve: the k-th
// arrival (from 0) belongs to barrier generation k / nblocks, which is complete once the count
// reaches (k / nblocks + 1) * nblocks.  Every launch of a solve runs the same grid and passes the
// same number of barriers in every CTA, so the count is a multiple of nblocks between launches
// (the control block is cleared at the start of every solve).  One acq_rel atomic per CTA and
// acquire polls of the same word: the last arrival releases everybody with its own add, with no
// second store to wait for.
__device__ __forceinline__ unsigned long long atom_add_acq_rel(unsigned long long* p, unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ bool grid_barrier(Ctl* ctl, unsigned nblocks, int64_t budget_ns) {
    __syncthreads();
    if (nblocks == 1) return true;  // one CTA: the CTA barrier orders its global accesses
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned long long k = atom_add_acq_rel(&ctl->bar_count, 1ull);
        const unsigned long long target = (k / nblocks + 1) * nblocks;
        if (k + 1 != target) {
            // poll without sleeping first (a level usually ends within microseconds), then back off;
            // the timer and the abort flag are read every 64 polls
            uint64_t t0 = 0;
            unsigned it = 0;
            while (ld_acquire(&ctl->bar_count) < target) {
                if ((++it & 63u) == 0) {
                    if (aborted(ctl)) { ok = 0; break; }
                    if (t0 == 0) t0 = gtimer();
                    else if ((int64_t)(gtimer() - t0) > budget_ns) { record_error(ctl, SPTRSV_ERR_TIMEOUT); ok = 0; break; }
                }
                if (it > 4096) __nanosleep(32);
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

}  // namespace sptrsv

#define CUDA_TRY(expr)                                                   \
    do {                                                                 \
        cudaError_t _e = (expr);                                         \
        if (_e != cudaSuccess) return ::sptrsv::set_cuda_error(_e, #expr); \
    } while (0)

namespace sptrsv {
int set_cuda_error(cudaError_t e, const char* what);
}
