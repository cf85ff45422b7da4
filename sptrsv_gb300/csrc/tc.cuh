// tc.cuh -- Blackwell tensor-core (tcgen05) and bulk-copy helpers in inline PTX, and the digit
// split of FP64 values used by the split-product panel kernels.
//
// Operand tiles in shared memory are K-major without swizzle: 8-row x 16-byte core matrices,
// the core matrices of one 8-row group adjacent along K (leading byte offset 128), the row groups
// one K extent apart (stride byte offset = K / 8 * 128).  The descriptor and instruction-descriptor
// fields follow the PTX ISA's tcgen05 shared-memory descriptor (start, leading and stride byte
// offsets in 16-byte units, version 1 at bit 46, no swizzle) and the kind::f16 instruction
// descriptor (F32 accumulator at bit 4, BF16 A and B at bits 7 and 10, N / 8 at bit 17, M / 16 at
// bit 24).  The accumulator of an M = 128, cta_group::1 MMA occupies TMEM lanes 0..127 (lane =
// row), one 32-bit column per output column; warp w of the CTA reads lanes 32 (w % 4) .. + 31.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include "common.cuh"

namespace sptrsv {
namespace tc {

__device__ __forceinline__ uint32_t smem(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ uint64_t desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
// byte offset of element (r, k) in a K-major tile with K extent kext
__host__ __device__ __forceinline__ int tile_off(int r, int k, int kext) {
    return (r >> 3) * (kext * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for phase `parity`: false on timeout (error recorded) or abort.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, Ctl* ctl, int64_t budget) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (aborted(ctl)) return false;
        if ((int64_t)(gtimer() - t0) > budget) {
            record_error(ctl, SPTRSV_ERR_TIMEOUT);
            return false;
        }
    }
}
// A wait that only ends early on its own bound (for copies and MMAs this CTA issued, which the
// hardware completes): used before returning, so nothing of ours is left in flight.
__device__ __forceinline__ void mbar_drain(uint64_t* bar, unsigned parity, int64_t budget) {
    const uint64_t t0 = gtimer();
    while (!mbar_try_wait(bar, parity) && (int64_t)(gtimer() - t0) <= budget) {
    }
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem(dst)),
                 "l"(src), "r"(bytes), "r"(smem(bar))
                 : "memory");
}

__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// TMEM allocation by one whole warp; the column base is written to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D (TMEM) = A * B (+ D when accumulate): one thread issues.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// The mbarrier completes when every MMA this thread issued before has finished.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem(bar))
                 : "memory");
}
// 16 consecutive 32-bit TMEM columns of this thread's lane, without waiting: the registers are
// valid after tmem_wait_ld (several loads can be in flight).
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// Placed after tmem_wait_ld: ties 16 loaded registers to a point after the wait, so no use of them
// is scheduled before it.
__device__ __forceinline__ void tmem_regs_after_wait(uint32_t* r) {
    asm volatile(""
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15]));
}
// 16 consecutive 32-bit TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// ---------------------------------------------------------------------------------------
// Digit split of FP64 values (the split-product scheme of Ozaki, Ogita, Oishi and Rump, 2012, in
// its fixed-point form): a row (or column) of values with common scale 2^e, e the smallest power
// with every |g| < 2^e, is written as g = 2^e sum_{p=1..8} d_p 2^(-7p) + (error below 2^(e-56)),
// with integer digits |d_p| <= 127 of |g|'s truncated 56-bit fixed-point fraction, signed like g.
// Products of two digits are below 2^14, so a 64-term dot product of digit vectors is below 2^20
// and up to eight such sums stay below 2^23: exact in FP32 accumulators.
constexpr int kDigits = 8;
constexpr int kDigitBits = 7;

// Smallest e with |g| < 2^e; kExpZero for g == 0.
constexpr int kExpZero = -2000;
__device__ __forceinline__ int exp_bound(double g) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(g) & 0x7FFFFFFFFFFFFFFFull;
    if (b == 0) return kExpZero;
    const int E = (int)(b >> 52);
    if (E == 0) return -1074 + (64 - __clzll((long long)b));  // subnormal: |g| = b * 2^-1074
    return E - 1022;
}
// The eight digits of g against the scale 2^e (e >= exp_bound(g)).
__device__ __forceinline__ void digits(double g, int e, float* d) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(g);
    const bool neg = (bits >> 63) != 0;
    const unsigned long long b = bits & 0x7FFFFFFFFFFFFFFFull;
    const int E = (int)(b >> 52);
    const unsigned long long m = E == 0 ? b : ((b & 0xFFFFFFFFFFFFFull) | (1ull << 52));
    const int ex = E == 0 ? -1074 : E - 1075;  // |g| = m * 2^ex
    int sh = ex - e + 56;                      // Y = trunc(|g| 2^(56 - e)) = m * 2^sh, sh <= 3
    unsigned long long Y = 0;
    if (m != 0) {
        if (sh > 3) sh = 3;
        Y = sh >= 0 ? (m << sh) : (sh > -64 ? (m >> -sh) : 0ull);
    }
#pragma unroll
    for (int p = 1; p <= kDigits; ++p) {
        const float v = (float)(int)((Y >> (56 - kDigitBits * p)) & 127ull);
        d[p - 1] = neg ? -v : v;
    }
}

}  // namespace tc
}  // namespace sptrsv
