// mma.cuh -- warp-level BF16 tensor-core helpers shared by the supernodal panel kernels.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

namespace sptrsv {

// D += A B for one m16n8k16 tile: A 16x16 bf16 (row-major fragment), B 16x8 bf16, FP32 accumulators.
__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// A fragment (16 x 16, row-major) of G rows [row0, row0+16), columns [k0, k0+16); rows past
// `nrows` and columns past `K` read as zero (G is padded to a multiple of 16 columns).
__device__ __forceinline__ void load_a(const __nv_bfloat16* g, int L, int row0, int nrows, int k0, uint32_t* a) {
    const int lane = threadIdx.x & 31;
    const int r = lane >> 2, c = (lane & 3) * 2;
    const int ra = row0 + r, rb = row0 + r + 8;
    const uint32_t* pa = reinterpret_cast<const uint32_t*>(g + (size_t)ra * L + k0 + c);
    const uint32_t* pb = reinterpret_cast<const uint32_t*>(g + (size_t)rb * L + k0 + c);
    a[0] = ra < nrows ? __ldg(pa) : 0u;
    a[1] = rb < nrows ? __ldg(pb) : 0u;
    a[2] = ra < nrows ? __ldg(pa + 4) : 0u;
    a[3] = rb < nrows ? __ldg(pb + 4) : 0u;
}

}  // namespace sptrsv
