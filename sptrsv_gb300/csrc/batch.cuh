// batch.cuh -- records shared by the batched path and the single-system supernodal path: system
// descriptors, dense panel chunks, and the exact FP64 panel kernel that both use.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include "common.cuh"

namespace sptrsv {

constexpr int kP64 = 64;      // columns of G per FP64 panel work item (and rows per panel)
constexpr int kP64Nc = 16;    // right-hand-side columns per pass of an FP64 panel work item
constexpr int kP64Near = 16;  // columns per block in the nearest solved region

// Right-hand-side columns per work item: 4 up to 16 columns, then 16 (at most kP64Nc), so that one
// item's work on the dependency chain stays short.  (Double-FP32 items of up to 16 columns, one G
// read for all of them, measured slower on the 512-system mix: 74.9 against 57.5 ms.)
__host__ __device__ __forceinline__ int p64_group_width(int rhs) { return rhs <= 16 ? 4 : kP64Nc; }
__host__ __device__ __forceinline__ int p64_groups(int rhs) {
    const int g = p64_group_width(rhs);
    return (rhs + g - 1) / g;
}

struct BSys {
    int n, rhs, sched, groups;  // groups: lanes per row in the row kernels (row_lanes)
    long long rp0, nz0, row0, xb0;
};

// A dense panel: rows [a + r0, a + r0 + pw) of a chunk whose rows [a, a + w) hold
// G = [T^-1 | -T^-1 Rect] (row-major, leading dimension ld, K = w + m columns; the first w
// columns multiply the chunk's own right-hand side, the others the solved rows rect[0 .. m)).
struct BChunk {
    int sys, a, w, m, ld, pad;
    const __nv_bfloat16* ghi;  // G ~ ghi + glo (two BF16 terms)
    const __nv_bfloat16* glo;
    const double* g64;         // G in FP64 (the exact panel schedule)
    const int* rect;
    long long poff;            // FP64 schedule: first partial-sum slot of the panel (doubles)
    int nblk;                  // FP64 schedule: column blocks of G
    int r0, pw;                // the panel's rows within the chunk
    int cbase;                 // FP64 schedule: first completion counter (one per RHS group)
    unsigned char* gtc;        // tensor-core FP64 schedule: the panel's digit-slice G records (panels_tc.cu)
    const float2* ghl;         // double-FP32 products: G 2^-e_r as FP32 pairs, laid out like g64 (or null)
    const int* gexp;           // their row exponents e_r, indexed by the chunk's row
};

// Column blocks of a panel's G (w own columns, then K - w solved columns): the own part in
// 64-column blocks; the nearest 64 solved columns in 16-column blocks (the rows published last, so
// only one narrow block per CTA lies on the dependency chain); then 64-column blocks.
__host__ __device__ __forceinline__ int p64_nown(int w) { return (w + kP64 - 1) / kP64; }
__host__ __device__ __forceinline__ int p64_nnear(int w, int K) {
    const int R = K - w;
    return R <= 0 ? 0 : min(kP64 / kP64Near, (R + kP64Near - 1) / kP64Near);
}
__host__ __device__ __forceinline__ int p64_nblk(int w, int K) {
    const int R = K - w;
    return p64_nown(w) + p64_nnear(w, K) + (R > kP64 ? (R - kP64 + kP64 - 1) / kP64 : 0);
}
__host__ __device__ __forceinline__ void p64_block(int w, int K, int blk, int& k0, int& kc) {
    const int no = p64_nown(w), nn = p64_nnear(w, K);
    if (blk < no) {
        k0 = blk * kP64;
        kc = min(kP64, w - k0);
    } else if (blk < no + nn) {
        k0 = w + (blk - no) * kP64Near;
        kc = min(kP64Near, K - k0);
    } else {
        k0 = w + kP64 + (blk - no - nn) * kP64;
        kc = min(kP64, K - k0);
    }
}

// Exact FP64 panel products over a ticketed queue of (panel, column block, RHS group) items
// (panels64.cu).  Batched (sys != nullptr): b and x are the arenas the systems' xb0 offsets index,
// items carry their group (block | group << 16), poff counts doubles and cbase counters.  One
// system (sys == nullptr, rhs columns, row-major n x rhs): every item runs for each of the
// p64_groups(rhs) groups, poff counts per column and cbase per group.  ncnt counters are cleared.
// Panels that carry double-FP32 copies of G (ghl) are multiplied in double-FP32.
int launch_panels64(const BSys* sys, int rhs, const double* b, double* x, Ctl* ctl, unsigned* ticket, int64_t budget,
                    const int2* items, unsigned nitems, const BChunk* panels, double* part, int* cnt, int ncnt,
                    int ctas_per_sm, int sm_count, cudaStream_t st, int64_t* launches);

// FP64-accurate panel products on the tensor cores (panels_tc.cu): the same items, partial sums
// and counters as launch_panels64, with tc_groups_host(rhs) groups per item for one system.  The
// panels' gtc records come from launch_tc_split over every (panel, block) pair in recs.
int launch_panels_tc(const BSys* sys, int rhs, const double* b, double* x, Ctl* ctl, unsigned* ticket, int64_t budget,
                     const int2* items, unsigned nitems, const BChunk* panels, double* part, int* cnt, int ncnt,
                     int sm_count, cudaStream_t st, int64_t* launches);
int launch_tc_split(const BChunk* panels, const int2* recs, int nrec, int sm_count, cudaStream_t st,
                    int64_t* launches);
size_t tc_panel_bytes(int w, int K);  // bytes of one panel's G records
int tc_groups_host(int rhs);
// Panel products of the exact FP64 schedules: 0 = FP64 FMAs (default), 1 = tensor cores
// (SPTRSV_PANELS=tc).
int panels_mode();
// Double-FP32 copies of every panel's G (ghl, gexp of each chunk; panels of one chunk share them):
// one CTA per panel writes its rows.
int launch_g_df(const BChunk* panels, int npanels, cudaStream_t st, int64_t* launches);

}  // namespace sptrsv
