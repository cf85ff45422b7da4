// kernels.cuh -- internal declarations shared by the .cu translation units.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include "common.cuh"

namespace sptrsv {

// Bump allocator over one device buffer; take() returns nullptr when the buffer is full.
struct Scratch {
    char* base = nullptr;
    size_t cap = 0;
    size_t used = 0;
    template <typename T>
    T* take(size_t count) {
        size_t off = (used + 255) & ~(size_t)255;
        size_t bytes = count * sizeof(T);
        if (off + bytes > cap) return nullptr;
        used = off + bytes;
        return reinterpret_cast<T*>(base + off);
    }
};

// api.cu
__global__ void k_narrow_rp(int count, const int64_t* in, int* out, Ctl* ctl);

// analysis.cu
__global__ void k_validate(int n, int nnz, const int* rp, const int* col, const double* val, int* in_degree,
                           double* invd, float* invd32, Ctl* ctl);
__global__ void k_to_f32(size_t count, const double* a, float* b);
__global__ void k_row_stats(int n, const int* rp, const int* col, const double* val,
                            unsigned long long* max_ratio_bits, unsigned long long* sum_len2, double* depth_sum,
                            unsigned long long* gapped_rows);
__global__ void k_levels(int n, const int* rp, const int* col, int* level, Ctl* ctl, int64_t budget);
__global__ void k_level_hist(int n, const int* level, int* cnt);
__global__ void k_level_tasks(int max_level, const int* lptr, const int* lrows, const int* rp, int T, int* tasks);
__global__ void k_level_passes(int max_level, const int* lptr, int ctas, unsigned long long* out);
__global__ void k_entry_rows(int n, const int* rp, int* erow);
__global__ void k_gather_csc(int nnz, const int* perm, const int* erow, const double* val, int* crow, double* cval);
__global__ void k_col_hist(int nnz, const int* col, int* cnt);
__global__ void k_in_degree_csc(int nnz, const int* crow, int* indeg);
__global__ void k_validate_csc(int n, int nnz, const int* cp, const int* crow, const double* cval, double* invd,
                               Ctl* ctl);
int scan_exclusive(const int* in, int* out, int count, int* part_scratch, cudaStream_t st, int64_t* launches);
int scan_partials_needed(int count);
int stable_sort_perm(const unsigned* keys_in, int count, int key_bits, int* perm, Scratch& scr, cudaStream_t st,
                     int64_t* launches);

// solve.cu -- launchers (return sptrsv_status; add their launches to *launches)
struct SolveArgs {
    int n;
    const int* rp;
    const int* col;
    const void* val;     // double* or float*
    const void* invd;    // double* or float*
    const void* b;       // row-major n x rhs
    void* x;             // row-major n x rhs
    int rhs;
    Ctl* ctl;
    int64_t budget;
    int sm_count;
    int warps;           // resident warps to launch (0 = full occupancy)
    long long nnz;       // entries of U (0 = unknown); the window kernel sizes its CTA by it
    cudaStream_t st;
    int64_t* launches;
};
int launch_fill_pending(bool f32, void* x, size_t count, cudaStream_t st, int64_t* launches);
int launch_pull_warp(bool f32, const SolveArgs& a, int rows_per_warp, int rhs_tile);
int launch_pull_thread(bool f32, const SolveArgs& a);
int launch_bsf(bool f32, const SolveArgs& a);
int launch_push_csc(const SolveArgs& a, const int* cp, const int* crow, const double* cval, int* indeg_work,
                    double* left_sum);
int launch_levelset(bool f32, const SolveArgs& a, int max_level, const int* lptr, const int* lrows);
// window.cu: one CTA walks the rows in 32-row blocks with recent x in a shared-memory ring
int launch_window(bool f32, const SolveArgs& a);
int launch_window_levels(int n, long long nnz, const int* rp, const int* col, int* level, Ctl* ctl, int64_t budget,
                         cudaStream_t st,
                         int64_t* launches);
int window_warps();
int launch_transpose(bool to_row_major, const double* src, double* dst, int n, int rhs, cudaStream_t st,
                     int64_t* launches);

// supernodal.cu -- the panel work list and dense panels of a supernode partition
struct SnArgs {
    int nitems;
    const int* item_s;     // supernode of every work item (ticket order: supernodes in reverse)
    const int* item_p;     // 64-row panel of every work item
    const int* sstart;     // supernode chunk boundaries
    const int* mrect;      // rectangle width of every chunk
    const int* roff;       // first rectangle column of every chunk in rect_cols
    const int* rect_cols;  // rectangle column indices
    const long long* goff; // first element of every chunk's G = [T^-1 | -T^-1 Rect] (row-major)
    const int* ld;         // leading dimension of every chunk's G (w + m rounded up to 16)
};

// refine.cu
struct RefineArgs {
    int n, nnz, rhs;
    const int* rp;
    const int* col;
    const double* val;
    const float* val32;
    const double* invd;
    const float* invd32;
    const int2* off;   // interleaved (column, FP32 value) off-diagonals, or nullptr
    const int* roff;   // first off-diagonal slot of every row (rp[i] - i), padded, or nullptr
    int pairs;         // off/roff in the paired layout: every row's slots padded to an even count
    const int* jmeta;  // group-jagged layout (off holds its entries): per group lane (row << 27) | count
    const int* jbase;  // group-jagged layout: first entry of every 32-row group
    int sweep_kernel;  // 0 lane per row over entry pairs (default), 1 warp tiles, 2 lane per row,
                       // 3 tiles at 8 blocks/SM, 4 two rows per lane, 5 bulk-copy pipeline,
                       // 6 SELL slices, 7/8 lane per row with 4/8-entry batches, 9 warp per
                       // 32-row group over the group-jagged layout
    int nslices;       // SELL: slices of 32 rows
    const int* sell_perm;  // SELL: row of every slice lane (-1 = padding)
    const int* sell_len;   // SELL: entries per lane of every slice
    const int* sell_ptr;   // SELL: first entry of every slice
    const int2* sell;      // SELL: column-major slice entries
    const double* b;   // row-major n x rhs
    double* x;         // row-major n x rhs
    double* x_out;     // rhs == 1: device-accessible host copy of x that every matrix residual
                       // rewrites (so the converged x is on the host when the graph ends), or nullptr
    float* r32;        // n x rhs
    float* d32[2];     // n x rhs ping-pong
    double* rn2;       // rhs  (||r_c||^2)
    double* bn2;       // rhs  (||b_c||^2)
    Ctl* ctl;
    double tol;
    int64_t budget;
    int sm_count;
    cudaStream_t st;
    int64_t* launches;
};
int launch_build_offdiag(int n, const int* rp, const int* col, const double* val, int2* off, int* roff,
                         int roff_pad, int sm_count, cudaStream_t st, int64_t* launches);
// Paired layout: roff[i] = sum over rows j < i of their off-diagonal count rounded up to even
// (roff[n .. n + roff_pad] = the total); launch_pair_offsets fills roff (len2 and part are
// scratch of n and scan_partials_needed(n) ints), launch_build_offdiag_pairs the entries: a row of
// odd length ends with the pad entry (its own column, value 0).
// Group-jagged layout of the `jds` sweep (32-row groups, rows ranked longest first, jagged
// diagonals contiguous): launch_jds_sizes writes every group's entry count into gsize (n/32
// rounded up ints) and sets *overflow when a row has 2^27 or more entries; after an exclusive scan
// of gsize into jbase, launch_jds_fill writes jmeta (32 ints per group) and the entries.
int launch_jds_sizes(int n, const int* rp, int* gsize, int* overflow, int sm_count, cudaStream_t st,
                     int64_t* launches);
int launch_jds_fill(int n, const int* rp, const int* col, const double* val, const int* jbase, int* jmeta, int2* jent,
                    int sm_count, cudaStream_t st, int64_t* launches);
int launch_pair_offsets(int n, const int* rp, int* len2, int* roff, int roff_pad, int* part, int sm_count,
                        cudaStream_t st, int64_t* launches);
int launch_build_offdiag_pairs(int n, const int* rp, const int* col, const double* val, const int* roff, int2* off,
                               int sm_count, cudaStream_t st, int64_t* launches);
int sell_prepare(int n, const int* rp, int* perm, int* slen, int* sptr, int* part, int sm_count, cudaStream_t st,
                 int64_t* launches, int* total);
int sell_fill(int n, const int* rp, const int* col, const double* val, const int* perm, const int* slen,
              const int* sptr, int2* sell, int sm_count, cudaStream_t st, int64_t* launches);
int sell_slices(int n);
int launch_refine_init(const RefineArgs& a, bool mark_zero);
int launch_residual(const RefineArgs& a, bool jacobi_seed, int final_check);
int launch_check(const RefineArgs& a, int step, bool reset_ticket);
int launch_check_outer(const RefineArgs& a, int max_refine, cudaGraphConditionalHandle ho,
                       cudaGraphConditionalHandle hi);
int launch_check_inner(const RefineArgs& a, float eps, int max_sweeps, cudaGraphConditionalHandle hi);
int launch_jacobi_sweep(const RefineArgs& a, int src, bool last, bool stats);
int launch_axpy_pending(const RefineArgs& a, int src);
int launch_exact_inner(const RefineArgs& a, int schedule, int rows_per_warp, int dst, int max_level,
                       const int* lptr, const int* lrows, int warps);

}  // namespace sptrsv
