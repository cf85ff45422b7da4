// analysis.cu -- matrix checks and the dependency analysis of U, all on the device.
//
//  * validate: row pointer monotone and starting at 0, diagonal first in every row, every
//    other column in (i, n), finite non-zero pivot.  Also writes in_degree (row length,
//    diagonal included -- the value kernel_full.cl:40-52 accumulates over the CSC), the
//    reciprocal diagonal in FP64 and FP32, and the FP32 copy of the values.
//  * levels (core.cpp:244-270): level[i] = 1 for a diagonal-only row, else
//    1 + max(1, max_j level[j]); computed by a sync-free pull over the same dependency DAG
//    as the solve, with 0 as the "pending" value.  Bit-exact with the reference.
//  * level buckets (core.cpp:282-288): rows grouped by level, ascending within a level --
//    a stable LSD radix sort of the level keys.
//  * level tasks (core.cpp:289-332): the reference's greedy nnz-balanced split of each
//    level into num_threads tasks, one device thread per level, same integer arithmetic.
//  * CSR -> CSC transpose (utils.cpp:128-159): stable radix sort of the entries by column,
//    so each column lists its rows in ascending order and the diagonal lands last.
#include "common.cuh"
#include "kernels.cuh"

namespace sptrsv {

__global__ void k_validate(int n, int nnz, const int* __restrict__ rp, const int* __restrict__ col,
                           const double* __restrict__ val, int* __restrict__ in_degree, double* __restrict__ invd,
                           float* __restrict__ invd32, Ctl* ctl) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int s = rp[i], e = rp[i + 1];
        if ((i == 0 && s != 0) || e < s || e > nnz || s < 0) {
            record_error(ctl, SPTRSV_ERR_ROW_PTR);
            in_degree[i] = 0;
            continue;
        }
        in_degree[i] = e - s;
        if (e == s || col[s] != i) {
            record_error(ctl, SPTRSV_ERR_MISSING_DIAG);
            continue;
        }
        const double d = val[s];
        if (d == 0.0 || !isfinite(d)) record_error(ctl, SPTRSV_ERR_ZERO_PIVOT);
        invd[i] = 1.0 / d;
        invd32[i] = (float)(1.0 / d);
        for (int k = s + 1; k < e; ++k) {
            const int c = col[k];
            if (c < 0 || c >= n) { record_error(ctl, SPTRSV_ERR_COL_RANGE); break; }
            if (c <= i) { record_error(ctl, SPTRSV_ERR_NOT_UPPER); break; }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && rp[n] != nnz) record_error(ctl, SPTRSV_ERR_ROW_PTR);
}

__global__ void k_to_f32(size_t count, const double* __restrict__ a, float* __restrict__ b) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x)
        b[k] = (float)a[k];
}

// Per-row dominance ratio sum_j |U_ij| / |U_ii| (reduced to its maximum) and the sum of
// squared row lengths, used to choose schedules.
// Per-matrix statistics: max_i sum|off| / |diag|, sum of squared row lengths, the sum over rows
// of 1 / (distance to the row's nearest dependency), which is about the depth of the DAG when
// dependencies chain through their nearest columns (the levels themselves take a DAG traversal),
// and the number of rows that are not one contiguous column range from the diagonal (zero for a
// banded factor stored with its explicit zeros: a skyline matrix).
__global__ void k_row_stats(int n, const int* __restrict__ rp, const int* __restrict__ col,
                            const double* __restrict__ val, unsigned long long* max_ratio_bits,
                            unsigned long long* sum_len2, double* depth_sum, unsigned long long* gapped_rows) {
    double mr = 0.0, dep = 0.0;
    unsigned long long l2 = 0, gapped = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int s = rp[i], e = rp[i + 1];
        double off = 0.0;
        int near = n;
        bool contiguous = true;
        for (int k = s + 1; k < e; ++k) {
            off += fabs(val[k]);
            near = min(near, col[k] - i);
            contiguous &= col[k] == i + (k - s);
        }
        const double r = off / fabs(val[s]);
        mr = fmax(mr, r);
        if (e > s + 1) dep += 1.0 / (double)near;
        gapped += contiguous ? 0ull : 1ull;
        l2 += (unsigned long long)(e - s) * (unsigned long long)(e - s);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
        dep += __shfl_xor_sync(0xffffffffu, dep, o);
        l2 += __shfl_xor_sync(0xffffffffu, l2, o);
        gapped += __shfl_xor_sync(0xffffffffu, gapped, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(max_ratio_bits, (unsigned long long)__double_as_longlong(mr));  // mr >= 0: bit order = value order
        atomicAdd(sum_len2, l2);
        atomicAdd(depth_sum, dep);
        atomicAdd(gapped_rows, gapped);
    }
}

// levels: warp per row, rows claimed in reverse order through ctl->ticket2.
__global__ void __launch_bounds__(256) k_levels(int n, const int* __restrict__ rp, const int* __restrict__ col,
                                                int* level, Ctl* ctl, int64_t budget) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(&ctl->ticket2, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= (unsigned)n || aborted(ctl)) break;
        const int i = n - 1 - (int)t;
        const int s = rp[i], e = rp[i + 1];
        int m = 1;
        bool ok = true;
        for (int k = s + 1 + lane; k < e; k += 32) {
            const int* p = level + col[k];
            int v = ld_relaxed(p);
            if (v == 0) {
                const uint64_t t0 = gtimer();
                unsigned ns = 20;
                while ((v = ld_relaxed(p)) == 0) {
                    if (aborted(ctl)) { ok = false; break; }
                    if ((int64_t)(gtimer() - t0) > budget) { record_error(ctl, SPTRSV_ERR_TIMEOUT); ok = false; break; }
                    __nanosleep(ns);
                    if (ns < 200) ns += ns;
                }
                if (!ok) break;
            }
            m = max(m, v);
        }
        if (__any_sync(0xffffffffu, !ok)) break;
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) {
            const int lv = (e - s > 1) ? 1 + m : 1;
            st_relaxed(level + i, lv);
            atomicMax(&ctl->max_level, lv);
        }
    }
}

// ---------------------------------------------------------------------------------------
// Exclusive scan of int32 (count elements) -> out[0..count], out[count] = total.
constexpr int kScanThreads = 256, kScanItems = 16, kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
    __shared__ int warp_tot[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int w = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0;
        int wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        warp_tot[lane] = wi - w;  // exclusive prefix of warp totals
        __syncwarp();
    }
    __syncthreads();
    const int res = warp_tot[wid] + inc - v;
    if (total) {
        __shared__ int s_tot;
        if (threadIdx.x == blockDim.x - 1) s_tot = res + v;
        __syncthreads();
        *total = s_tot;
    }
    __syncthreads();
    return res;
}

__global__ void k_scan_partials(const int* in, int count, int* part) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) s += (base + q < count) ? in[base + q] : 0;
    int tot;
    block_exclusive_scan(s, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void k_scan_single(int* part, int count) {
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b = 0; b < count; b += blockDim.x) {
        const int i = b + threadIdx.x;
        const int v = (i < count) ? part[i] : 0;
        int tot;
        const int ex = block_exclusive_scan(v, &tot);
        if (i < count) part[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
}

__global__ void k_scan_final(const int* in, int count, const int* part, int* out) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) { v[q] = (base + q < count) ? in[base + q] : 0; s += v[q]; }
    int tot;
    int ex = block_exclusive_scan(s, &tot) + part[blockIdx.x];
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
        if (base + q < count) out[base + q] = ex;
        ex += v[q];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[count] = ex;
}

int scan_exclusive(const int* in, int* out, int count, int* part_scratch, cudaStream_t st, int64_t* launches) {
    if (count <= 0) {
        CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int), st));
        return 0;
    }
    const int nb = (count + kScanTile - 1) / kScanTile;
    k_scan_partials<<<nb, kScanThreads, 0, st>>>(in, count, part_scratch);
    k_scan_single<<<1, 1024, 0, st>>>(part_scratch, nb);
    k_scan_final<<<nb, kScanThreads, 0, st>>>(in, count, part_scratch, out);
    *launches += 3;
    CUDA_TRY(cudaGetLastError());
    return 0;
}
int scan_partials_needed(int count) { return (count + kScanTile - 1) / kScanTile + 1; }

// ---------------------------------------------------------------------------------------
// Stable LSD radix sort of (key, idx) pairs, 8-bit digits; one warp per tile, tiles in order.
constexpr int kRadixTile = 4096;  // items per warp-tile
constexpr int kRadixWarps = 4;    // warps per block

__global__ void k_radix_hist(const unsigned* __restrict__ keys, int count, int shift, int ntiles, int* __restrict__ hist) {
    __shared__ int cnt[kRadixWarps][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int tile = blockIdx.x * kRadixWarps + w;
    for (int d = lane; d < 256; d += 32) cnt[w][d] = 0;
    __syncwarp();
    if (tile < ntiles) {
        const int beg = tile * kRadixTile, end = min(count, beg + kRadixTile);
        for (int k = beg + lane; k < end; k += 32) atomicAdd(&cnt[w][(keys[k] >> shift) & 255u], 1);
    }
    __syncwarp();
    if (tile < ntiles)
        for (int d = lane; d < 256; d += 32) hist[d * ntiles + tile] = cnt[w][d];
}

__global__ void k_radix_scatter(const unsigned* __restrict__ keys, const int* __restrict__ idx, int count, int shift,
                                int ntiles, const int* __restrict__ offs, unsigned* __restrict__ keys_out,
                                int* __restrict__ idx_out) {
    __shared__ int cnt[kRadixWarps][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int tile = blockIdx.x * kRadixWarps + w;
    if (tile >= ntiles) return;
    for (int d = lane; d < 256; d += 32) cnt[w][d] = offs[d * ntiles + tile];
    __syncwarp();
    const int beg = tile * kRadixTile, end = min(count, beg + kRadixTile);
    const unsigned lt = (1u << lane) - 1u;
    for (int k0 = beg; k0 < end; k0 += 32) {
        const int k = k0 + lane;
        const bool valid = k < end;
        const unsigned active = __ballot_sync(0xffffffffu, valid);
        unsigned key = 0;
        int id = 0, d = 0, pos = 0;
        unsigned peers = 0;
        if (valid) {
            key = keys[k];
            id = idx ? idx[k] : k;
            d = (int)((key >> shift) & 255u);
            peers = __match_any_sync(active, d);
            pos = cnt[w][d] + __popc(peers & lt);
        }
        __syncwarp();
        if (valid && (__ffs(peers) - 1) == lane) cnt[w][d] += __popc(peers);
        __syncwarp();
        if (valid) { keys_out[pos] = key; idx_out[pos] = id; }
    }
}

// Sorts keys (count items, values < 2^key_bits) stably; writes the permutation into
// perm (perm[p] = original index of the p-th smallest).  Needs scratch:
// 2*count unsigned/int + 256*ntiles + scan partials.
int stable_sort_perm(const unsigned* keys_in, int count, int key_bits, int* perm, Scratch& scr, cudaStream_t st,
                     int64_t* launches) {
    if (count <= 0) return 0;
    const int ntiles = (count + kRadixTile - 1) / kRadixTile;
    const int nblocks = (ntiles + kRadixWarps - 1) / kRadixWarps;
    unsigned* ka = scr.take<unsigned>(count);
    unsigned* kb = scr.take<unsigned>(count);
    int* ia = scr.take<int>(count);
    int* ib = perm;
    const int hist_n = 256 * ntiles;
    int* hist = scr.take<int>(hist_n + 1);
    int* part = scr.take<int>(scan_partials_needed(hist_n));
    if (!ka || !kb || !ia || !hist || !part) return SPTRSV_ERR_CUDA;
    const int passes = key_bits <= 0 ? 1 : (key_bits + 7) / 8;
    const unsigned* kin = keys_in;
    const int* iin = nullptr;
    // ping-pong so that the last pass writes into perm
    unsigned* kouts[2] = {ka, kb};
    int* iouts[2] = {(passes % 2 == 1) ? ib : ia, (passes % 2 == 1) ? ia : ib};
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        k_radix_hist<<<nblocks, 32 * kRadixWarps, 0, st>>>(kin, count, shift, ntiles, hist);
        ++*launches;
        int rc = scan_exclusive(hist, hist, hist_n, part, st, launches);
        if (rc) return rc;
        unsigned* ko = kouts[p & 1];
        int* io = iouts[p & 1];
        k_radix_scatter<<<nblocks, 32 * kRadixWarps, 0, st>>>(kin, iin, count, shift, ntiles, hist, ko, io);
        ++*launches;
        kin = ko;
        iin = io;
    }
    CUDA_TRY(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------------------
__global__ void k_level_hist(int n, const int* __restrict__ level, int* __restrict__ cnt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) atomicAdd(&cnt[level[i]], 1);
}

// Passes over the levels of a level-set solve: out[0] = sum over levels of ceil(width / 32) (one
// CTA of 32 warps, a warp per row), out[1] = the same with 32 x `ctas` warps (the full grid).
__global__ void k_level_passes(int max_level, const int* __restrict__ lptr, int ctas, unsigned long long* out) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x + 1;
    unsigned p1 = 0, pg = 0;
    if (l <= max_level) {
        const unsigned w = (unsigned)(lptr[l + 1] - lptr[l]);
        p1 = (w + 31) / 32;
        pg = (w + 32u * ctas - 1) / (32u * ctas);
    }
    p1 = __reduce_add_sync(0xffffffffu, p1);
    pg = __reduce_add_sync(0xffffffffu, pg);
    if ((threadIdx.x & 31) == 0 && p1) {
        atomicAdd(&out[0], (unsigned long long)p1);
        atomicAdd(&out[1], (unsigned long long)pg);
    }
}

__global__ void k_level_tasks(int max_level, const int* __restrict__ lptr, const int* __restrict__ lrows,
                              const int* __restrict__ rp, int T, int* __restrict__ tasks) {
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l <= max_level; l += gridDim.x * blockDim.x) {
        int* t = tasks + (size_t)l * (T + 1);
        uint64_t level_nz = 0;
        for (int k = lptr[l]; k < lptr[l + 1]; ++k) {
            const int v = lrows[k];
            level_nz += (uint64_t)(rp[v + 1] - rp[v]);
        }
        const uint64_t limit = level_nz / (uint64_t)T;
        for (int j = 0; j <= T; ++j) t[j] = 0;
        int cur = 1;
        uint64_t cur_nz = 0;
        for (int k = lptr[l]; k < lptr[l + 1]; ++k) {
            const int v = lrows[k];
            const uint64_t len = (uint64_t)(rp[v + 1] - rp[v]);
            if (cur == T) { t[cur] += 1; continue; }
            if (len + cur_nz > limit) { cur_nz = len; cur++; t[cur] += 1; }
            else { t[cur] += 1; cur_nz += len; }
        }
        for (int j = 1; j <= T; ++j) t[j] += t[j - 1];
    }
}

// Row id of every entry (warp per row).
__global__ void k_entry_rows(int n, const int* __restrict__ rp, int* __restrict__ erow) {
    const int lane = threadIdx.x & 31;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += (gridDim.x * blockDim.x) >> 5)
        for (int k = rp[i] + lane; k < rp[i + 1]; k += 32) erow[k] = i;
}

__global__ void k_gather_csc(int nnz, const int* __restrict__ perm, const int* __restrict__ erow,
                             const double* __restrict__ val, int* __restrict__ crow, double* __restrict__ cval) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x) {
        const int k = perm[p];
        crow[p] = erow[k];
        cval[p] = val[k];
    }
}

__global__ void k_col_hist(int nnz, const int* __restrict__ col, int* __restrict__ cnt) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x) atomicAdd(&cnt[col[k]], 1);
}

// kernel_full.cl:40-52: in_degree[row_idx[k]] += 1 over every CSC entry.
__global__ void k_in_degree_csc(int nnz, const int* __restrict__ crow, int* __restrict__ indeg) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x) atomicAdd(&indeg[crow[k]], 1);
}

// CSC checks for the push solve: diagonal last in each column, other rows in [0, j).
__global__ void k_validate_csc(int n, int nnz, const int* __restrict__ cp, const int* __restrict__ crow,
                               const double* __restrict__ cval, double* __restrict__ invd, Ctl* ctl) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int s = cp[j], e = cp[j + 1];
        if ((j == 0 && s != 0) || e < s || e > nnz || s < 0) { record_error(ctl, SPTRSV_ERR_ROW_PTR); continue; }
        if (e == s || crow[e - 1] != j) { record_error(ctl, SPTRSV_ERR_MISSING_DIAG); continue; }
        const double d = cval[e - 1];
        if (d == 0.0 || !isfinite(d)) record_error(ctl, SPTRSV_ERR_ZERO_PIVOT);
        invd[j] = 1.0 / d;
        for (int k = s; k < e - 1; ++k) {
            const int r = crow[k];
            if (r < 0 || r >= n) { record_error(ctl, SPTRSV_ERR_COL_RANGE); break; }
            if (r >= j) { record_error(ctl, SPTRSV_ERR_NOT_UPPER); break; }
        }
    }
}

}  // namespace sptrsv
