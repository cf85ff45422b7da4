// batch.cu -- many independent upper-triangular systems of uneven size and RHS count solved
// together from one packed device arena.
//
// Arena: the systems' CSR matrices one after another (each with its own local int32 row
// pointer, column indices local to the system), FP32 copies of the values, the inverse
// diagonals, and per-system descriptors (BSys) with the offsets of every part.  Right-hand sides
// and solutions are row-major n x rhs per system, one system after another.
//
// Two solve modes, each one CUDA graph:
//   * plain: every system by the FP64 sync-free pull (warp per row, RHS columns across lanes)
//     in ONE persistent launch over a device work queue that interleaves the systems row by row
//     from their last rows (queue position t holds row n_s - 1 - t of every system still that
//     long), so all systems advance together and the longest chain sets the makespan;
//   * chosen: every system by its own schedule (BS_*), the mixed ones inside one device-driven
//     FP64 iterative refinement (conditional WHILE nodes): per step an FP32 inner solve (Jacobi
//     sweeps to a relative change test, BF16x3 tensor-core products over dense panels, or the
//     FP32 sync-free pull), x += d in FP64 and the FP64 residual r = b - U x, until every
//     system's ||r||_F / ||b||_F <= tol.  Converged systems drop out of the later steps.
//     Systems scheduled BS_PLAIN are solved exactly in FP64 first, by the same persistent pull;
//     systems scheduled BS_PANEL64 exactly in FP64 on their dense panels, each panel's product
//     split into 64-column blocks taken by different CTAs (the FP64 work spreads over the GPU,
//     only the block of the nearest solved rows lies on the dependency chain).
//
// Every wait is a bounded pending-sentinel poll (common.cuh); per-system reductions are flushed
// once per run of rows of one system, so no address sees one atomic per row.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <cuda_bf16.h>
#include "common.cuh"
#include "kernels.cuh"
#include "handle.cuh"
#include "mma.cuh"
#include "batch.cuh"

namespace sptrsv {

enum { BS_PLAIN = 0, BS_JACOBI = 1, BS_PANEL = 2, BS_SF32 = 3, BS_PANEL64 = 4, BS_COUNT = 5 };

constexpr int kBPanel = 64;     // rows per panel work item (4 warps x 16-row MMA tiles)
constexpr int kBKc = 64;        // K rows staged per chunk (a multiple of 16: chunk starts stay aligned)
constexpr int kBNc = 32;        // right-hand-side columns per pass
constexpr int kBRowChunk = 32;  // rows per warp task in the row kernels
constexpr int kBatchKinds = 14;  // kernel kinds of the profiled replay
constexpr int kP64CtasPerSm = 4; // FP64 panel CTAs per SM beside the refinement (measured: 2: 190, 3: 137, 4: 135, 5: 146 ms)



struct BState {
    double bnorm2, rnorm2, rel;
    int done;  // 0 refining, 1 converged, 2 gave up
    int steps, status;
    int inner_done, inner_count, final_idx;
    unsigned dmax_bits, dchg_bits;
    unsigned ratio_bits;  // analysis: max_i sum|off| / |diag| (float bits)
    int sweeps;           // Jacobi sweeps over the whole solve
    int gapped;           // analysis: some row is not one contiguous column range from its diagonal
    int pad;
};

struct BCtl {
    Ctl c;
    int active;      // mixed systems still refining
    int jac_active;  // Jacobi systems still sweeping in this step
    int sweep_k;     // sweep index inside the current inner solve
    int outer;       // refinement steps taken
    int total_sweeps;
    int nmixed;
    unsigned ticket_p64;  // work queue of the exact FP64 panels (runs beside the refinement)
    int pad;
};



// A list of systems with the prefix of their row (or element) counts.
struct SegList {
    const int* sys;
    const long long* off;  // nseg + 1 entries
    int nseg;
    long long total;
};

struct BArgs {
    const BSys* sys;
    BState* st;
    BCtl* bc;
    const int* rp;
    const int* col;
    const double* val;
    const float* val32;
    double* invd;
    float* invd32;
    const double* b;
    double* x;
    float* r32;
    float* d0;
    float* d1;
    int64_t budget;
    double tol;
    float inner_eps;
    int max_refine, max_sweeps;
};

__device__ __forceinline__ int seg_find(const SegList& L, long long q) {
    int lo = 0, hi = L.nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (L.off[mid] <= q) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Lanes of a warp on one row: nc RHS columns side by side, groups = floor(32 / nc) strided walks
// over the row's entries; lane = g * nc + c (lanes from groups * nc on stay idle).
__device__ __forceinline__ void lane_split(int nc, int& groups, int& g, int& c) {
    groups = 32 / nc;
    const int lane = threadIdx.x & 31;
    g = lane / nc;
    c = lane - g * nc;
}

// Sum over the groups of each column, into the lanes of group 0 (a guarded tree: any group count).
template <typename T>
__device__ __forceinline__ T group_sum(T v, int groups, int nc) {
    const int g = (threadIdx.x & 31) / nc;
    for (int off = 1; off < groups; off <<= 1) {
        const T o = __shfl_down_sync(0xffffffffu, v, off * nc);
        if ((g & (2 * off - 1)) == 0 && g + off < groups) v += o;
    }
    return v;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Warp-wide iteration over a row list in tasks of kBRowChunk consecutive rows; f(seg, sys, i)
// per row, flush(sys) whenever the system changes and at the end of each task.
template <typename F, typename Flush>
__device__ __forceinline__ void for_rows(const SegList& rows, F f, Flush flush) {
    const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long t = gw; t * kBRowChunk < rows.total; t += nw) {
        const long long q0 = t * kBRowChunk, q1 = min(rows.total, q0 + kBRowChunk);
        int seg = seg_find(rows, q0);
        int cur = rows.sys[seg];
        for (long long q = q0; q < q1; ++q) {
            while (q >= rows.off[seg + 1]) ++seg;
            const int s = rows.sys[seg];
            if (s != cur) { flush(cur); cur = s; }
            f(s, (int)(q - rows.off[seg]));
        }
        flush(cur);
    }
}

// --- analysis ----------------------------------------------------------------------------------

// Warp per row of every system: diagonal first and nonzero, off-diagonals strictly right of it
// and inside the system; inverse diagonals (FP64, FP32); per-system max row ratio.
__global__ void __launch_bounds__(256) k_b_setup(BArgs A, SegList rows) {
    const int lane = threadIdx.x & 31;
    float rmax = 0.f;
    for_rows(
        rows,
        [&](int s, int i) {
            const BSys S = A.sys[s];
            const int* rp = A.rp + S.rp0;
            const int beg = rp[i], end = rp[i + 1];
            const int* cl = A.col + S.nz0;
            const double* vl = A.val + S.nz0;
            int bad = end <= beg ? SPTRSV_ERR_MISSING_DIAG : 0;
            double off = 0.0;
            int gap = 0;
            if (!bad) {
                for (int k = beg + 1 + lane; k < end; k += 32) {
                    const int j = cl[k];
                    if (j <= i) bad = SPTRSV_ERR_NOT_UPPER;
                    else if (j >= S.n) bad = SPTRSV_ERR_COL_RANGE;
                    gap |= j != i + (k - beg);
                    off += fabs(vl[k]);
                }
            }
            bad = __reduce_min_sync(0xffffffffu, bad);  // statuses are negative: min = any error
            gap = __reduce_or_sync(0xffffffffu, gap);
            off = warp_sum(off);
            if (gap && lane == 0 && !A.st[s].gapped) A.st[s].gapped = 1;
            if (!bad) {
                if (cl[beg] != i) bad = SPTRSV_ERR_MISSING_DIAG;
                else if (vl[beg] == 0.0) bad = SPTRSV_ERR_ZERO_PIVOT;
            }
            if (bad) {
                if (lane == 0) {
                    atomicCAS(&A.st[s].status, 0, bad);
                    atomicCAS(&A.bc->c.status, 0, bad);
                }
                return;
            }
            const double d = vl[beg];
            if (lane == 0) {
                A.invd[S.row0 + i] = 1.0 / d;
                A.invd32[S.row0 + i] = (float)(1.0 / d);
            }
            rmax = fmaxf(rmax, (float)(off / fabs(d)));
        },
        [&](int s) {
            if (lane == 0 && rmax > 0.f) atomicMax(&A.st[s].ratio_bits, __float_as_uint(rmax));
            rmax = 0.f;
        });
}

// --- element kernels ---------------------------------------------------------------------------

// x := pending sentinel over a list of systems' solution elements (all of them, or only the
// systems still refining when `only_active`).
template <typename T>
__global__ void k_b_fill_pending(BArgs A, SegList el, T* x, bool only_active) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < el.total;
         e += (long long)gridDim.x * blockDim.x) {
        const int seg = seg_find(el, e);
        const int s = el.sys[seg];
        if (only_active && A.st[s].done) continue;
        x[A.sys[s].xb0 + (e - el.off[seg])] = Pend<T>::value();
    }
}

// Mixed systems: x = 0, r = b (in FP32: the first inner right-hand side), ||b||^2 per system.
__global__ void k_b_init_mixed(BArgs A, SegList el) {
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long base0 = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31);
    for (long long wb = base0; wb < el.total; wb += stride) {  // warp-uniform trip count
        const long long e = wb + lane;
        int s = -1;
        double v = 0.0;
        if (e < el.total) {
            const int seg = seg_find(el, e);
            s = el.sys[seg];
            const long long o = A.sys[s].xb0 + (e - el.off[seg]);
            const double bv = A.b[o];
            A.x[o] = 0.0;
            A.r32[o] = (float)bv;
            v = bv * bv;
        }
        const int s0 = __shfl_sync(0xffffffffu, s, 0);
        if (__all_sync(0xffffffffu, s == s0)) {
            v = warp_sum(v);
            if (lane == 0 && s0 >= 0) atomicAdd(&A.st[s0].bnorm2, v);
        } else if (s >= 0) {
            atomicAdd(&A.st[s].bnorm2, v);
        }
    }
}

// x += d (the correction buffer that finished the system's inner solve), systems still refining.
__global__ void k_b_axpy(BArgs A, SegList el) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < el.total;
         e += (long long)gridDim.x * blockDim.x) {
        const int seg = seg_find(el, e);
        const int s = el.sys[seg];
        const BState& S = A.st[s];
        if (S.done) continue;
        const long long o = A.sys[s].xb0 + (e - el.off[seg]);
        const float d = (S.final_idx ? A.d1 : A.d0)[o];
        A.x[o] += (double)d;
    }
}

// --- FP64 / FP32 sync-free pull (persistent, ticketed work queue) -------------------------------

// Warp per row taken from `order` by ticket; the row waits on its solved columns (pending-sentinel
// polls), sums in its lane groups, and publishes x_i = (b_i - sum) * invd_i.  Rows of one system
// appear in the queue after every row they depend on, so the ticket order alone guarantees
// progress.
template <typename T>
__global__ void __launch_bounds__(256) k_b_pull(BArgs A, const int2* __restrict__ order, unsigned count,
                                                const T* __restrict__ bsrc, T* xdst, const T* __restrict__ vals,
                                                const T* __restrict__ invd, int which_ticket, bool skip_done) {
    Ctl* ctl = &A.bc->c;
    unsigned* ticket = which_ticket ? &ctl->ticket2 : &ctl->ticket;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned t = 0;
        if (lane == 0) t = aborted(ctl) ? 0xFFFFFFFFu : atomicAdd(ticket, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= count) break;
        const int2 it = order[t];
        if (skip_done && A.st[it.x].done) continue;
        const BSys S = A.sys[it.x];
        const int i = it.y, r = S.rhs;
        const int* rp = A.rp + S.rp0;
        const int beg = __ldg(rp + i), end = __ldg(rp + i + 1);
        const int* cl = A.col + S.nz0;
        const T* vl = vals + S.nz0;
        const T* bb = bsrc + S.xb0;
        T* xx = xdst + S.xb0;
        const T dinv = invd[S.row0 + i];
        bool ok = true;
        for (int c0 = 0; c0 < r; c0 += 32) {
            const int nc = min(32, r - c0);
            int groups, g, c;
            lane_split(nc, groups, g, c);
            T s0 = 0, s1 = 0, s2 = 0, s3 = 0;
            bool lok = true;
            if (g < groups) {
                // entries from the farthest column down to the nearest: the far ones were solved
                // long ago, so when the nearest (the last to be published) arrives only its own
                // product is left; four loads issue together and only a pending value waits
                int k = end - 1 - g;
                for (; lok && k - 3 * groups > beg; k -= 4 * groups) {
                    const T* p0 = xx + (size_t)__ldg(cl + k) * r + c0 + c;
                    const T* p1 = xx + (size_t)__ldg(cl + k - groups) * r + c0 + c;
                    const T* p2 = xx + (size_t)__ldg(cl + k - 2 * groups) * r + c0 + c;
                    const T* p3 = xx + (size_t)__ldg(cl + k - 3 * groups) * r + c0 + c;
                    T v0 = ld_relaxed(p0), v1 = ld_relaxed(p1), v2 = ld_relaxed(p2), v3 = ld_relaxed(p3);
                    if (Pend<T>::is(v0)) lok = wait_ready<T>(p0, v0, ctl, A.budget);
                    if (lok && Pend<T>::is(v1)) lok = wait_ready<T>(p1, v1, ctl, A.budget);
                    if (lok && Pend<T>::is(v2)) lok = wait_ready<T>(p2, v2, ctl, A.budget);
                    if (lok && Pend<T>::is(v3)) lok = wait_ready<T>(p3, v3, ctl, A.budget);
                    s0 = fma(__ldg(vl + k), v0, s0);
                    s1 = fma(__ldg(vl + k - groups), v1, s1);
                    s2 = fma(__ldg(vl + k - 2 * groups), v2, s2);
                    s3 = fma(__ldg(vl + k - 3 * groups), v3, s3);
                }
                for (; lok && k > beg; k -= groups) {
                    T xv;
                    if (!wait_ready<T>(xx + (size_t)__ldg(cl + k) * r + c0 + c, xv, ctl, A.budget)) {
                        lok = false;
                        break;
                    }
                    s0 = fma(__ldg(vl + k), xv, s0);
                }
            }
            T sum = group_sum((s0 + s1) + (s2 + s3), groups, nc);
            if (__any_sync(0xffffffffu, !lok)) { ok = false; break; }
            if (lane < nc) {
                const size_t o = (size_t)i * r + c0 + lane;
                st_relaxed(xx + o, Pend<T>::fix((bb[o] - sum) * dinv));
            }
        }
        if (!ok) break;
    }
}

// --- BF16x3 panel products (persistent) -------------------------------------------------------

// One 64-row panel of a dense chunk G = [T^-1 | -T^-1 Rect] per work item: d[rows] = G [r ; d_R].
// The panel's own right-hand side chunk first, then the solved columns farthest-first, so the
// columns solved last (the nearest rows) are waited on last.  Items of converged systems are skipped (nobody waits on them: only the same system's
// panels read its rows).
__global__ void __launch_bounds__(128, 4) k_b_panels(BArgs A, const int2* __restrict__ items, unsigned nitems,
                                                  const BChunk* __restrict__ chunks) {
    __shared__ __align__(16) __nv_bfloat16 Vhi[kBNc][kBKc + 8];
    __shared__ __align__(16) __nv_bfloat16 Vlo[kBNc][kBKc + 8];
    __shared__ unsigned s_t;
    __shared__ int s_ok;
    Ctl* ctl = &A.bc->c;
    const int lane = threadIdx.x & 31, wv = threadIdx.x >> 5;
    for (;;) {
        if (threadIdx.x == 0) s_t = aborted(ctl) ? 0xFFFFFFFFu : atomicAdd(&ctl->ticket, 1u);
        __syncthreads();
        const unsigned t = s_t;
        __syncthreads();
        if (t >= nitems) break;
        const int2 it = items[t];
        const BChunk C = chunks[it.x];
        if (A.st[C.sys].done) continue;
        const BSys S = A.sys[C.sys];
        const int a = C.a, w = C.w, K = C.w + C.m, L = C.ld, rhs = S.rhs;
        const float* b = A.r32 + S.xb0;
        float* x = A.d0 + S.xb0;
        const int row0 = it.y * kBPanel + 16 * wv;  // this warp's 16-row tile
        bool ok = true;
        for (int c0 = 0; c0 < rhs; c0 += kBNc) {
            const int nc = min(kBNc, rhs - c0);
            const int nc8 = (nc + 7) & ~7;
            float acc[kBNc / 8][4];
#pragma unroll
            for (int q = 0; q < kBNc / 8; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
            // chunk 0 (the panel's own right-hand side, never waited on) first, then the solved
            // columns from the farthest chunk to the nearest, so that only the last chunk's
            // products follow the arrival of the rows solved just before this panel
            const int nk = (K + kBKc - 1) / kBKc;
            for (int ci = 0; ci < nk; ++ci) {
                const int kb = ci == 0 ? 0 : nk - ci;
                const int k0 = kb * kBKc, kc = min(kBKc, K - k0);
                // this chunk's G fragments are loaded before any wait on solved columns, so their
                // memory latency overlaps the wait instead of following it
                uint32_t ahs[kBKc / 16][4], als[kBKc / 16][4];
#pragma unroll
                for (int u = 0; u < kBKc / 16; ++u) {
                    if (row0 < w && u * 16 < kc) {
                        load_a(C.ghi, L, row0, w, k0 + u * 16, ahs[u]);
                        load_a(C.glo, L, row0, w, k0 + u * 16, als[u]);
                    }
                }
                if (threadIdx.x == 0) s_ok = 1;
                __syncthreads();
                // every element of the chunk is loaded first (independent loads in flight together),
                // then only the solved-column values still pending are waited on
                constexpr int kStage = kBKc * kBNc / 128;
                const int tot = kBKc * nc8;
                float v[kStage];
#pragma unroll
                for (int u = 0; u < kStage; ++u) {
                    const int e = threadIdx.x + u * 128;
                    float val = 0.f;
                    if (e < tot) {
                        const int j = e / kBKc, kk = e - j * kBKc, k = k0 + kk;
                        if (kk < kc && j < nc)
                            val = k < w ? b[(size_t)(a + k) * rhs + c0 + j]
                                        : ld_relaxed(x + (size_t)C.rect[k - w] * rhs + c0 + j);
                    }
                    v[u] = val;
                }
#pragma unroll
                for (int u = 0; u < kStage; ++u) {
                    const int e = threadIdx.x + u * 128;
                    if (e < tot) {
                        const int j = e / kBKc, kk = e - j * kBKc, k = k0 + kk;
                        float val = v[u];
                        if (kk < kc && j < nc && k >= w && Pend<float>::is(val) &&
                            !wait_ready<float>(x + (size_t)C.rect[k - w] * rhs + c0 + j, val, ctl, A.budget)) {
                            s_ok = 0;
                            val = 0.f;
                        }
                        const __nv_bfloat16 h = __float2bfloat16_rn(val);
                        Vhi[j][kk] = h;
                        Vlo[j][kk] = __float2bfloat16_rn(val - __bfloat162float(h));
                    }
                }
                __syncthreads();
                if (!s_ok) { ok = false; break; }
                if (row0 < w) {
#pragma unroll
                    for (int u = 0; u < kBKc / 16; ++u) {
                        if (u * 16 >= kc) break;
                        const int kb2 = u * 16 + (lane & 3) * 2;
#pragma unroll
                        for (int q = 0; q < kBNc / 8; ++q) {
                            if (q * 8 >= nc) break;
                            const int nn = q * 8 + (lane >> 2);
                            const uint32_t bh0 = *reinterpret_cast<const uint32_t*>(&Vhi[nn][kb2]);
                            const uint32_t bh1 = *reinterpret_cast<const uint32_t*>(&Vhi[nn][kb2 + 8]);
                            const uint32_t bl0 = *reinterpret_cast<const uint32_t*>(&Vlo[nn][kb2]);
                            const uint32_t bl1 = *reinterpret_cast<const uint32_t*>(&Vlo[nn][kb2 + 8]);
                            // BF16x3: the cross terms first, then hi x hi
                            mma_bf16(acc[q], als[u], bh0, bh1);
                            mma_bf16(acc[q], ahs[u], bl0, bl1);
                            mma_bf16(acc[q], ahs[u], bh0, bh1);
                        }
                    }
                }
                __syncthreads();
            }
            if (!ok) break;
            if (row0 < w) {
                const int ra = row0 + (lane >> 2), rb = ra + 8;
#pragma unroll
                for (int q = 0; q < kBNc / 8; ++q) {
                    const int cj = q * 8 + (lane & 3) * 2;
                    if (ra < w && cj < nc) st_relaxed(x + (size_t)(a + ra) * rhs + c0 + cj, Pend<float>::fix(acc[q][0]));
                    if (ra < w && cj + 1 < nc)
                        st_relaxed(x + (size_t)(a + ra) * rhs + c0 + cj + 1, Pend<float>::fix(acc[q][1]));
                    if (rb < w && cj < nc) st_relaxed(x + (size_t)(a + rb) * rhs + c0 + cj, Pend<float>::fix(acc[q][2]));
                    if (rb < w && cj + 1 < nc)
                        st_relaxed(x + (size_t)(a + rb) * rhs + c0 + cj + 1, Pend<float>::fix(acc[q][3]));
                }
            }
        }
        if (__syncthreads_or(!ok)) break;
    }
}

// --- row tasks ---------------------------------------------------------------------------------

// A row task: consecutive rows of one system (about the same number of entries x RHS columns in
// every task, so long-row systems get short tasks).  A warp takes a task and works on `rpw` rows of
// it at a time: lane = slot * (nc * G) + g * nc + c, where nc = min(rhs, 32) RHS columns sit side
// by side, G (BSys::groups) lanes stride over a row's entries, and rpw = 32 / (nc * G) rows run
// side by side.  G follows the system's mean row length, so short rows put many independent rows
// in one warp and long rows use every lane that the column count leaves.
constexpr int kTaskWork = 1 << 16;  // entries x columns per task
constexpr int kTaskRowsMax = 256;

struct RowLanes {
    int nc, G, rpw, slot, g, c;
    bool on;
};

__device__ __forceinline__ RowLanes row_lanes(int rhs, int G) {
    RowLanes L;
    L.nc = min(rhs, 32);
    L.G = rhs > 32 ? 1 : G;
    const int width = L.nc * L.G;
    L.rpw = max(1, 32 / width);
    const int lane = threadIdx.x & 31;
    L.slot = lane / width;
    L.g = (lane % width) / L.nc;
    L.c = lane % L.nc;
    L.on = L.slot < L.rpw;
    return L;
}

// sum over the G entry groups of a row slot, into its g = 0 lanes (a guarded tree: any G)
template <typename T>
__device__ __forceinline__ T slot_sum(T v, const RowLanes& L) {
    for (int off = 1; off < L.G; off <<= 1) {
        const T o = __shfl_down_sync(0xffffffffu, v, off * L.nc);
        if ((L.g & (2 * off - 1)) == 0 && L.g + off < L.G) v += o;
    }
    return v;
}

// --- FP32 Jacobi sweep ------------------------------------------------------------------------

// d_new = (r - N d_old) * invd for the Jacobi systems still sweeping (sweep k reads d[k & 1] and
// writes d[(k + 1) & 1]; sweep 0 starts from d = 0), with per-system max |d_new| and
// max |d_new - d_old| (flushed once per task).  One thread per (row, RHS column) element: the
// lanes of a warp cover 32 consecutive elements of the row-major n x rhs block (coalesced r, d
// accesses; the lanes of one row read the same entries), each thread walks its row's entries
// eight at a time (all eight column/value loads, then all eight gathers, in flight together) and
// fetches the row pointers of its next element before it starts on the current one.
__global__ void __launch_bounds__(256) k_b_jacobi(BArgs A, const int4* __restrict__ tasks, int ntasks) {
    constexpr int kB = 8;
    const int k = *(volatile const int*)&A.bc->sweep_k;
    const float* src = (k & 1) ? A.d1 : A.d0;
    float* dst = (k & 1) ? A.d0 : A.d1;
    const int lane = threadIdx.x & 31;
    const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long t = gw; t < ntasks; t += nw) {
        const int4 T = tasks[t];
        const int s = T.x;
        const BState& St = A.st[s];
        if (St.done || St.inner_done) continue;
        const BSys S = A.sys[s];
        const int m = S.rhs;
        const int* rp = A.rp + S.rp0;
        const int* cl = A.col + S.nz0;
        const float* vl = A.val32 + S.nz0;
        const float* invd = A.invd32 + S.row0;
        const float* rr = A.r32 + S.xb0;
        const float* so = src + S.xb0;
        float* dd = dst + S.xb0;
        const long long e_end = (long long)(T.y + T.z) * m;
        long long e = (long long)T.y * m + lane;
        int i = (int)(e / m);
        int beg = 0, end = 0;
        if (e < e_end) { beg = __ldg(rp + i); end = __ldg(rp + i + 1); }
        float mx = 0.f, ch = 0.f;
        for (; e - lane < e_end; e += 32) {
            const bool on = e < e_end;
            const int c = (int)(e - (long long)i * m);
            // the next element's row pointers, in flight while this one is summed
            const long long en = e + 32;
            const int inext = (int)(en / m);
            int bn = 0, ennd = 0;
            if (en < e_end) { bn = __ldg(rp + inext); ennd = __ldg(rp + inext + 1); }
            float sum = 0.f;
            if (on && k > 0) {
                for (int q0 = beg + 1; q0 < end; q0 += kB) {
                    int jj[kB];
                    float vv[kB], gg[kB];
#pragma unroll
                    for (int u = 0; u < kB; ++u) {
                        const bool in = q0 + u < end;
                        jj[u] = in ? __ldg(cl + q0 + u) : i;
                        vv[u] = in ? __ldg(vl + q0 + u) : 0.f;
                    }
#pragma unroll
                    for (int u = 0; u < kB; ++u) gg[u] = so[(size_t)jj[u] * m + c];
#pragma unroll
                    for (int u = 0; u < kB; ++u) sum = fmaf(vv[u], gg[u], sum);
                }
            }
            if (on) {
                const float dn = (rr[e] - sum) * __ldg(invd + i);
                const float old = k > 0 ? so[e] : 0.f;
                dd[e] = dn;
                mx = fmaxf(mx, fabsf(dn));
                ch = fmaxf(ch, fabsf(dn - old));
            }
            i = inext;
            beg = bn;
            end = ennd;
        }
        const float m1 = warp_max(mx), m2 = warp_max(ch);
        if (lane == 0 && (m1 > 0.f || m2 > 0.f)) {
            atomicMax(&A.st[s].dmax_bits, __float_as_uint(m1));
            atomicMax(&A.st[s].dchg_bits, __float_as_uint(m2));
        }
    }
}

// The same sweep with one thread per ROW holding all of the row's right-hand-side columns in
// registers (M >= rhs, columns c >= rhs predicated off): each lane walks its own row, so a warp has
// 32 rows' column/value loads in flight per round trip instead of 32 / rhs rows' (the element
// layout above shares one row's loads among rhs lanes), and each entry's rhs gathers are contiguous.
// Entries go min(8, 16 / M) at a time (at least one): their column/value loads, then their
// gathers (at most 16 values in flight, which keeps the kernel at 64 registers), then their FMAs
// in entry order.
template <int M>
__device__ __forceinline__ void b_jacobi_rows(const BArgs& A, const int4 T, int k, int c0, const float* src,
                                              float* dst, float& mx, float& ch) {
    constexpr int kB = (16 / M) < 1 ? 1 : ((16 / M) < 8 ? (16 / M) : 8);
    const int s = T.x, lane = threadIdx.x & 31;
    const BSys S = A.sys[s];
    const int m = S.rhs, mc = m - c0;  // this call's columns: c0 .. c0 + min(M, mc)
    const int* rp = A.rp + S.rp0;
    const int* cl = A.col + S.nz0;
    const float* vl = A.val32 + S.nz0;
    const float* invd = A.invd32 + S.row0;
    const float* rr = A.r32 + S.xb0 + c0;
    const float* so = src + S.xb0 + c0;
    float* dd = dst + S.xb0 + c0;
    for (int i0 = T.y; i0 < T.y + T.z; i0 += 32) {
        const int i = i0 + lane;
        if (i >= T.y + T.z) break;
        float acc[M];
#pragma unroll
        for (int c = 0; c < M; ++c) acc[c] = 0.f;
        if (k > 0) {
            const int beg = __ldg(rp + i) + 1, end = __ldg(rp + i + 1);
            for (int q0 = beg; q0 < end; q0 += kB) {
                int jj[kB];
                float vv[kB];
#pragma unroll
                for (int u = 0; u < kB; ++u) {
                    const bool in = q0 + u < end;
                    jj[u] = in ? __ldg(cl + q0 + u) : i;
                    vv[u] = in ? __ldg(vl + q0 + u) : 0.f;
                }
                float g[kB][M];
#pragma unroll
                for (int u = 0; u < kB; ++u)
#pragma unroll
                    for (int c = 0; c < M; ++c) g[u][c] = (c < mc) ? so[(size_t)jj[u] * m + c] : 0.f;
#pragma unroll
                for (int u = 0; u < kB; ++u)
#pragma unroll
                    for (int c = 0; c < M; ++c) acc[c] = fmaf(vv[u], g[u][c], acc[c]);
            }
        }
        const float di = __ldg(invd + i);
#pragma unroll
        for (int c = 0; c < M; ++c) {
            if (c < mc) {
                const size_t e = (size_t)i * m + c;
                const float dn = (rr[e] - acc[c]) * di;
                const float old = k > 0 ? so[e] : 0.f;
                dd[e] = dn;
                mx = fmaxf(mx, fabsf(dn));
                ch = fmaxf(ch, fabsf(dn - old));
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_b_jacobi_rows(BArgs A, const int4* __restrict__ tasks, int ntasks) {
    const int k = *(volatile const int*)&A.bc->sweep_k;
    const float* src = (k & 1) ? A.d1 : A.d0;
    float* dst = (k & 1) ? A.d0 : A.d1;
    const int lane = threadIdx.x & 31;
    const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long t = gw; t < ntasks; t += nw) {
        const int4 T = tasks[t];
        const int s = T.x;
        const BState& St = A.st[s];
        if (St.done || St.inner_done) continue;
        const int m = A.sys[s].rhs;
        float mx = 0.f, ch = 0.f;
        if (m == 1) b_jacobi_rows<1>(A, T, k, 0, src, dst, mx, ch);
        else if (m == 2) b_jacobi_rows<2>(A, T, k, 0, src, dst, mx, ch);
        else if (m <= 4) b_jacobi_rows<4>(A, T, k, 0, src, dst, mx, ch);
        else if (m <= 8) b_jacobi_rows<8>(A, T, k, 0, src, dst, mx, ch);
        else
            for (int c0 = 0; c0 < m; c0 += 16) b_jacobi_rows<16>(A, T, k, c0, src, dst, mx, ch);
        const float m1 = warp_max(mx), m2 = warp_max(ch);
        if (lane == 0 && (m1 > 0.f || m2 > 0.f)) {
            atomicMax(&A.st[s].dmax_bits, __float_as_uint(m1));
            atomicMax(&A.st[s].dchg_bits, __float_as_uint(m2));
        }
    }
}

// --- FP64 residual ----------------------------------------------------------------------------

// r = b - U x in FP64 for the systems still refining; r32 = (float) r; ||r||^2 per system
// (flushed once per task).
__global__ void __launch_bounds__(256) k_b_residual(BArgs A, const int4* __restrict__ tasks, int ntasks) {
    const int lane = threadIdx.x & 31;
    const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long t = gw; t < ntasks; t += nw) {
        const int4 T = tasks[t];
        const int s = T.x;
        if (A.st[s].done) continue;
        const BSys S = A.sys[s];
        const int r = S.rhs;
        const RowLanes L = row_lanes(r, S.groups);
        const int* rp = A.rp + S.rp0;
        const int* cl = A.col + S.nz0;
        const double* vl = A.val + S.nz0;
        const double* xx = A.x + S.xb0;
        const double* bb = A.b + S.xb0;
        double acc = 0.0;
        for (int i0 = T.y; i0 < T.y + T.z; i0 += L.rpw) {
            const int i = i0 + L.slot;
            const bool on = L.on && i < T.y + T.z;
            const int beg = on ? rp[i] : 0, end = on ? rp[i + 1] : 0;
            for (int c0 = 0; c0 < r; c0 += 32) {
                const int cc = c0 + L.c;
                const bool col_on = on && cc < r;
                double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
                if (col_on) {
                    int q = beg + L.g;
                    for (; q + 3 * L.G < end; q += 4 * L.G) {
                        s0 = fma(__ldg(vl + q), xx[(size_t)__ldg(cl + q) * r + cc], s0);
                        s1 = fma(__ldg(vl + q + L.G), xx[(size_t)__ldg(cl + q + L.G) * r + cc], s1);
                        s2 = fma(__ldg(vl + q + 2 * L.G), xx[(size_t)__ldg(cl + q + 2 * L.G) * r + cc], s2);
                        s3 = fma(__ldg(vl + q + 3 * L.G), xx[(size_t)__ldg(cl + q + 3 * L.G) * r + cc], s3);
                    }
                    for (; q < end; q += L.G) s0 = fma(__ldg(vl + q), xx[(size_t)__ldg(cl + q) * r + cc], s0);
                }
                const double sum = slot_sum((s0 + s1) + (s2 + s3), L);
                if (col_on && L.g == 0) {
                    const size_t o = (size_t)i * r + cc;
                    const double rv = bb[o] - sum;
                    A.r32[S.xb0 + o] = (float)rv;
                    acc = fma(rv, rv, acc);
                }
            }
        }
        const double v = warp_sum(acc);
        if (lane == 0 && v != 0.0) atomicAdd(&A.st[s].rnorm2, v);
    }
}

// --- control (one block) ------------------------------------------------------------------------

__device__ __forceinline__ int block_count(int v) {
    __shared__ int s_cnt;
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    const int w = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(&s_cnt, w);
    __syncthreads();
    const int r = s_cnt;
    __syncthreads();
    return r;
}

// Start of the chosen solve: the mixed systems begin refining.
__global__ void k_b_state_init(BArgs A, int count, cudaGraphConditionalHandle outer, bool set_cond) {
    int mine = 0;
    for (int s0 = 0; s0 < count; s0 += blockDim.x) {
        const int s = s0 + threadIdx.x;
        int m = 0;
        if (s < count) {
            BState& T = A.st[s];
            T.done = (A.sys[s].sched == BS_PLAIN || A.sys[s].sched == BS_PANEL64) ? 1 : 0;
            m = !T.done;
        }
        mine += block_count(m);
    }
    if (threadIdx.x == 0) {
        A.bc->active = mine;
        A.bc->nmixed = mine;
        if (set_cond) cudaGraphSetConditional(outer, mine > 0 ? 1u : 0u);
    }
}

// Start of a refinement step: reset the inner solves of the systems still refining.
__global__ void k_b_inner_begin(BArgs A, int count, cudaGraphConditionalHandle inner, bool set_cond) {
    int jac = 0;
    for (int s0 = 0; s0 < count; s0 += blockDim.x) {
        const int s = s0 + threadIdx.x;
        int j = 0;
        if (s < count) {
            BState& T = A.st[s];
            T.final_idx = 0;
            if (!T.done && A.sys[s].sched == BS_JACOBI) {
                T.inner_done = 0;
                T.inner_count = 0;
                T.dmax_bits = T.dchg_bits = 0u;
                j = 1;
            }
        }
        jac += block_count(j);
    }
    if (threadIdx.x == 0) {
        A.bc->jac_active = jac;
        A.bc->sweep_k = 0;
        A.bc->c.ticket = 0u;
        A.bc->c.ticket2 = 0u;
        if (set_cond) cudaGraphSetConditional(inner, jac > 0 && !A.bc->c.status ? 1u : 0u);
    }
}

// After a Jacobi sweep: per-system change test |d_new - d_old| <= eps |d_new| (max norms) or the
// sweep cap; eps = max(10^-inner_tol_exp, 0.1 tol / the system's last relative residual).
__global__ void k_b_jcheck(BArgs A, int count, cudaGraphConditionalHandle inner, bool set_cond) {
    const int k = A.bc->sweep_k;
    int still = 0, swept = 0;
    for (int s0 = 0; s0 < count; s0 += blockDim.x) {
        const int s = s0 + threadIdx.x;
        int st = 0, sw = 0;
        if (s < count) {
            BState& T = A.st[s];
            if (!T.done && A.sys[s].sched == BS_JACOBI && !T.inner_done) {
                sw = 1;
                ++T.inner_count;
                ++T.sweeps;
                const float mx = __uint_as_float(T.dmax_bits), ch = __uint_as_float(T.dchg_bits);
                // a correction (after the first residual) only needs a tenth of what takes this
                // system's residual to the tolerance, never tighter than the FP32 floor
                const float eps = (T.steps > 0 && T.rel > 0.0)
                                      ? fmaxf(A.inner_eps, (float)fmin(1.0, 0.1 * A.tol / T.rel))
                                      : A.inner_eps;
                const bool conv = k > 0 ? ch <= eps * mx : mx == 0.f;
                if (conv || T.inner_count >= A.max_sweeps || !(ch == ch)) {
                    T.inner_done = 1;
                    T.final_idx = (k + 1) & 1;
                } else {
                    st = 1;
                }
                T.dmax_bits = T.dchg_bits = 0u;
            }
        }
        still += block_count(st);
        swept += block_count(sw);
    }
    if (threadIdx.x == 0) {
        A.bc->jac_active = still;
        A.bc->sweep_k = k + 1;
        A.bc->total_sweeps += swept > 0 ? 1 : 0;
        if (set_cond) cudaGraphSetConditional(inner, still > 0 && !A.bc->c.status ? 1u : 0u);
    }
}

// After the residual: per-system convergence; the step loop runs while any system refines.
__global__ void k_b_check(BArgs A, int count, cudaGraphConditionalHandle outer, bool set_cond) {
    int act = 0;
    for (int s0 = 0; s0 < count; s0 += blockDim.x) {
        const int s = s0 + threadIdx.x;
        int a = 0;
        if (s < count) {
            BState& T = A.st[s];
            if (!T.done) {
                ++T.steps;
                const double rel = T.bnorm2 > 0.0 ? sqrt(T.rnorm2 / T.bnorm2) : sqrt(T.rnorm2);
                T.rel = rel;
                T.rnorm2 = 0.0;
                if (rel <= A.tol) {
                    T.done = 1;
                } else if (T.steps >= A.max_refine || !(rel == rel)) {
                    T.done = 2;
                    T.status = SPTRSV_ERR_NOT_CONVERGED;
                } else {
                    a = 1;
                }
            }
        }
        act += block_count(a);
    }
    if (threadIdx.x == 0) {
        A.bc->active = act;
        A.bc->outer += 1;
        if (set_cond) cudaGraphSetConditional(outer, act > 0 && !A.bc->c.status ? 1u : 0u);
    }
}

// --- host side --------------------------------------------------------------------------------

struct HostSeg {
    std::vector<int> sys;
    std::vector<long long> off{0};
    void add(int s, long long cnt) {
        sys.push_back(s);
        off.push_back(off.back() + cnt);
    }
    long long total() const { return off.back(); }
};

struct DevSeg {
    DevBuf sys, off;
    int nseg = 0;
    long long total = 0;
    int upload(const HostSeg& h, cudaStream_t st) {
        nseg = (int)h.sys.size();
        total = h.total();
        if (!nseg) return 0;
        int rc;
        if ((rc = sys.ensure(sizeof(int) * nseg)) || (rc = off.ensure(sizeof(long long) * (nseg + 1)))) return rc;
        CUDA_TRY(cudaMemcpyAsync(sys.p, h.sys.data(), sizeof(int) * nseg, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(off.p, h.off.data(), sizeof(long long) * (nseg + 1), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return 0;
    }
    SegList list() const { return SegList{sys.as<int>(), off.as<long long>(), nseg, total}; }
    void release() { sys.release(); off.release(); nseg = 0; total = 0; }
};

struct Batch {
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaStream_t st2 = nullptr;                // the exact FP64 panels, beside the refinement
    int p64_ctas_per_sm = kP64CtasPerSm;       // tuning override: SPTRSV_P64_CTAS
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int sm_count = 0;
    int count = 0;
    std::vector<BSys> sys;
    std::vector<float> ratio;
    std::vector<int> sched;
    std::vector<int> panel_ok;  // -1 unknown, 0 no, 1 yes
    std::vector<char> have_bf16, have_f64, have_tc;  // have_tc: tensor-core records of the FP64 panels
    bool use_tc = false;  // the FP64 panel items run on the tensor cores (set by build_lists)
    long long tot_rows = 0, tot_nnz = 0, tot_x = 0, tot_rp = 0;
    DevBuf rp, col, val, val32, invd, invd32, dsys, dstate, dctl;
    DevBuf r32, d0, d1, bw, xw;
    // schedule-dependent work lists
    DevBuf order_all, order_plain, order_sf32, items, chunks, tasks_mixed, tasks_jac;
    int n_tasks_mixed = 0, n_tasks_jac = 0;
    DevBuf items64, chunks64, part64, cnt64;  // exact FP64 panels
    unsigned n_items64 = 0;
    long long g_entries64 = 0, g_fma64 = 0;   // G entries (w x K over the chunks) and FMAs per solve
    int n_chunks64 = 0, n_cnt64 = 0;
    unsigned n_order_all = 0, n_order_plain = 0, n_order_sf32 = 0, n_items = 0;
    DevSeg all_rows, all_el, mixed_rows, mixed_el, jac_rows, pend_el, plain_el;
    std::vector<DevBuf> gbufs;            // per panel system: hi, lo, rect
    std::vector<std::vector<BChunk>> pchunks;  // per system (host copies, pointers into gbufs)
    std::vector<int> gidx;                // per system: first of its 3 gbufs, or -1
    bool lists_ready = false;
    // options
    double tol = 1e-12;
    int max_refine = 20, max_sweeps = 200, inner_tol_exp = 6;
    int64_t budget = kDefaultBudgetNs;
    // graphs
    struct G {
        int mode = -1;
        const double* b = nullptr;
        double* x = nullptr;
        cudaGraphExec_t exec = nullptr;
        int64_t fixed = 0;
    };
    std::vector<G> graphs;
    int64_t launches = 0;
    int last_mode = -1;
    int64_t last_fixed = 0;
    Handle* scratch = nullptr;

    ~Batch();
    BArgs args(const double* b, double* x) const;
    int build_lists();
    int build_panels(int s, bool f64);
    bool jacobi_elem = false;  // tuning override (SPTRSV_BJAC=elem): the thread-per-element sweep
    void launch_jacobi(const BArgs& A);
    int build_graph(int mode, const double* b, double* x, cudaGraphExec_t* out, int64_t* fixed);
    int solve(int mode, const double* b, double* x);
    int sync(int64_t* kernels);
    int profile(int mode, const double* b, double* x, float* kind_ms, int* kind_launches, float* kind_first_ms);
    void drop_graphs() {
        for (auto& g : graphs) if (g.exec) cudaGraphExecDestroy(g.exec);
        graphs.clear();
    }
};

Batch::~Batch() {
    if (device >= 0) cudaSetDevice(device);
    drop_graphs();
    DevBuf* bufs[] = {&rp, &col, &val, &val32, &invd, &invd32, &dsys, &dstate, &dctl, &r32, &d0, &d1, &bw, &xw,
                      &order_all, &order_plain, &order_sf32, &items, &chunks, &tasks_mixed, &tasks_jac,
                      &items64, &chunks64, &part64, &cnt64};
    for (DevBuf* b : bufs) b->release();
    DevSeg* segs[] = {&all_rows, &all_el, &mixed_rows, &mixed_el, &jac_rows, &pend_el, &plain_el};
    for (DevSeg* s : segs) s->release();
    for (auto& b : gbufs) b.release();
    if (scratch) sptrsv_destroy(reinterpret_cast<sptrsv_handle>(scratch));
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (st2) cudaStreamDestroy(st2);
    if (st) cudaStreamDestroy(st);
}

BArgs Batch::args(const double* b, double* x) const {
    BArgs A{};
    A.sys = dsys.as<BSys>();
    A.st = dstate.as<BState>();
    A.bc = dctl.as<BCtl>();
    A.rp = rp.as<int>();
    A.col = col.as<int>();
    A.val = val.as<double>();
    A.val32 = val32.as<float>();
    A.invd = invd.as<double>();
    A.invd32 = invd32.as<float>();
    A.b = b;
    A.x = x;
    A.r32 = r32.as<float>();
    A.d0 = d0.as<float>();
    A.d1 = d1.as<float>();
    A.budget = budget;
    A.tol = tol;
    A.inner_eps = powf(10.f, -(float)inner_tol_exp);
    A.max_refine = max_refine;
    A.max_sweeps = max_sweeps;
    return A;
}

// Queue order interleaving the systems from their last rows: position t holds row n_s - 1 - t of
// every listed system with n_s > t (systems by decreasing n, then index).
static std::vector<int2> interleave_rows(const std::vector<BSys>& sys, const std::vector<int>& pick) {
    std::vector<int> ord = pick;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return sys[a].n > sys[b].n; });
    long long tot = 0;
    for (int s : ord) tot += sys[s].n;
    std::vector<int2> out;
    out.reserve(tot);
    const int nmax = ord.empty() ? 0 : sys[ord[0]].n;
    size_t live = ord.size();
    for (int t = 0; t < nmax; ++t) {
        while (live > 0 && sys[ord[live - 1]].n <= t) --live;
        for (size_t k = 0; k < live; ++k) out.push_back(make_int2(ord[k], sys[ord[k]].n - 1 - t));
    }
    return out;
}

template <typename T>
static int upload_vec(DevBuf& d, const std::vector<T>& h, cudaStream_t st) {
    if (h.empty()) return 0;
    int rc = d.ensure(sizeof(T) * h.size());
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(d.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return 0;
}

// Dense panels of system s: uniform 64-row chunks (each one a skyline or exact supernode chunk),
// G = [T^-1 | -T^-1 Rect] formed in FP64 by the single-system supernodal analysis and kept as
// its BF16 hi/lo split.
int Batch::build_panels(int s, bool f64) {
    if (panel_ok[s] == 0) return SPTRSV_ERR_SUPERNODES;
    if (panel_ok[s] == 1 && (f64 ? have_f64[s] : have_bf16[s])) return 0;
    int rc;
    if (!scratch) {
        sptrsv_handle h = nullptr;
        if ((rc = sptrsv_create(&h, device))) return rc;
        scratch = reinterpret_cast<Handle*>(h);
    }
    Handle& H = *scratch;
    H.build_tc = false;  // the batch builds its own tensor-core records per chunk below
    const BSys& S = sys[s];
    H.drop_matrix();
    H.n = S.n;
    H.nnz = (int)(s + 1 < count ? sys[s + 1].nz0 - S.nz0 : tot_nnz - S.nz0);
    H.rp = rp.as<int>() + S.rp0;
    H.col = col.as<int>() + S.nz0;
    H.val = val.as<double>() + S.nz0;
    if ((rc = H.analyse())) return rc;
    std::vector<int> sn;
    for (int a = 0; a < S.n; a += kBPanel) sn.push_back(a);
    sn.push_back(S.n);
    rc = H.set_supernodes((int)sn.size() - 1, sn.data());
    if (rc == SPTRSV_ERR_SUPERNODES) {
        panel_ok[s] = 0;
        return rc;
    }
    if (rc) return rc;
    const int C = H.sn_count;
    std::vector<int> ss(C + 1), mm(C), roff(C + 1), ld(C);
    std::vector<long long> goff(C + 1);
    CUDA_TRY(cudaMemcpy(ss.data(), H.sn_start.p, sizeof(int) * (C + 1), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(mm.data(), H.sn_m.p, sizeof(int) * C, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(roff.data(), H.sn_roff.p, sizeof(int) * (C + 1), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(ld.data(), H.sn_ld.p, sizeof(int) * C, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(goff.data(), H.sn_goff.p, sizeof(long long) * (C + 1), cudaMemcpyDeviceToHost));
    const long long gtot = goff[C];
    // buffers of this system: [bf16 hi, bf16 lo] and/or [f64], then the rectangle columns
    const int k0 = (int)gbufs.size();
    gbufs.resize(k0 + 7);  // + [4] tensor-core records, [5] double-FP32 G, [6] its row exponents
    if ((rc = gbufs[k0 + 3].ensure(sizeof(int) * ((size_t)roff[C] + 1)))) return rc;
    if (!f64) {
        if ((rc = gbufs[k0].ensure(2 * (size_t)gtot)) || (rc = gbufs[k0 + 1].ensure(2 * (size_t)gtot))) return rc;
        CUDA_TRY(cudaMemcpyAsync(gbufs[k0].p, H.sn_Ghi.p, 2 * (size_t)gtot, cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(gbufs[k0 + 1].p, H.sn_Glo.p, 2 * (size_t)gtot, cudaMemcpyDeviceToDevice, st));
    } else {
        if ((rc = gbufs[k0 + 2].ensure(sizeof(double) * (size_t)gtot))) return rc;
        CUDA_TRY(cudaMemcpyAsync(gbufs[k0 + 2].p, H.sn_G.p, sizeof(double) * (size_t)gtot, cudaMemcpyDeviceToDevice, st));
    }
    if (roff[C] > 0)
        CUDA_TRY(cudaMemcpyAsync(gbufs[k0 + 3].p, H.sn_rect.p, sizeof(int) * roff[C], cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    // keep the other precision's pointers of an earlier build
    std::vector<BChunk> old = pchunks[s];
    pchunks[s].clear();
    for (int c = 0; c < C; ++c) {
        BChunk ch{};
        ch.sys = s;
        ch.a = ss[c];
        ch.w = ss[c + 1] - ss[c];
        ch.m = mm[c];
        ch.ld = ld[c];
        ch.nblk = p64_nblk(ch.w, ch.w + ch.m);
        ch.r0 = 0;
        ch.pw = ch.w;
        if (!f64) {
            ch.ghi = gbufs[k0].as<__nv_bfloat16>() + goff[c];
            ch.glo = gbufs[k0 + 1].as<__nv_bfloat16>() + goff[c];
            if ((int)old.size() == C) {
                ch.g64 = old[c].g64;
                ch.gtc = old[c].gtc;
                ch.ghl = old[c].ghl;
                ch.gexp = old[c].gexp;
            }
        } else {
            ch.g64 = gbufs[k0 + 2].as<double>() + goff[c];
            if ((int)old.size() == C) {
                ch.ghi = old[c].ghi;
                ch.glo = old[c].glo;
            }
        }
        ch.rect = gbufs[k0 + 3].as<int>() + roff[c];
        pchunks[s].push_back(ch);
    }
    have_tc[s] = 0;
    if (f64 && panels_mode() == 1) {
        // the tensor-core schedule's digit-slice G records of every chunk (one 64-row panel each)
        std::vector<size_t> toff(C + 1, 0);
        std::vector<int2> recs;
        for (int c = 0; c < C; ++c) {
            const BChunk& b = pchunks[s][c];
            toff[c + 1] = toff[c] + ((tc_panel_bytes(b.w, b.w + b.m) + 127) & ~(size_t)127);
            for (int q = 0; q < b.nblk; ++q) recs.push_back(make_int2(c, q));
        }
        if ((rc = gbufs[k0 + 4].ensure(std::max<size_t>(toff[C], 128)))) return rc;
        for (int c = 0; c < C; ++c) pchunks[s][c].gtc = gbufs[k0 + 4].as<unsigned char>() + toff[c];
        DevBuf tch, trec;
        if ((rc = tch.ensure(sizeof(BChunk) * C)) || (rc = trec.ensure(sizeof(int2) * std::max<size_t>(1, recs.size()))))
            return rc;
        CUDA_TRY(cudaMemcpyAsync(tch.p, pchunks[s].data(), sizeof(BChunk) * C, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(trec.p, recs.data(), sizeof(int2) * recs.size(), cudaMemcpyHostToDevice, st));
        int64_t lsplit = 0;
        rc = launch_tc_split(tch.as<BChunk>(), trec.as<int2>(), (int)recs.size(), sm_count, st, &lsplit);
        if (!rc) CUDA_TRY(cudaStreamSynchronize(st));
        tch.release();
        trec.release();
        if (rc) return rc;
        have_tc[s] = 1;
    }
    if (f64 && panels_mode() == 2) {
        // the double-FP32 schedule: G as scaled FP32 pairs (laid out like g64) and the row exponents,
        // indexed by the system's row
        if ((rc = gbufs[k0 + 5].ensure(sizeof(float2) * (size_t)std::max(1LL, gtot))) ||
            (rc = gbufs[k0 + 6].ensure(sizeof(int) * (size_t)std::max(1, S.n))))
            return rc;
        for (int c = 0; c < C; ++c) {
            pchunks[s][c].ghl = gbufs[k0 + 5].as<float2>() + goff[c];
            pchunks[s][c].gexp = gbufs[k0 + 6].as<int>() + ss[c];
        }
        DevBuf tch;
        if ((rc = tch.ensure(sizeof(BChunk) * C))) return rc;
        CUDA_TRY(cudaMemcpyAsync(tch.p, pchunks[s].data(), sizeof(BChunk) * C, cudaMemcpyHostToDevice, st));
        int64_t lconv = 0;
        rc = launch_g_df(tch.as<BChunk>(), C, st, &lconv);
        if (!rc) CUDA_TRY(cudaStreamSynchronize(st));
        tch.release();
        if (rc) return rc;
    }
    H.drop_matrix();
    panel_ok[s] = 1;
    (f64 ? have_f64 : have_bf16)[s] = 1;
    return 0;
}

int Batch::build_lists() {
    if (lists_ready) return 0;
    int rc;
    for (int s = 0; s < count; ++s)
        if ((sched[s] == BS_PANEL || sched[s] == BS_PANEL64) && (rc = build_panels(s, sched[s] == BS_PANEL64)))
            return rc;
    std::vector<int> plain, sf32;
    HostSeg mr, me, jr, pe, pl;
    for (int s = 0; s < count; ++s) {
        const long long n = sys[s].n, ne = n * sys[s].rhs;
        sys[s].sched = sched[s];
        if (sched[s] == BS_PLAIN || sched[s] == BS_PANEL64) {
            if (sched[s] == BS_PLAIN) plain.push_back(s);
            pl.add(s, ne);
            continue;
        }
        mr.add(s, n);
        me.add(s, ne);
        if (sched[s] == BS_JACOBI) jr.add(s, n);
        if (sched[s] == BS_PANEL || sched[s] == BS_SF32) pe.add(s, ne);
        if (sched[s] == BS_SF32) sf32.push_back(s);
    }
    // row tasks of the mixed systems and of the Jacobi ones
    std::vector<int4> tm, tj;
    for (int s = 0; s < count; ++s) {
        if (sched[s] == BS_PLAIN || sched[s] == BS_PANEL64) continue;
        const long long nnz_s = (s + 1 < count ? sys[s + 1].nz0 : tot_nnz) - sys[s].nz0;
        const int nc = std::min(sys[s].rhs, 32);
        const int rpw = std::max(1, 32 / (nc * sys[s].groups));
        const double per_row = std::max(1.0, (double)nnz_s / sys[s].n) * nc;
        int rows = (int)std::min<double>(kTaskRowsMax, std::max<double>(rpw, kTaskWork / per_row));
        rows = std::max(rpw, rows / rpw * rpw);
        for (int r0 = 0; r0 < sys[s].n; r0 += rows) tm.push_back(make_int4(s, r0, std::min(rows, sys[s].n - r0), 0));
        if (sched[s] == BS_JACOBI) {
            // about 1,024 (row, column) elements per task, whole warps of rows
            const int jrows = std::max(32, (1024 / sys[s].rhs + 31) / 32 * 32);
            for (int r0 = 0; r0 < sys[s].n; r0 += jrows)
                tj.push_back(make_int4(s, r0, std::min(jrows, sys[s].n - r0), 0));
        }
    }
    n_tasks_mixed = (int)tm.size();
    n_tasks_jac = (int)tj.size();
    if ((rc = upload_vec(tasks_mixed, tm, st)) || (rc = upload_vec(tasks_jac, tj, st))) return rc;
    if ((rc = upload_vec(dsys, sys, st))) return rc;
    if ((rc = mixed_rows.upload(mr, st)) || (rc = mixed_el.upload(me, st)) || (rc = jac_rows.upload(jr, st)) ||
        (rc = pend_el.upload(pe, st)) || (rc = plain_el.upload(pl, st)))
        return rc;
    std::vector<int2> op = interleave_rows(sys, plain), os = interleave_rows(sys, sf32);
    n_order_plain = (unsigned)op.size();
    n_order_sf32 = (unsigned)os.size();
    if ((rc = upload_vec(order_plain, op, st)) || (rc = upload_vec(order_sf32, os, st))) return rc;
    // panel work items: per system its chunks' panels from the last, interleaved across systems
    std::vector<BChunk> ch;
    std::vector<std::vector<int2>> per;
    for (int s = 0; s < count; ++s) {
        if (sched[s] != BS_PANEL) continue;
        const int base = (int)ch.size();
        std::vector<int2> its;
        for (int c = (int)pchunks[s].size() - 1; c >= 0; --c)
            for (int p = (pchunks[s][c].w + kBPanel - 1) / kBPanel - 1; p >= 0; --p) its.push_back(make_int2(base + c, p));
        for (const BChunk& b : pchunks[s]) ch.push_back(b);
        per.push_back(std::move(its));
    }
    std::vector<int2> it;
    size_t longest = 0;
    for (auto& v : per) longest = std::max(longest, v.size());
    for (size_t t = 0; t < longest; ++t)
        for (auto& v : per)
            if (t < v.size()) it.push_back(v[t]);
    n_items = (unsigned)it.size();
    if ((rc = upload_vec(chunks, ch, st)) || (rc = upload_vec(items, it, st))) return rc;
    // exact FP64 panel items: per chunk (last first) its own right-hand-side blocks, then the solved
    // column blocks farthest first, each block once per RHS group; chunks interleaved across
    // systems; partial-sum slots per chunk, completion counters per (chunk, group)
    std::vector<BChunk> ch64;
    std::vector<std::vector<std::vector<int2>>> per64;  // per system, per step (chunk from the last)
    // the tensor cores take the FP64 panels when every panel system has its records
    use_tc = panels_mode() == 1;
    for (int s = 0; s < count; ++s)
        if (sched[s] == BS_PANEL64 && !have_tc[s]) use_tc = false;
    long long poff = 0;
    int cbase = 0;
    g_entries64 = g_fma64 = 0;
    for (int s = 0; s < count; ++s) {
        if (sched[s] != BS_PANEL64) continue;
        const int base = (int)ch64.size(), ng = use_tc ? tc_groups_host(sys[s].rhs) : p64_groups(sys[s].rhs);
        if (ng > 0x7FFF) return SPTRSV_ERR_TOO_LARGE;  // items carry the group in 15 bits
        for (const BChunk& b : pchunks[s])
            if (b.nblk > 0xFFFF) return SPTRSV_ERR_TOO_LARGE;  // and the block in 16
        std::vector<std::vector<int2>> steps;
        for (int c = (int)pchunks[s].size() - 1; c >= 0; --c) {
            const BChunk& b = pchunks[s][c];
            std::vector<int2> its;
            for (int q = 0; q < b.nblk; ++q)
                for (int g = 0; g < ng; ++g) its.push_back(make_int2(base + c, (q == 0 ? 0 : b.nblk - q) | g << 16));
            steps.push_back(std::move(its));
        }
        for (BChunk b : pchunks[s]) {
            if (panels_mode() != 2) b.ghl = nullptr;  // double-FP32 products only in that mode
            b.poff = poff;
            b.cbase = cbase;
            cbase += ng;
            poff += (long long)b.nblk * b.w * sys[s].rhs;
            g_entries64 += (long long)b.w * (b.w + b.m);
            g_fma64 += (long long)b.w * (b.w + b.m) * sys[s].rhs;
            ch64.push_back(b);
        }
        per64.push_back(std::move(steps));
    }
    // queue order: step by step across the systems (every system's last chunk, then every
    // system's second-last, ...), so a system's chunk enters the queue when its dependency chain
    // can reach it, whatever its blocks per chunk; the longest chains then run at their own pace
    std::vector<int2> it64;
    size_t longest64 = 0;
    for (auto& v : per64) longest64 = std::max(longest64, v.size());
    for (size_t t = 0; t < longest64; ++t)
        for (auto& v : per64)
            if (t < v.size()) it64.insert(it64.end(), v[t].begin(), v[t].end());
    n_items64 = (unsigned)it64.size();
    n_chunks64 = (int)ch64.size();
    n_cnt64 = cbase;
    if ((rc = upload_vec(chunks64, ch64, st)) || (rc = upload_vec(items64, it64, st))) return rc;
    if (n_chunks64 && ((rc = part64.ensure(sizeof(double) * (size_t)std::max(1LL, poff))) ||
                       (rc = cnt64.ensure(sizeof(int) * (size_t)n_cnt64))))
        return rc;
    lists_ready = true;
    drop_graphs();
    return 0;
}

static int resident(const void* kernel, int threads, int sm_count, long long want) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess) per_sm = 1;
    const long long g = (long long)std::max(1, per_sm) * sm_count;
    return (int)std::max(1LL, std::min(g, want));
}

static int elem_grid(int sm_count, long long total) {
    return (int)std::max(1LL, std::min((long long)sm_count * 16, (total + 255) / 256));
}

static int task_grid(int sm_count, long long tasks) {
    return (int)std::max(1LL, std::min((long long)sm_count * 8, (tasks + 7) / 8));
}

void Batch::launch_jacobi(const BArgs& A) {
    if (jacobi_elem)
        k_b_jacobi<<<task_grid(sm_count, n_tasks_jac), 256, 0, st>>>(A, tasks_jac.as<int4>(), n_tasks_jac);
    else
        k_b_jacobi_rows<<<task_grid(sm_count, n_tasks_jac), 256, 0, st>>>(A, tasks_jac.as<int4>(), n_tasks_jac);
}

static int row_grid(int sm_count, long long rows) {
    const long long tasks = (rows + kBRowChunk - 1) / kBRowChunk;
    return (int)std::max(1LL, std::min((long long)sm_count * 8, (tasks + 7) / 8));
}

int Batch::build_graph(int mode, const double* b, double* x, cudaGraphExec_t* out, int64_t* fixed) {
    *out = nullptr;
    int rc = mode == 1 ? build_lists() : 0;
    if (rc) return rc;
    const BArgs A = args(b, x);
    int64_t nk = 0;
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle ho = 0, hi = 0;
    cudaError_t e = cudaSuccess;
    // a conditional handle exists only with the WHILE node that reads it
    if (mode == 1 && mixed_el.nseg) {
        e = cudaGraphConditionalHandleCreate(&ho, g, 1, cudaGraphCondAssignDefault);
        if (e == cudaSuccess && jac_rows.nseg) e = cudaGraphConditionalHandleCreate(&hi, g, 0, cudaGraphCondAssignDefault);
    }
    if (e != cudaSuccess) { cudaGraphDestroy(g); return set_cuda_error(e, "batch conditional handle"); }
    auto add_while = [&](cudaGraph_t parent, cudaGraphConditionalHandle h, cudaGraph_t* body) -> cudaError_t {
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        cudaError_t er = cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd);
        if (er != cudaSuccess) return er;
        alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)];
        memset(raw, 0, sizeof(raw));
        cudaGraphNodeParams* p = reinterpret_cast<cudaGraphNodeParams*>(raw);
        p->type = cudaGraphNodeTypeConditional;
        p->conditional.handle = h;
        p->conditional.type = cudaGraphCondTypeWhile;
        p->conditional.size = 1;
        cudaGraphNode_t node;
        er = cudaGraphAddNode(&node, parent, deps, nullptr, nd, p);
        if (er != cudaSuccess) return er;
        *body = p->conditional.phGraph_out[0];
        return cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    };
    auto launch_pull64 = [&](const DevBuf& order, unsigned n) {
        const int grid = resident((const void*)k_b_pull<double>, 256, sm_count, ((long long)n + 7) / 8);
        k_b_pull<double><<<grid, 256, 0, st>>>(A, order.as<int2>(), n, b, x, A.val, A.invd, 0, false);
        ++nk;
    };
    cudaGraph_t obody = nullptr, ibody = nullptr;
    e = cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return set_cuda_error(e, "batch capture"); }
    cudaMemsetAsync(A.bc, 0, sizeof(BCtl), st);
    cudaMemsetAsync(A.st, 0, sizeof(BState) * count, st);
    if (mode == 0) {
        // plain: every system by the FP64 pull, one persistent launch
        k_b_fill_pending<double><<<elem_grid(sm_count, all_el.total), 256, 0, st>>>(A, all_el.list(), x, false);
        ++nk;
        launch_pull64(order_all, n_order_all);
    } else {
        k_b_state_init<<<1, 512, 0, st>>>(A, count, ho, mixed_el.nseg > 0);
        ++nk;
        if (plain_el.nseg) {
            k_b_fill_pending<double><<<elem_grid(sm_count, plain_el.total), 256, 0, st>>>(A, plain_el.list(), x, false);
            ++nk;
        }
        if (n_items64) {
            // the exact FP64 panels on a second captured stream, beside everything below (their
            // CTAs take a fraction of the SMs; the refinement's kernels fill the rest)
            cudaEventRecord(ev_fork, st);
            cudaStreamWaitEvent(st2, ev_fork, 0);
            int64_t l64 = 0;
            if (use_tc
                    ? launch_panels_tc(A.sys, 0, A.b, A.x, &A.bc->c, &A.bc->ticket_p64, A.budget, items64.as<int2>(),
                                       n_items64, chunks64.as<BChunk>(), part64.as<double>(), cnt64.as<int>(),
                                       n_cnt64, sm_count, st2, &l64)
                    : launch_panels64(A.sys, 0, A.b, A.x, &A.bc->c, &A.bc->ticket_p64, A.budget, items64.as<int2>(),
                                      n_items64, chunks64.as<BChunk>(), part64.as<double>(), cnt64.as<int>(), n_cnt64,
                                      p64_ctas_per_sm, sm_count, st2, &l64))
                rc = SPTRSV_ERR_CUDA;
            cudaEventRecord(ev_join, st2);
            nk += (int)l64;
        }
        if (n_order_plain) launch_pull64(order_plain, n_order_plain);
        if (mixed_el.nseg) {
            k_b_init_mixed<<<elem_grid(sm_count, mixed_el.total), 256, 0, st>>>(A, mixed_el.list());
            ++nk;
            if (add_while(g, ho, &obody) != cudaSuccess) rc = SPTRSV_ERR_CUDA;
        }
    }
    if (mode == 1 && n_items64) cudaStreamWaitEvent(st, ev_join, 0);
    cudaGraph_t g2 = nullptr;
    e = cudaStreamEndCapture(st, &g2);
    if (!rc && e != cudaSuccess) rc = set_cuda_error(e, "batch capture end");
    *fixed = nk;
    int64_t per_outer = 0;
    if (!rc && obody) {
        e = cudaStreamBeginCaptureToGraph(st, obody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            int64_t k0 = nk;
            k_b_inner_begin<<<1, 512, 0, st>>>(A, count, hi, jac_rows.nseg > 0);
            ++nk;
            if (pend_el.nseg) {
                k_b_fill_pending<float><<<elem_grid(sm_count, pend_el.total), 256, 0, st>>>(A, pend_el.list(), A.d0, true);
                ++nk;
            }
            if (n_items) {
                const int grid = resident((const void*)k_b_panels, 128, sm_count, n_items);
                k_b_panels<<<grid, 128, 0, st>>>(A, items.as<int2>(), n_items, chunks.as<BChunk>());
                ++nk;
            }
            if (n_order_sf32) {
                const int grid = resident((const void*)k_b_pull<float>, 256, sm_count, ((long long)n_order_sf32 + 7) / 8);
                k_b_pull<float><<<grid, 256, 0, st>>>(A, order_sf32.as<int2>(), n_order_sf32, A.r32, A.d0, A.val32,
                                                      A.invd32, 1, true);
                ++nk;
            }
            if (jac_rows.nseg && add_while(obody, hi, &ibody) != cudaSuccess) rc = SPTRSV_ERR_CUDA;
            k_b_axpy<<<elem_grid(sm_count, mixed_el.total), 256, 0, st>>>(A, mixed_el.list());
            k_b_residual<<<task_grid(sm_count, n_tasks_mixed), 256, 0, st>>>(A, tasks_mixed.as<int4>(), n_tasks_mixed);
            k_b_check<<<1, 512, 0, st>>>(A, count, ho, true);
            nk += 3;
            per_outer = nk - k0;
            e = cudaStreamEndCapture(st, &g2);
            if (!rc && e != cudaSuccess) rc = set_cuda_error(e, "batch capture outer");
        } else {
            rc = set_cuda_error(e, "batch capture outer begin");
        }
    }
    if (!rc && ibody) {
        e = cudaStreamBeginCaptureToGraph(st, ibody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            launch_jacobi(A);
            k_b_jcheck<<<1, 512, 0, st>>>(A, count, hi, true);
            e = cudaStreamEndCapture(st, &g2);
            if (!rc && e != cudaSuccess) rc = set_cuda_error(e, "batch capture inner");
        } else {
            rc = set_cuda_error(e, "batch capture inner begin");
        }
    }
    if (!rc) {
        e = cudaGraphInstantiate(out, g, 0);
        if (e != cudaSuccess) rc = set_cuda_error(e, "batch instantiate");
    }
    cudaGraphDestroy(g);
    (void)cudaGetLastError();
    // launches per refinement step in the upper 32 bits, fixed ones in the lower
    *fixed = (per_outer << 32) | *fixed;
    return rc;
}

int Batch::solve(int mode, const double* b, double* x) {
    if (mode != 0 && mode != 1) return SPTRSV_ERR_INVALID_ARG;
    if (!b || !x) return SPTRSV_ERR_INVALID_ARG;
    int rc = mode == 1 ? build_lists() : 0;
    if (rc) return rc;
    G* hit = nullptr;
    for (auto& gg : graphs)
        if (gg.mode == mode && gg.b == b && gg.x == x) { hit = &gg; break; }
    if (!hit) {
        if (graphs.size() >= 8) drop_graphs();
        G gg;
        gg.mode = mode;
        gg.b = b;
        gg.x = x;
        if ((rc = build_graph(mode, b, x, &gg.exec, &gg.fixed))) return rc;
        graphs.push_back(gg);
        hit = &graphs.back();
    }
    CUDA_TRY(cudaGraphLaunch(hit->exec, st));
    last_mode = mode;
    last_fixed = hit->fixed;
    return 0;
}

// The same solve as the graph, driven from the host with CUDA events around every kernel (the
// loop decisions are read back from the device after each check): per-kernel-kind device time.
// Kinds: 0 fill x, 1 FP64 pull, 2 state init, 3 mixed init, 4 step begin, 5 fill d, 6 panels,
// 7 FP32 pull, 8 Jacobi sweep, 9 sweep check, 10 axpy, 11 residual, 12 step check, 13 FP64 panels.
int Batch::profile(int mode, const double* b, double* x, float* kind_ms, int* kind_launches, float* kind_first_ms) {
    if ((mode != 0 && mode != 1) || !b || !x) return SPTRSV_ERR_INVALID_ARG;
    int rc = mode == 1 ? build_lists() : 0;
    if (rc) return rc;
    int seen[kBatchKinds] = {0};
    for (int k = 0; k < kBatchKinds; ++k) {
        if (kind_ms) kind_ms[k] = 0.f;
        if (kind_launches) kind_launches[k] = 0;
        if (kind_first_ms) kind_first_ms[k] = 0.f;
    }
    const BArgs A = args(b, x);
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    int64_t nk = 0;
    auto timed = [&](int kind, auto launch) -> int {
        CUDA_TRY(cudaEventRecord(e0, st));
        launch();
        CUDA_TRY(cudaEventRecord(e1, st));
        CUDA_TRY(cudaEventSynchronize(e1));
        CUDA_TRY(cudaGetLastError());
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (kind_ms) kind_ms[kind] += ms;
        if (kind_launches) ++kind_launches[kind];
        if (kind_first_ms && !seen[kind]++) kind_first_ms[kind] = ms;
        ++nk;
        return 0;
    };
    auto read_ctl = [&](BCtl* c) -> int {
        CUDA_TRY(cudaMemcpyAsync(c, dctl.p, sizeof(BCtl), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return 0;
    };
    cudaGraphConditionalHandle none = 0;
    CUDA_TRY(cudaMemsetAsync(A.bc, 0, sizeof(BCtl), st));
    CUDA_TRY(cudaMemsetAsync(A.st, 0, sizeof(BState) * count, st));
    auto pull64 = [&](const DevBuf& order, unsigned n) {
        const int grid = resident((const void*)k_b_pull<double>, 256, sm_count, ((long long)n + 7) / 8);
        return timed(1, [&] { k_b_pull<double><<<grid, 256, 0, st>>>(A, order.as<int2>(), n, b, x, A.val, A.invd, 0, false); });
    };
    if (mode == 0) {
        if ((rc = timed(0, [&] { k_b_fill_pending<double><<<elem_grid(sm_count, all_el.total), 256, 0, st>>>(A, all_el.list(), x, false); })) ||
            (rc = pull64(order_all, n_order_all)))
            goto out;
    } else {
        if ((rc = timed(2, [&] { k_b_state_init<<<1, 512, 0, st>>>(A, count, none, false); }))) goto out;
        if (plain_el.nseg &&
            (rc = timed(0, [&] { k_b_fill_pending<double><<<elem_grid(sm_count, plain_el.total), 256, 0, st>>>(A, plain_el.list(), x, false); })))
            goto out;
        if (n_order_plain && (rc = pull64(order_plain, n_order_plain))) goto out;
        if (n_items64) {
            int64_t l64 = 0;
            if ((rc = timed(13, [&] {
                     if (use_tc)
                         launch_panels_tc(A.sys, 0, A.b, A.x, &A.bc->c, &A.bc->ticket_p64, A.budget, items64.as<int2>(),
                                          n_items64, chunks64.as<BChunk>(), part64.as<double>(), cnt64.as<int>(),
                                          n_cnt64, sm_count, st, &l64);
                     else
                         launch_panels64(A.sys, 0, A.b, A.x, &A.bc->c, &A.bc->ticket_p64, A.budget, items64.as<int2>(),
                                         n_items64, chunks64.as<BChunk>(), part64.as<double>(), cnt64.as<int>(),
                                         n_cnt64, 64, sm_count, st, &l64);
                 })))
                goto out;
        }
        if (mixed_el.nseg) {
            if ((rc = timed(3, [&] { k_b_init_mixed<<<elem_grid(sm_count, mixed_el.total), 256, 0, st>>>(A, mixed_el.list()); })))
                goto out;
            BCtl c{};
            for (int step = 0; step < 1000; ++step) {
                if ((rc = timed(4, [&] { k_b_inner_begin<<<1, 512, 0, st>>>(A, count, none, false); }))) goto out;
                if (pend_el.nseg &&
                    (rc = timed(5, [&] { k_b_fill_pending<float><<<elem_grid(sm_count, pend_el.total), 256, 0, st>>>(A, pend_el.list(), A.d0, true); })))
                    goto out;
                if (n_items) {
                    const int grid = resident((const void*)k_b_panels, 128, sm_count, n_items);
                    if ((rc = timed(6, [&] { k_b_panels<<<grid, 128, 0, st>>>(A, items.as<int2>(), n_items, chunks.as<BChunk>()); })))
                        goto out;
                }
                if (n_order_sf32) {
                    const int grid = resident((const void*)k_b_pull<float>, 256, sm_count, ((long long)n_order_sf32 + 7) / 8);
                    if ((rc = timed(7, [&] {
                             k_b_pull<float><<<grid, 256, 0, st>>>(A, order_sf32.as<int2>(), n_order_sf32, A.r32, A.d0,
                                                                   A.val32, A.invd32, 1, true);
                         })))
                        goto out;
                }
                if (jac_rows.nseg) {
                    if ((rc = read_ctl(&c))) goto out;
                    for (int sw = 0; sw < 100000 && c.jac_active > 0 && !c.c.status; ++sw) {
                        if ((rc = timed(8, [&] { launch_jacobi(A); })) ||
                            (rc = timed(9, [&] { k_b_jcheck<<<1, 512, 0, st>>>(A, count, none, false); })) ||
                            (rc = read_ctl(&c)))
                            goto out;
                    }
                }
                if ((rc = timed(10, [&] { k_b_axpy<<<elem_grid(sm_count, mixed_el.total), 256, 0, st>>>(A, mixed_el.list()); })) ||
                    (rc = timed(11, [&] { k_b_residual<<<task_grid(sm_count, n_tasks_mixed), 256, 0, st>>>(A, tasks_mixed.as<int4>(), n_tasks_mixed); })) ||
                    (rc = timed(12, [&] { k_b_check<<<1, 512, 0, st>>>(A, count, none, false); })) || (rc = read_ctl(&c)))
                    goto out;
                if (c.active == 0 || c.c.status) break;
            }
        }
    }
out:
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    launches += nk;
    BCtl c{};
    CUDA_TRY(cudaMemcpy(&c, dctl.p, sizeof(c), cudaMemcpyDeviceToHost));
    return c.c.status;
}

int Batch::sync(int64_t* kernels) {
    CUDA_TRY(cudaStreamSynchronize(st));
    BCtl c{};
    CUDA_TRY(cudaMemcpy(&c, dctl.p, sizeof(c), cudaMemcpyDeviceToHost));
    const int64_t fixed = last_fixed & 0xffffffffLL, per_outer = last_fixed >> 32;
    const int64_t k = fixed + per_outer * c.outer + 2 * (int64_t)c.total_sweeps;
    launches += k;
    if (kernels) *kernels = k;
    if (c.c.status) return c.c.status;
    if (last_mode == 1) {
        std::vector<BState> h(count);
        CUDA_TRY(cudaMemcpy(h.data(), dstate.p, sizeof(BState) * count, cudaMemcpyDeviceToHost));
        for (const BState& t : h)
            if (t.status) return t.status;
    }
    return 0;
}

// Default schedule from the analysis: dense row ranges (banded / skyline) -> exact FP64 panels
// (measured faster in the batch than the BF16x3 panels' refinement); rows dominated by their
// diagonal -> Jacobi; otherwise the FP32 sync-free pull.
static int default_schedule(const BSys& S, long long nnz, float ratio, int gapped) {
    if (!gapped && nnz >= 8LL * S.n) return BS_PANEL64;
    if (ratio < 1.f) return BS_JACOBI;
    return BS_SF32;
}

}  // namespace sptrsv

using sptrsv::Batch;

extern "C" {

int sptrsv_batch_create(sptrsv_batch* out, int device, int count, const int* n, const int* rhs,
                        const int64_t* row_ptr, const int* col, const double* val) {
    using namespace sptrsv;
    if (!out) return SPTRSV_ERR_INVALID_ARG;
    *out = nullptr;
    if (count < 1 || !n || !rhs || !row_ptr || !col || !val) return SPTRSV_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        (void)cudaGetLastError();
        return SPTRSV_ERR_NO_DEVICE;
    }
    if (device < 0) CUDA_TRY(cudaGetDevice(&device));
    if (device >= ndev) return SPTRSV_ERR_INVALID_ARG;
    // host-side layout and row-pointer checks
    std::vector<BSys> sys(count);
    std::vector<long long> nnz(count);
    long long rp0 = 0, nz0 = 0, row0 = 0, xb0 = 0;
    for (int s = 0; s < count; ++s) {
        if (n[s] < 1 || rhs[s] < 1) return SPTRSV_ERR_INVALID_ARG;
        const int64_t* r = row_ptr + rp0;
        if (r[0] != 0) return SPTRSV_ERR_ROW_PTR;
        for (int i = 0; i < n[s]; ++i)
            if (r[i + 1] < r[i]) return SPTRSV_ERR_ROW_PTR;
        if (r[n[s]] > 0x7fffffffLL) return SPTRSV_ERR_TOO_LARGE;
        if ((long long)n[s] * rhs[s] > 0x7fffffffLL) return SPTRSV_ERR_TOO_LARGE;
        nnz[s] = r[n[s]];
        // lanes per row: about eight entries per lane, within the 32 / nc lanes (short rows:
        // several rows side by side in a warp)
        const int nc = std::min(rhs[s], 32);
        const double mean = (double)nnz[s] / n[s];
        const int G = (int)std::max(1.0, std::min((double)(32 / nc), std::ceil(mean / 8.0)));
        sys[s] = BSys{n[s], rhs[s], BS_PLAIN, G, rp0, nz0, row0, xb0};
        rp0 += n[s] + 1;
        nz0 += nnz[s];
        row0 += n[s];
        xb0 += (long long)n[s] * rhs[s];
    }
    if (row0 > 0x7fffffffLL) return SPTRSV_ERR_TOO_LARGE;
    CUDA_TRY(cudaSetDevice(device));
    Batch* B = new Batch;
    B->device = device;
    B->count = count;
    B->sys = sys;
    B->tot_rp = rp0;
    B->tot_nnz = nz0;
    B->tot_rows = row0;
    B->tot_x = xb0;
    B->sched.assign(count, BS_PLAIN);
    B->panel_ok.assign(count, -1);
    B->have_bf16.assign(count, 0);
    if (const char* e = getenv("SPTRSV_P64_CTAS")) B->p64_ctas_per_sm = std::max(1, atoi(e));
    if (const char* e = getenv("SPTRSV_BJAC")) B->jacobi_elem = strcmp(e, "elem") == 0;
    B->have_f64.assign(count, 0);
    B->have_tc.assign(count, 0);
    B->gidx.assign(count, -1);
    B->pchunks.resize(count);
    int rc = 0;
    auto fail = [&](int code) {
        delete B;
        return code;
    };
    cudaError_t er;
    if ((er = cudaStreamCreateWithFlags(&B->st, cudaStreamNonBlocking)) != cudaSuccess ||
        (er = cudaEventCreate(&B->ev0)) != cudaSuccess || (er = cudaEventCreate(&B->ev1)) != cudaSuccess ||
        (er = cudaStreamCreateWithFlags(&B->st2, cudaStreamNonBlocking)) != cudaSuccess ||
        (er = cudaEventCreateWithFlags(&B->ev_fork, cudaEventDisableTiming)) != cudaSuccess ||
        (er = cudaEventCreateWithFlags(&B->ev_join, cudaEventDisableTiming)) != cudaSuccess ||
        (er = cudaDeviceGetAttribute(&B->sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
        return fail(set_cuda_error(er, "batch setup"));
    {
        std::vector<int> rp32(rp0);
        for (long long k = 0; k < rp0; ++k) rp32[k] = (int)row_ptr[k];
        if ((rc = B->rp.ensure(sizeof(int) * rp0)) || (rc = B->col.ensure(sizeof(int) * std::max(1LL, nz0))) ||
            (rc = B->val.ensure(sizeof(double) * std::max(1LL, nz0))) ||
            (rc = B->val32.ensure(sizeof(float) * std::max(1LL, nz0))) || (rc = B->invd.ensure(sizeof(double) * row0)) ||
            (rc = B->invd32.ensure(sizeof(float) * row0)) || (rc = B->dstate.ensure(sizeof(BState) * count)) ||
            (rc = B->dctl.ensure(sizeof(BCtl))) || (rc = B->r32.ensure(sizeof(float) * xb0)) ||
            (rc = B->d0.ensure(sizeof(float) * xb0)) || (rc = B->d1.ensure(sizeof(float) * xb0)))
            return fail(rc);
        // stream-ordered copies: the kernels below run on the batch's non-blocking stream
        if ((er = cudaMemcpyAsync(B->rp.p, rp32.data(), sizeof(int) * rp0, cudaMemcpyHostToDevice, B->st)) !=
                cudaSuccess ||
            (er = cudaStreamSynchronize(B->st)) != cudaSuccess)
            return fail(set_cuda_error(er, "batch upload"));
    }
    if (nz0 > 0) {
        if ((er = cudaMemcpyAsync(B->col.p, col, sizeof(int) * nz0, cudaMemcpyHostToDevice, B->st)) != cudaSuccess ||
            (er = cudaMemcpyAsync(B->val.p, val, sizeof(double) * nz0, cudaMemcpyHostToDevice, B->st)) !=
                cudaSuccess)
            return fail(set_cuda_error(er, "batch upload"));
        k_to_f32<<<B->sm_count * 16, 256, 0, B->st>>>((size_t)nz0, B->val.as<double>(), B->val32.as<float>());
        ++B->launches;
    }
    if ((rc = upload_vec(B->dsys, sys, B->st))) return fail(rc);
    HostSeg ar, ae;
    std::vector<int> all(count);
    for (int s = 0; s < count; ++s) {
        ar.add(s, sys[s].n);
        ae.add(s, (long long)sys[s].n * sys[s].rhs);
        all[s] = s;
    }
    if ((rc = B->all_rows.upload(ar, B->st)) || (rc = B->all_el.upload(ae, B->st))) return fail(rc);
    {
        std::vector<int2> oa = interleave_rows(sys, all);
        B->n_order_all = (unsigned)oa.size();
        if ((rc = upload_vec(B->order_all, oa, B->st))) return fail(rc);
    }
    if ((er = cudaMemsetAsync(B->dstate.p, 0, sizeof(BState) * count, B->st)) != cudaSuccess ||
        (er = cudaMemsetAsync(B->dctl.p, 0, sizeof(BCtl), B->st)) != cudaSuccess)
        return fail(set_cuda_error(er, "batch memset"));
    const BArgs A = B->args(nullptr, nullptr);
    k_b_setup<<<row_grid(B->sm_count, row0), 256, 0, B->st>>>(A, B->all_rows.list());
    ++B->launches;
    if ((er = cudaGetLastError()) != cudaSuccess || (er = cudaStreamSynchronize(B->st)) != cudaSuccess)
        return fail(set_cuda_error(er, "batch setup kernels"));
    BCtl c{};
    std::vector<BState> hs(count);
    if ((er = cudaMemcpy(&c, B->dctl.p, sizeof(c), cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (er = cudaMemcpy(hs.data(), B->dstate.p, sizeof(BState) * count, cudaMemcpyDeviceToHost)) != cudaSuccess)
        return fail(set_cuda_error(er, "batch setup read"));
    if (c.c.status) return fail(c.c.status);
    B->ratio.resize(count);
    for (int s = 0; s < count; ++s) {
        float r;
        memcpy(&r, &hs[s].ratio_bits, sizeof(float));
        B->ratio[s] = r;
        B->sched[s] = default_schedule(sys[s], nnz[s], r, hs[s].gapped);
        if (hs[s].gapped) B->panel_ok[s] = 0;
    }
    *out = reinterpret_cast<sptrsv_batch>(B);
    return 0;
}

int sptrsv_batch_destroy(sptrsv_batch bh) {
    Batch* B = reinterpret_cast<Batch*>(bh);
    if (!B) return SPTRSV_ERR_INVALID_ARG;
    delete B;
    return 0;
}

#define BH()                                                        \
    Batch* B = reinterpret_cast<Batch*>(bh);                        \
    if (!B) return SPTRSV_ERR_INVALID_ARG;                          \
    if (cudaSetDevice(B->device) != cudaSuccess) return SPTRSV_ERR_CUDA

int sptrsv_batch_get_schedule(sptrsv_batch bh, int* sched) {
    BH();
    if (!sched) return SPTRSV_ERR_INVALID_ARG;
    for (int s = 0; s < B->count; ++s) sched[s] = B->sched[s];
    return 0;
}

int sptrsv_batch_set_schedule(sptrsv_batch bh, const int* sched) {
    using namespace sptrsv;
    BH();
    if (!sched) return SPTRSV_ERR_INVALID_ARG;
    for (int s = 0; s < B->count; ++s)
        if (sched[s] < -1 || sched[s] >= BS_COUNT) return SPTRSV_ERR_INVALID_ARG;
    for (int s = 0; s < B->count; ++s) {
        if (sched[s] == BS_PANEL || sched[s] == BS_PANEL64) {
            const int rc = B->build_panels(s, sched[s] == BS_PANEL64);
            if (rc) return rc;
        }
        if (sched[s] == BS_JACOBI && !(B->ratio[s] < 1.f)) return SPTRSV_ERR_UNSUPPORTED;
    }
    for (int s = 0; s < B->count; ++s)
        if (sched[s] >= 0) B->sched[s] = sched[s];
    B->lists_ready = false;
    B->drop_graphs();
    return 0;
}

int sptrsv_batch_set_options(sptrsv_batch bh, double tol, int max_refine, int inner_tol_exp, int64_t budget_ns) {
    BH();
    if (tol > 0) B->tol = tol;
    if (max_refine > 0) B->max_refine = max_refine;
    if (inner_tol_exp > 0) B->inner_tol_exp = inner_tol_exp;
    if (budget_ns > 0) B->budget = budget_ns;
    B->drop_graphs();
    return 0;
}

int sptrsv_batch_solve(sptrsv_batch bh, int mode, const double* d_b, double* d_x) {
    BH();
    const int rc = B->solve(mode, d_b, d_x);
    sptrsv::set_last_status(rc);
    return rc;
}

int sptrsv_batch_sync(sptrsv_batch bh, int64_t* kernels) {
    BH();
    const int rc = B->sync(kernels);
    sptrsv::set_last_status(rc);
    return rc;
}

int sptrsv_batch_solve_host(sptrsv_batch bh, int mode, const double* h_b, double* h_x) {
    BH();
    if (!h_b || !h_x) return SPTRSV_ERR_INVALID_ARG;
    int rc;
    const size_t bytes = sizeof(double) * (size_t)B->tot_x;
    if ((rc = B->bw.ensure(bytes)) || (rc = B->xw.ensure(bytes))) return rc;
    CUDA_TRY(cudaMemcpyAsync(B->bw.p, h_b, bytes, cudaMemcpyHostToDevice, B->st));
    if ((rc = B->solve(mode, B->bw.as<double>(), B->xw.as<double>()))) return rc;
    CUDA_TRY(cudaMemcpyAsync(h_x, B->xw.p, bytes, cudaMemcpyDeviceToHost, B->st));
    return 0;
}

int sptrsv_batch_profile(sptrsv_batch bh, int mode, const double* d_b, double* d_x, float* kind_ms,
                         int* kind_launches, float* kind_first_ms) {
    BH();
    const int rc = B->profile(mode, d_b, d_x, kind_ms, kind_launches, kind_first_ms);
    sptrsv::set_last_status(rc);
    return rc;
}

int sptrsv_batch_stats(sptrsv_batch bh, int* status, int* steps, double* rel, int* sweeps) {
    BH();
    std::vector<sptrsv::BState> hs(B->count);
    CUDA_TRY(cudaStreamSynchronize(B->st));
    CUDA_TRY(cudaMemcpy(hs.data(), B->dstate.p, sizeof(sptrsv::BState) * B->count, cudaMemcpyDeviceToHost));
    for (int s = 0; s < B->count; ++s) {
        if (status) status[s] = hs[s].status;
        if (steps) steps[s] = hs[s].steps;
        if (rel) rel[s] = hs[s].rel;
        if (sweeps) sweeps[s] = hs[s].sweeps;
    }
    return 0;
}

int sptrsv_batch_info(sptrsv_batch bh, int64_t* totals, float* ratio) {
    BH();
    if (totals) {
        totals[0] = B->tot_rows;
        totals[1] = B->tot_nnz;
        totals[2] = B->tot_x;
        totals[3] = B->count;
        const int rc = B->build_lists();
        if (rc) return rc;
        totals[4] = B->g_entries64;
        totals[5] = B->g_fma64;
    }
    if (ratio)
        for (int s = 0; s < B->count; ++s) ratio[s] = B->ratio[s];
    return 0;
}

int sptrsv_batch_features(sptrsv_batch bh, int s, float* f) {
    BH();
    if (s < 0 || s >= B->count || !f) return SPTRSV_ERR_INVALID_ARG;
    int rc;
    if (!B->scratch) {
        sptrsv_handle h = nullptr;
        if ((rc = sptrsv_create(&h, B->device))) return rc;
        B->scratch = reinterpret_cast<sptrsv::Handle*>(h);
    }
    sptrsv::Handle& H = *B->scratch;
    const sptrsv::BSys& S = B->sys[s];
    H.drop_matrix();
    H.n = S.n;
    H.nnz = (int)((s + 1 < B->count ? B->sys[s + 1].nz0 : B->tot_nnz) - S.nz0);
    H.rp = B->rp.as<int>() + S.rp0;
    H.col = B->col.as<int>() + S.nz0;
    H.val = B->val.as<double>() + S.nz0;
    if ((rc = H.analyse())) return rc;
    if (B->panel_ok[s] != 0) {
        // the panel structure the batched path would use (uniform 64-row chunks), as in the
        // selector's training data for banded factors
        std::vector<int> sn;
        for (int a = 0; a < S.n; a += 64) sn.push_back(a);
        sn.push_back(S.n);
        rc = H.set_supernodes((int)sn.size() - 1, sn.data());
        if (rc && rc != SPTRSV_ERR_SUPERNODES) return rc;
    }
    rc = H.features(f, S.rhs);
    H.drop_matrix();
    return rc;
}

int sptrsv_batch_timer_begin(sptrsv_batch bh) {
    BH();
    CUDA_TRY(cudaEventRecord(B->ev0, B->st));
    return 0;
}

int sptrsv_batch_timer_end(sptrsv_batch bh, float* ms) {
    BH();
    CUDA_TRY(cudaEventRecord(B->ev1, B->st));
    CUDA_TRY(cudaEventSynchronize(B->ev1));
    float t = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&t, B->ev0, B->ev1));
    if (ms) *ms = t;
    return 0;
}

int64_t sptrsv_batch_launches(sptrsv_batch bh) {
    Batch* B = reinterpret_cast<Batch*>(bh);
    return B ? B->launches : -1;
}

}  // extern "C"
