// tune.cu -- the exhaustive autotuner and the matrix features of the learned selector.
//
// The autotuner times every applicable schedule of a fixed candidate table on the resident
// matrix (device buffers, a seeded random right-hand side, CUDA events on the handle's stream),
// keeps the fastest that reaches the accuracy contract (FP64 paths exact; mixed paths at the
// refinement tolerance) and caches it per RHS class, where AUTO picks it up.  A candidate whose
// first run exceeds the per-candidate cap is measured once; failures (for instance a refinement
// that does not converge) are recorded as infinite.  The timing table is returned so that it can
// train and judge the learned selector.
//
// The features (24 values, log-scaled where sizes are concerned) describe the matrix: size,
// density, row-length moments, dependency depth, level-width histogram, dominance of the
// diagonal, supernode-width histogram, and the number of right-hand sides.
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>
#include "common.cuh"
#include "kernels.cuh"
#include "handle.cuh"

namespace sptrsv {

// The candidate table (index = schedule id used by the selector).
const sptrsv_opts* tune_candidates(int* count) {
    static sptrsv_opts table[SPTRSV_TUNE_CANDIDATES];
    static bool init = false;
    if (!init) {
        for (int k = 0; k < SPTRSV_TUNE_CANDIDATES; ++k) sptrsv_default_opts(&table[k]);
        int k = 0;
        table[k].schedule = SPTRSV_SCHED_SYNCFREE_BLOCK; ++k;                                   // 0
        table[k].schedule = SPTRSV_SCHED_SYNCFREE_THREAD; ++k;                                  // 1
        table[k].schedule = SPTRSV_SCHED_SYNCFREE_WARP; table[k].rows_per_warp = 1; ++k;        // 2
        table[k].schedule = SPTRSV_SCHED_SYNCFREE_WARP; table[k].rows_per_warp = 4; ++k;        // 3
        table[k].schedule = SPTRSV_SCHED_SYNCFREE_WARP; table[k].rows_per_warp = 8; ++k;        // 4
        table[k].schedule = SPTRSV_SCHED_SYNCFREE_CSC; ++k;                                     // 5
        table[k].schedule = SPTRSV_SCHED_LEVELSET; ++k;                                         // 6
        table[k].schedule = SPTRSV_SCHED_JACOBI; table[k].precision = SPTRSV_PREC_MIXED; ++k;   // 7
        table[k].schedule = SPTRSV_SCHED_SYNCFREE_BLOCK; table[k].precision = SPTRSV_PREC_MIXED; ++k;  // 8
        table[k].schedule = SPTRSV_SCHED_SYNCFREE_WARP; table[k].precision = SPTRSV_PREC_MIXED;
        table[k].rows_per_warp = 4; ++k;                                                          // 9
        table[k].schedule = SPTRSV_SCHED_LEVELSET; table[k].precision = SPTRSV_PREC_MIXED; ++k; // 10
        table[k].schedule = SPTRSV_SCHED_SUPERNODAL; ++k;                                       // 11
        table[k].schedule = SPTRSV_SCHED_SUPERNODAL; table[k].precision = SPTRSV_PREC_MIXED; ++k;  // 12
        table[k].schedule = SPTRSV_SCHED_SYNCFREE_WARP; table[k].rows_per_warp = 2; ++k;        // 13
        table[k].schedule = SPTRSV_SCHED_JACOBI; table[k].precision = SPTRSV_PREC_MIXED;
        table[k].inner_tol_exp = 5; ++k;                                                          // 14
        table[k].schedule = SPTRSV_SCHED_SYNCFREE_THREAD; table[k].precision = SPTRSV_PREC_MIXED; ++k;  // 15
        init = true;
    }
    *count = SPTRSV_TUNE_CANDIDATES;
    return table;
}

bool Handle::applicable(const sptrsv_opts& o, int rhs) const {
    if (o.schedule == SPTRSV_SCHED_SUPERNODAL && !have_supernodes) return false;
    if ((o.schedule == SPTRSV_SCHED_SYNCFREE_THREAD || o.schedule == SPTRSV_SCHED_SYNCFREE_BLOCK) && rhs != 1)
        return false;
    if (o.schedule == SPTRSV_SCHED_JACOBI && !(max_ratio < 1.0)) return false;  // would not contract
    return true;
}

__global__ void k_fill_uniform(size_t count, uint64_t seed, double* __restrict__ b) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x) {
        uint64_t z = (k + 1) * 0x9E3779B97F4A7C15ull + seed;  // splitmix64
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        b[k] = 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
    }
}

// Raise the abort flag of the running solve from a second stream (the copy engine runs beside the
// solve's kernels); every spin and ticket loop polls it and returns, so the solve ends early with
// a meaningless result.  Re-raised until the solve's stream drains, in case a graph's own reset of
// the control block ran after the first raise.
int Handle::cancel_until_idle() {
    if (!cancel_st) CUDA_TRY(cudaStreamCreateWithFlags(&cancel_st, cudaStreamNonBlocking));
    if (!cancel_flag) {
        CUDA_TRY(cudaHostAlloc((void**)&cancel_flag, sizeof(int), cudaHostAllocDefault));
        *cancel_flag = 1;
    }
    for (int k = 0; k < 100000; ++k) {
        CUDA_TRY(cudaMemcpyAsync(&ctl->abort, cancel_flag, sizeof(int), cudaMemcpyHostToDevice, cancel_st));
        CUDA_TRY(cudaStreamSynchronize(cancel_st));
        const cudaError_t q = cudaStreamQuery(st);
        if (q == cudaSuccess) return 0;
        if (q != cudaErrorNotReady) return set_cuda_error(q, "cancel");
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    return 0;
}

// One timed solve of candidate o.  With abort_ms > 0 the host watches the solve and cancels it
// once it has run longer than abort_ms: the time is then a lower bound and *censored is set.
int Handle::timed_candidate(const sptrsv_opts& o, int rhs, float abort_ms, float* ms, bool* censored) {
    *censored = false;
    *ms = INFINITY;
    CUDA_TRY(cudaEventRecord(ev0, st));
    int rc = solve(&o, tune_b.as<double>(), tune_x.as<double>(), rhs, SPTRSV_ROW_MAJOR);
    if (rc) return rc;
    CUDA_TRY(cudaEventRecord(ev1, st));
    if (abort_ms > 0.f) {
        const auto t0 = std::chrono::steady_clock::now();
        for (;;) {
            const cudaError_t q = cudaEventQuery(ev1);
            if (q == cudaSuccess) break;
            if (q != cudaErrorNotReady) return set_cuda_error(q, "tune query");
            const float el = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
            if (el > abort_ms) {
                if ((rc = cancel_until_idle())) return rc;
                (void)sync();  // status of a cancelled run is meaningless; clears it
                *censored = true;
                *ms = el;
                return 0;
            }
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
    }
    if ((rc = sync())) return rc;
    CUDA_TRY(cudaEventElapsedTime(ms, ev0, ev1));
    return 0;
}

// Exhaustive tuning.  Candidates run in a fixed order that usually finds a fast one early; with
// abort_ms > 0, once one candidate has finished, a later one still running after
// max(abort_ms, 20 x the best so far) is cancelled and reported as censored (its time a lower
// bound).
int Handle::autotune(int rhs, float cap_ms, int reps, float abort_ms, float* ms_out, int* censored_out, int* best_id) {
    if (!analysed) return SPTRSV_ERR_NO_ANALYSIS;
    int rc;
    if ((rc = ensure_levels())) return rc;
    const size_t nr = (size_t)n * rhs;
    if ((rc = tune_b.ensure(sizeof(double) * nr)) || (rc = tune_x.ensure(sizeof(double) * nr))) return rc;
    k_fill_uniform<<<sm_count * 4, 256, 0, st>>>(nr, 0x5EEDull + (uint64_t)rhs, tune_b.as<double>());
    ++launches;
    CUDA_TRY(cudaGetLastError());
    int K = 0;
    const sptrsv_opts* cand = tune_candidates(&K);
    static const int order[SPTRSV_TUNE_CANDIDATES] = {7, 14, 11, 12, 0, 8, 13, 2, 3, 4, 9, 10, 6, 5, 1, 15};
    float best = INFINITY;
    int bid = -1;
    for (int q = 0; q < K; ++q) {
        const int k = order[q];
        float t = INFINITY;
        bool cens = false;
        if (applicable(cand[k], rhs)) {
            const sptrsv_opts o = cand[k];
            // nothing is cancelled before one candidate has finished, so a pick always exists
            const float lim = abort_ms > 0.f && std::isfinite(best) ? std::max(abort_ms, 20.f * best) : 0.f;
            float first = INFINITY;
            rc = timed_candidate(o, rhs, lim, &first, &cens);
            if (rc == 0 && !cens) {
                t = first;
                for (int r = 0; r < reps && first <= cap_ms; ++r) {
                    float e = INFINITY;
                    bool c2 = false;
                    if ((rc = timed_candidate(o, rhs, lim, &e, &c2)) || c2) break;
                    t = std::min(t, e);
                }
                if (rc) t = INFINITY;
            } else if (rc == 0 && cens) {
                t = first;
            } else if (rc == SPTRSV_ERR_CUDA || rc == SPTRSV_ERR_NO_DEVICE) {
                return rc;
            }
            rc = 0;
        }
        if (ms_out) ms_out[k] = t;
        if (censored_out) censored_out[k] = cens ? 1 : 0;
        if (!cens && t < best) { best = t; bid = k; }
    }
    if (bid < 0) return SPTRSV_ERR_UNSUPPORTED;
    const int cls = rhs_class(rhs);
    tuned[cls] = cand[bid];
    tuned_valid[cls] = true;
    if (best_id) *best_id = bid;
    return 0;
}

int rhs_class(int rhs) { return rhs <= 1 ? 0 : (rhs <= 8 ? 1 : (rhs <= 32 ? 2 : 3)); }

// level-width histogram (log2 bins of rows per level) on the device
__global__ void k_width_hist(int max_level, const int* __restrict__ lptr, unsigned* __restrict__ hist) {
    for (int l = blockIdx.x * blockDim.x + threadIdx.x + 1; l <= max_level; l += gridDim.x * blockDim.x) {
        const int w = lptr[l + 1] - lptr[l];
        int b = 0;
        while ((1 << (b + 1)) <= w && b < 7) ++b;
        atomicAdd(&hist[b], 1u);
    }
}

int Handle::features(float* f, int rhs) {
    if (!analysed) return SPTRSV_ERR_NO_ANALYSIS;
    int rc;
    if ((rc = ensure_levels())) return rc;
    if ((rc = scratch.ensure(64 * sizeof(unsigned)))) return rc;
    CUDA_TRY(cudaMemsetAsync(scratch.p, 0, 8 * sizeof(unsigned), st));
    k_width_hist<<<std::max(1, std::min(1024, (max_level + 255) / 256)), 256, 0, st>>>(max_level, level_ptr.as<int>(),
                                                                                    (unsigned*)scratch.p);
    ++launches;
    unsigned hist[8];
    CUDA_TRY(cudaMemcpyAsync(hist, scratch.p, sizeof(hist), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    const double L = std::max(1, max_level);
    int k = 0;
    f[k++] = (float)std::log2((double)n);
    f[k++] = (float)std::log2((double)nnz);
    f[k++] = (float)std::log2(mean_len);
    f[k++] = (float)std::log2(1.0 + std_len);
    f[k++] = (float)std::log2(L);
    f[k++] = (float)std::log2((double)n / L);           // mean level width
    f[k++] = (float)std::log2(1.0 + max_ratio);         // diagonal dominance
    f[k++] = max_ratio < 1.0 ? 1.f : 0.f;
    for (int b = 0; b < 8; ++b) f[k++] = (float)(hist[b] / L);  // level-width histogram (fractions)
    // supernode-width histogram: <=8, <=32, <=128, wider (fractions of rows), and their count
    float sw[4] = {0.f, 0.f, 0.f, 0.f};
    const bool user_sn = have_supernodes && !auto_supernodes;  // the caller's partition, not uniform chunks
    if (user_sn) {
        std::vector<int> ss(sn_count + 1);
        CUDA_TRY(cudaMemcpy(ss.data(), sn_start.p, sizeof(int) * (sn_count + 1), cudaMemcpyDeviceToHost));
        for (int s = 0; s < sn_count; ++s) {
            const int w = ss[s + 1] - ss[s];
            sw[w <= 8 ? 0 : (w <= 32 ? 1 : (w <= 128 ? 2 : 3))] += (float)w / n;
        }
    }
    for (int b = 0; b < 4; ++b) f[k++] = sw[b];
    f[k++] = user_sn ? (float)std::log2(1.0 + sn_count) : 0.f;
    f[k++] = user_sn ? 1.f : 0.f;
    f[k++] = (float)std::log2(1.0 + (double)nnz / n * (double)n / L);  // work per level
    f[k++] = (float)std::log2((double)std::max(1, rhs));                 // right-hand sides
    return 0;
}

}  // namespace sptrsv

using sptrsv::Handle;

extern "C" {

int sptrsv_autotune(sptrsv_handle hh, int rhs, float cap_ms, int reps, float* cand_ms, int* best_id, sptrsv_opts* best) {
    return sptrsv_autotune_bounded(hh, rhs, cap_ms, reps, 0.f, cand_ms, nullptr, best_id, best);
}

int sptrsv_autotune_bounded(sptrsv_handle hh, int rhs, float cap_ms, int reps, float abort_ms, float* cand_ms,
                            int* censored, int* best_id, sptrsv_opts* best) {
    Handle* h = reinterpret_cast<Handle*>(hh);
    if (!h || rhs < 1) return SPTRSV_ERR_INVALID_ARG;
    if (cudaSetDevice(h->device) != cudaSuccess) return SPTRSV_ERR_CUDA;
    int id = -1;
    int rc = h->autotune(rhs, cap_ms > 0 ? cap_ms : 50.f, reps >= 0 ? reps : 2, abort_ms, cand_ms, censored, &id);
    if (rc) return rc;
    if (best_id) *best_id = id;
    if (best) {
        int K;
        *best = sptrsv::tune_candidates(&K)[id];
    }
    return 0;
}

int sptrsv_candidate(int id, sptrsv_opts* o) {
    int K = 0;
    const sptrsv_opts* c = sptrsv::tune_candidates(&K);
    if (id < 0 || id >= K || !o) return SPTRSV_ERR_INVALID_ARG;
    *o = c[id];
    return 0;
}

int sptrsv_candidate_applicable(sptrsv_handle hh, int id, int rhs) {
    Handle* h = reinterpret_cast<Handle*>(hh);
    int K = 0;
    const sptrsv_opts* c = sptrsv::tune_candidates(&K);
    if (!h || id < 0 || id >= K) return 0;
    return h->applicable(c[id], rhs) ? 1 : 0;
}

int sptrsv_features(sptrsv_handle hh, int rhs, float* features) {
    Handle* h = reinterpret_cast<Handle*>(hh);
    if (!h || !features || rhs < 1) return SPTRSV_ERR_INVALID_ARG;
    if (cudaSetDevice(h->device) != cudaSuccess) return SPTRSV_ERR_CUDA;
    return h->features(features, rhs);
}

int sptrsv_set_tuned(sptrsv_handle hh, int rhs, const sptrsv_opts* o) {
    Handle* h = reinterpret_cast<Handle*>(hh);
    if (!h || !o) return SPTRSV_ERR_INVALID_ARG;
    const int cls = sptrsv::rhs_class(rhs);
    h->tuned[cls] = *o;
    h->tuned_valid[cls] = true;
    h->drop_graphs();
    return 0;
}

}  // extern "C"
