// api.cu -- the handle API of include/sptrsv_gb300.h: device context, analysis driver,
// schedule selection, solve enqueue (replayed from cached CUDA graphs) and host helpers.
// The reference-signature entry points live in dropin.cu on top of this file.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>
#include "common.cuh"
#include "kernels.cuh"
#include "handle.cuh"
#include "batch.cuh"

namespace sptrsv {

static thread_local int t_last_status = 0;
void set_last_status(int s) { t_last_status = s; }

int set_cuda_error(cudaError_t e, const char* what) {
    if (getenv("SPTRSV_VERBOSE")) fprintf(stderr, "sptrsv: CUDA error %s at %s\n", cudaGetErrorString(e), what);
    (void)cudaGetLastError();
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return SPTRSV_ERR_NO_DEVICE;
    return SPTRSV_ERR_CUDA;
}

int DevBuf::ensure(size_t bytes) {
    if (bytes == 0) bytes = 1;
    if (cap >= bytes) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    CUDA_TRY(cudaMalloc(&p, bytes));
    cap = bytes;
    return 0;
}
void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
}

__global__ void k_narrow_rp(int count, const int64_t* __restrict__ in, int* __restrict__ out, Ctl* ctl) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int64_t v = in[i];
        if (v < 0 || v > 0x7fffffffll) { record_error(ctl, SPTRSV_ERR_TOO_LARGE); out[i] = 0; }
        else out[i] = (int)v;
    }
}

int Handle::mark(int kind) {
    if (!profiling) return 0;
    if (prof_n >= (int)prof_ev.size()) {
        cudaEvent_t e;
        CUDA_TRY(cudaEventCreate(&e));
        prof_ev.push_back(e);
        prof_kind.push_back(0);
    }
    CUDA_TRY(cudaEventRecord(prof_ev[prof_n], st));
    prof_kind[prof_n] = kind;
    ++prof_n;
    return 0;
}

int Handle::read_ctl(Ctl* out) {
    CUDA_TRY(cudaMemcpyAsync(out, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return 0;
}

int Handle::reset_ctl() {
    CUDA_TRY(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st));
    return 0;
}

void Handle::drop_graphs() {
    for (auto& g : graphs) if (g.exec) cudaGraphExecDestroy(g.exec);
    graphs.clear();
}

void Handle::drop_matrix() {
    drop_graphs();
    analysed = false;
    levels_ready = false;
    have_csc = false;
    have_offdiag = false;
    have_supernodes = false;
    auto_supernodes = false;
    skyline = false;
    for (bool& v : tuned_valid) v = false;
    n = nnz = max_level = 0;
    rp = col = nullptr;
    val = nullptr;
}

// Runs validation and the full analysis on (rp, col, val) already on the device.
int Handle::analyse() {
    int rc;
    Ctl c{};
    if ((rc = reset_ctl())) return rc;
    if ((rc = in_degree.ensure(sizeof(int) * (size_t)n))) return rc;
    if ((rc = invd.ensure(sizeof(double) * (size_t)n))) return rc;
    if ((rc = invd32.ensure(sizeof(float) * (size_t)n))) return rc;
    if ((rc = val32.ensure(sizeof(float) * (size_t)nnz))) return rc;
    if ((rc = levels.ensure(sizeof(int) * (size_t)n))) return rc;
    if ((rc = stats.ensure(4 * sizeof(unsigned long long)))) return rc;
    const int sgrid = sm_count * 4;
    k_validate<<<sgrid, 256, 0, st>>>(n, nnz, rp, col, val, in_degree.as<int>(), invd.as<double>(),
                                      invd32.as<float>(), ctl);
    ++launches;
    CUDA_TRY(cudaGetLastError());
    if ((rc = read_ctl(&c))) return rc;
    if (c.status) return c.status;
    k_to_f32<<<sgrid, 256, 0, st>>>((size_t)nnz, val, val32.as<float>());
    CUDA_TRY(cudaMemsetAsync(stats.p, 0, 4 * sizeof(unsigned long long), st));
    k_row_stats<<<sgrid, 256, 0, st>>>(n, rp, col, val, stats.as<unsigned long long>(),
                                       stats.as<unsigned long long>() + 1,
                                       reinterpret_cast<double*>(stats.as<unsigned long long>() + 2),
                                       stats.as<unsigned long long>() + 3);
    launches += 2;
    CUDA_TRY(cudaGetLastError());
    unsigned long long hs[4];
    CUDA_TRY(cudaMemcpyAsync(hs, stats.p, sizeof(hs), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    double mr;
    memcpy(&mr, &hs[0], sizeof(double));
    max_ratio = mr;
    memcpy(&depth_est, &hs[2], sizeof(double));
    skyline = hs[3] == 0;
    mean_len = (double)nnz / n;
    const double ex2 = (double)hs[1] / n;
    std_len = std::sqrt(std::fmax(0.0, ex2 - mean_len * mean_len));
    analysed = true;
    return 0;
}

// Level kernel: 0 = one CTA over a shared-memory ring (window.cu, the default), 1 = warp per row
// over the whole GPU (SPTRSV_LEVELS_KERNEL=warp), kept for comparison.
static int levels_kernel() {
    static int k = [] {
        const char* e = getenv("SPTRSV_LEVELS_KERNEL");
        return (e && strcmp(e, "warp") == 0) ? 1 : 0;
    }();
    return k;
}

// Levels (core.cpp:244-270) and level buckets (core.cpp:282-288), computed on first need.
int Handle::ensure_levels() {
    if (levels_ready) return 0;
    if (!analysed) return SPTRSV_ERR_NO_ANALYSIS;
    int rc;
    Ctl c{};
    if ((rc = reset_ctl())) return rc;
    const int sgrid = sm_count * 4;
    CUDA_TRY(cudaMemsetAsync(levels.p, 0, sizeof(int) * (size_t)n, st));
    if (levels_kernel() == 0) {
        if ((rc = launch_window_levels(n, nnz, rp, col, levels.as<int>(), ctl, kDefaultBudgetNs, st, &launches))) return rc;
    } else {
        k_levels<<<sm_count * 2, 256, 0, st>>>(n, rp, col, levels.as<int>(), ctl, kDefaultBudgetNs);
        ++launches;
        CUDA_TRY(cudaGetLastError());
    }
    if ((rc = read_ctl(&c))) return rc;
    if (c.status) return c.status;
    max_level = c.max_level;
    // level buckets: counts -> level_ptr; stable radix sort of level keys -> level_rows
    if ((rc = level_ptr.ensure(sizeof(int) * (size_t)(max_level + 2)))) return rc;
    if ((rc = level_rows.ensure(sizeof(int) * (size_t)n))) return rc;
    const size_t need = (size_t)4 * n * sizeof(int) + (size_t)(max_level + 2) * sizeof(int) +
                        (size_t)256 * ((n + 4095) / 4096 + 1) * sizeof(int) * 2 + (1 << 20);
    if ((rc = scratch.ensure(need))) return rc;
    Scratch scr{(char*)scratch.p, scratch.cap, 0};
    int* cnt = scr.take<int>(max_level + 2);
    int* part = scr.take<int>(scan_partials_needed(max_level + 1));
    CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)(max_level + 2), st));
    k_level_hist<<<sgrid, 256, 0, st>>>(n, levels.as<int>(), cnt);
    ++launches;
    if ((rc = scan_exclusive(cnt, level_ptr.as<int>(), max_level + 1, part, st, &launches))) return rc;
    int bits = 0;
    while ((1ll << bits) <= (long long)max_level) ++bits;
    if ((rc = stable_sort_perm((const unsigned*)levels.p, n, bits, level_rows.as<int>(), scr, st, &launches)))
        return rc;
    // level-set grid: one CTA when its cost model wins.  Measured on GB300: a level costs ~0.3 us of
    // CTA barrier plus ~0.5 us per pass of 32 rows with one CTA; a grid barrier through L2 costs
    // ~1.5 us (one GPU-scope acq_rel atomic per CTA, acquire polls) plus ~0.5 us per pass.
    unsigned long long* passes = scr.take<unsigned long long>(2);
    unsigned long long hp[2] = {0, 0};
    CUDA_TRY(cudaMemsetAsync(passes, 0, sizeof(hp), st));
    if (max_level > 0) {
        k_level_passes<<<(max_level + 255) / 256, 256, 0, st>>>(max_level, level_ptr.as<int>(), sm_count, passes);
        ++launches;
    }
    CUDA_TRY(cudaMemcpyAsync(hp, passes, sizeof(hp), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    levelset_one_cta = 0.3 * max_level + 0.5 * (double)hp[0] < 1.5 * max_level + 0.5 * (double)hp[1];
    levels_ready = true;
    return 0;
}

int Handle::build_csc() {
    if (have_csc) return 0;
    int rc;
    if ((rc = csc_ptr.ensure(sizeof(int) * (size_t)(n + 1)))) return rc;
    if ((rc = csc_row.ensure(sizeof(int) * (size_t)nnz))) return rc;
    if ((rc = csc_val.ensure(sizeof(double) * (size_t)nnz))) return rc;
    const size_t need = (size_t)5 * nnz * sizeof(int) + (size_t)(n + 2) * sizeof(int) +
                        (size_t)256 * ((nnz + 4095) / 4096 + 1) * sizeof(int) * 2 + (1 << 20);
    if ((rc = scratch.ensure(need))) return rc;
    Scratch scr{(char*)scratch.p, scratch.cap, 0};
    int* erow = scr.take<int>(nnz);
    int* perm = scr.take<int>(nnz);
    int* cnt = scr.take<int>(n + 1);
    int* part = scr.take<int>(scan_partials_needed(n));
    k_entry_rows<<<sm_count * 8, 256, 0, st>>>(n, rp, erow);
    ++launches;
    int bits = 0;
    while ((1ll << bits) < (long long)n) ++bits;
    if ((rc = stable_sort_perm((const unsigned*)col, nnz, bits, perm, scr, st, &launches))) return rc;
    k_gather_csc<<<sm_count * 8, 256, 0, st>>>(nnz, perm, erow, val, csc_row.as<int>(), csc_val.as<double>());
    CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)(n + 1), st));
    k_col_hist<<<sm_count * 8, 256, 0, st>>>(nnz, col, cnt);
    launches += 2;
    if ((rc = scan_exclusive(cnt, csc_ptr.as<int>(), n, part, st, &launches))) return rc;
    CUDA_TRY(cudaStreamSynchronize(st));
    have_csc = true;
    return 0;
}

// FP64 AUTO with one RHS: the one-CTA window kernel up to ~90 entries per row, the block kernel on
// longer rows, whose many entries per lane the window kernel walks one a round.  Measured on GB300
// (kernel times, same GPU): random factors of 200k rows with 8.6 / 27 / 54 / 80 / 106 entries per
// row 11.8 / 28.4 / 54.3 / 96.4 / 123.6 ms against 32.0 / 87.5 / 99.2 / 104.3 / 106.8 ms for the
// block kernel; 64 x 64 band factor (65 entries per row) 1.33 against 2.26 ms; 2M-row system
// 118 against 324 ms.  SPTRSV_AUTO_WINDOW=0 / 1 forces either.
static bool auto_window(double mean_len) {
    static int w = [] {
        const char* e = getenv("SPTRSV_AUTO_WINDOW");
        return e ? (strcmp(e, "1") == 0 ? 1 : 0) : -1;
    }();
    return w < 0 ? mean_len <= 90.0 : w == 1;
}

// Schedule choice from the analysis features (the autotuner overrides it).
sptrsv_opts Handle::resolve(const sptrsv_opts* o, int rhs) const {
    sptrsv_opts r;
    sptrsv_default_opts(&r);
    if (o) r = *o;
    // a schedule chosen by the autotuner or the learned selector for this RHS class replaces AUTO
    // (schedule and precision: every candidate meets the accuracy contract)
    if (r.schedule == SPTRSV_SCHED_AUTO && tuned_valid[rhs_class(rhs)]) {
        const sptrsv_opts t = tuned[rhs_class(rhs)];
        r.schedule = t.schedule;
        r.precision = t.precision;
        r.rows_per_warp = t.rows_per_warp;
        r.inner_tol_exp = t.inner_tol_exp;
    }
    if (r.spin_budget_ns <= 0) r.spin_budget_ns = kDefaultBudgetNs;
    if (r.tol <= 0) r.tol = 1e-12;
    if (r.max_refine <= 0) r.max_refine = 8;
    // FP64 accuracy through refinement: FP32 Jacobi sweeps with FP64 residuals and updates, run
    // until the relative residual is at the level of an exact FP64 solve
    if (r.precision == SPTRSV_PREC_FP64 && r.schedule == SPTRSV_SCHED_JACOBI) {
        r.precision = SPTRSV_PREC_MIXED;
        r.tol = std::min(r.tol, kFp64RefineTol);
    }
    const double width = (double)n / (max_level > 0 ? max_level : 1);
    if (r.schedule == SPTRSV_SCHED_AUTO) {
        if (have_supernodes || (r.precision == SPTRSV_PREC_FP64 && dense_skyline())) {
            // banded / skyline rows without a partition: uniform chunks are built on first use
            r.schedule = SPTRSV_SCHED_SUPERNODAL;
        } else if (r.precision == SPTRSV_PREC_MIXED) {
            r.schedule = SPTRSV_SCHED_JACOBI;
        } else {
            // wide, shallow DAGs: one grid barrier per level is cheap; otherwise the block
            // sync-free kernel for one RHS (and, once per column, for several RHS on long rows)
            // and the RHS-tiled warp kernel for several RHS on short rows
            if (levels_ready && width >= 2048.0 && max_level <= 2000) r.schedule = SPTRSV_SCHED_LEVELSET;
            else if (rhs == 1) r.schedule = auto_window(mean_len) ? SPTRSV_SCHED_SYNCFREE_WINDOW : SPTRSV_SCHED_SYNCFREE_BLOCK;
            else if (mean_len >= kBlockPerColumnLen) r.schedule = SPTRSV_SCHED_SYNCFREE_BLOCK;
            else r.schedule = SPTRSV_SCHED_SYNCFREE_WARP;
        }
    }
    if (r.precision == SPTRSV_PREC_MIXED) {
        r.inner = (r.schedule == SPTRSV_SCHED_JACOBI) ? SPTRSV_SCHED_JACOBI : r.schedule;
        if (r.inner == SPTRSV_SCHED_SYNCFREE_CSC) r.inner = SPTRSV_SCHED_SYNCFREE_WARP;
        // Jacobi sweeps contract only for strictly diagonally dominant U
        if (r.inner == SPTRSV_SCHED_JACOBI && !(max_ratio < 1.0)) r.inner = SPTRSV_SCHED_SYNCFREE_WARP;
        // flat (unlooped) graphs run a fixed number of sweeps per correction
        if (r.inner_sweeps <= 0) r.inner_sweeps = 16;
        // the floor of the inner change test; a correction that needs less (its residual is
        // already near the tolerance) stops earlier, see k_check_outer
        if (r.inner_tol_exp <= 0) r.inner_tol_exp = 6;
    }
    if (r.rows_per_warp <= 0) {
        const double m = mean_len;
        r.rows_per_warp = m <= 6 ? 8 : (m <= 12 ? 4 : (m <= 24 ? 2 : 1));
    }
    return r;
}

int Handle::prepare(const sptrsv_opts& o, int rhs, int layout) {
    int rc;
    if (o.schedule == SPTRSV_SCHED_SUPERNODAL && !have_supernodes && skyline) {
        // exact FP64 panels over uniform chunks of a skyline matrix (every row contiguous from its
        // diagonal)
        std::vector<int> part;
        for (int a = 0; a < n; a += kAutoChunkRows) part.push_back(a);
        part.push_back(n);
        if ((rc = set_supernodes((int)part.size() - 1, part.data()))) return rc;
        auto_supernodes = true;
    }
    // a work buffer that grows moves: graphs captured with its old address are dropped
    bool moved = false;
    auto grow = [&](DevBuf& d, size_t bytes) {
        void* old = d.p;
        const int r = d.ensure(bytes);
        moved |= old && d.p != old;
        return r;
    };
    if (o.schedule == SPTRSV_SCHED_LEVELSET || (o.precision == SPTRSV_PREC_MIXED && o.inner == SPTRSV_SCHED_LEVELSET))
        if ((rc = ensure_levels())) return rc;
    const size_t nr = (size_t)n * rhs;
    if (rhs > 1 && layout == SPTRSV_COL_MAJOR) {
        if ((rc = grow(bw, sizeof(double) * nr))) return rc;
        if ((rc = grow(xw, sizeof(double) * nr))) return rc;
    }
    if (o.precision == SPTRSV_PREC_MIXED) {
        if (o.inner == SPTRSV_SCHED_JACOBI && rhs == 1)
            if ((rc = ensure_offdiag())) return rc;
        if ((rc = grow(r32, sizeof(float) * nr))) return rc;
        if ((rc = grow(d32a, sizeof(float) * nr))) return rc;
        if ((rc = grow(d32b, sizeof(float) * nr))) return rc;
        if ((rc = grow(norms, sizeof(double) * 2 * (size_t)rhs))) return rc;
    }
    if (o.schedule == SPTRSV_SCHED_SYNCFREE_CSC && o.precision == SPTRSV_PREC_FP64) {
        if ((rc = build_csc())) return rc;
        if ((rc = grow(indeg_work, sizeof(int) * (size_t)n))) return rc;
        if ((rc = grow(left, sizeof(double) * nr))) return rc;
    }
    if (o.schedule == SPTRSV_SCHED_SUPERNODAL && o.precision == SPTRSV_PREC_FP64 && have_supernodes) {
        if ((rc = grow(sn_ppart, sizeof(double) * (size_t)sn_prows * rhs))) return rc;
        if ((rc = grow(sn_pcnt, sizeof(int) * (size_t)sn_npan * p64_groups(rhs)))) return rc;
    }
    if (moved) drop_graphs();
    return 0;
}

// Only stream work (captured into a graph).
int Handle::enqueue(const sptrsv_opts& o, const double* b, double* x, int rhs, int layout) {
    int rc;
    const double* brm = b;
    double* xrm = x;
    const bool percol = block_per_column(o, rhs, layout);
    const bool conv = rhs > 1 && layout == SPTRSV_COL_MAJOR && !percol;
    prof_n = 0;
    if (profiling) {
        if (!prof0) CUDA_TRY(cudaEventCreate(&prof0));
        CUDA_TRY(cudaEventRecord(prof0, st));
    }
    if (conv) {
        if ((rc = launch_transpose(true, b, bw.as<double>(), n, rhs, st, &launches))) return rc;
        if ((rc = mark(SPTRSV_K_TRANSPOSE))) return rc;
        brm = bw.as<double>();
        xrm = xw.as<double>();
    }
    CUDA_TRY(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st));
    SolveArgs a{};
    a.n = n;
    a.rp = rp;
    a.col = col;
    a.val = val;
    a.invd = invd.p;
    a.b = brm;
    a.x = xrm;
    a.rhs = rhs;
    a.ctl = ctl;
    a.budget = o.spin_budget_ns;
    a.sm_count = sm_count;
    a.warps = resident_warps(o);
    a.nnz = nnz;
    a.st = st;
    a.launches = &launches;
    if (o.precision == SPTRSV_PREC_FP64) {
        switch (o.schedule) {
            case SPTRSV_SCHED_SYNCFREE_THREAD:
                if (rhs == 1) {
                    if ((rc = launch_fill_pending(false, xrm, (size_t)n * rhs, st, &launches))) return rc;
                    if ((rc = mark(SPTRSV_K_FILL))) return rc;
                    if ((rc = launch_pull_thread(false, a))) return rc;
                    if ((rc = mark(SPTRSV_K_PULL_THREAD))) return rc;
                    break;
                }
                // fallthrough: one lane per row has no multi-RHS form
            case SPTRSV_SCHED_SYNCFREE_WARP:
                if ((rc = launch_fill_pending(false, xrm, (size_t)n * rhs, st, &launches))) return rc;
                if ((rc = mark(SPTRSV_K_FILL))) return rc;
                if ((rc = launch_pull_warp(false, a, o.rows_per_warp, o.rhs_tile))) return rc;
                if ((rc = mark(SPTRSV_K_PULL_WARP))) return rc;
                break;
            case SPTRSV_SCHED_SYNCFREE_BLOCK:
                if (rhs == 1 || percol) {
                    // one column at a time (column-major b / x), each from a fresh row ticket
                    for (int c = 0; c < rhs; ++c) {
                        SolveArgs ac = a;
                        ac.b = brm + (size_t)c * n;
                        ac.x = xrm + (size_t)c * n;
                        ac.rhs = 1;
                        if (c > 0) CUDA_TRY(cudaMemsetAsync(&ctl->ticket, 0, sizeof(ctl->ticket), st));
                        if ((rc = launch_fill_pending(false, xrm + (size_t)c * n, (size_t)n, st, &launches))) return rc;
                        if ((rc = mark(SPTRSV_K_FILL))) return rc;
                        if ((rc = launch_bsf(false, ac))) return rc;
                        if ((rc = mark(SPTRSV_K_PULL_BLOCK))) return rc;
                    }
                    break;
                }
                if ((rc = launch_fill_pending(false, xrm, (size_t)n * rhs, st, &launches))) return rc;
                if ((rc = mark(SPTRSV_K_FILL))) return rc;
                if ((rc = launch_pull_warp(false, a, o.rows_per_warp, o.rhs_tile))) return rc;
                if ((rc = mark(SPTRSV_K_PULL_WARP))) return rc;
                break;
            case SPTRSV_SCHED_SYNCFREE_WINDOW:
                if (rhs == 1 || percol) {
                    for (int c = 0; c < rhs; ++c) {
                        SolveArgs ac = a;
                        ac.b = brm + (size_t)c * n;
                        ac.x = xrm + (size_t)c * n;
                        ac.rhs = 1;
                        if ((rc = launch_fill_pending(false, xrm + (size_t)c * n, (size_t)n, st, &launches))) return rc;
                        if ((rc = mark(SPTRSV_K_FILL))) return rc;
                        if ((rc = launch_window(false, ac))) return rc;
                        if ((rc = mark(SPTRSV_K_WINDOW))) return rc;
                    }
                    break;
                }
                // row-major right-hand sides: the RHS-tiled warp kernel
                if ((rc = launch_fill_pending(false, xrm, (size_t)n * rhs, st, &launches))) return rc;
                if ((rc = mark(SPTRSV_K_FILL))) return rc;
                if ((rc = launch_pull_warp(false, a, o.rows_per_warp, o.rhs_tile))) return rc;
                if ((rc = mark(SPTRSV_K_PULL_WARP))) return rc;
                break;
            case SPTRSV_SCHED_SYNCFREE_CSC:
                CUDA_TRY(cudaMemcpyAsync(indeg_work.p, in_degree.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, st));
                CUDA_TRY(cudaMemsetAsync(left.p, 0, sizeof(double) * (size_t)n * rhs, st));
                if ((rc = launch_push_csc(a, csc_ptr.as<int>(), csc_row.as<int>(), csc_val.as<double>(),
                                          indeg_work.as<int>(), left.as<double>())))
                    return rc;
                if ((rc = mark(SPTRSV_K_PUSH_CSC))) return rc;
                break;
            case SPTRSV_SCHED_LEVELSET: {
                SolveArgs al = a;
                al.warps = levelset_warps(o);
                if ((rc = launch_levelset(false, al, max_level, level_ptr.as<int>(), level_rows.as<int>()))) return rc;
                if ((rc = mark(SPTRSV_K_LEVELSET))) return rc;
                break;
            }
            case SPTRSV_SCHED_SUPERNODAL:
                if (!have_supernodes) return SPTRSV_ERR_SUPERNODES;
                if ((rc = launch_fill_pending(false, xrm, (size_t)n * rhs, st, &launches))) return rc;
                if ((rc = mark(SPTRSV_K_FILL))) return rc;
                if ((rc = launch_sn_solve(*this, false, brm, xrm, rhs, o.spin_budget_ns, &launches))) return rc;
                if ((rc = mark(SPTRSV_K_SUPERNODAL))) return rc;
                break;
            default:
                return SPTRSV_ERR_UNSUPPORTED;
        }
    } else {
        RefineArgs ra{};
        if ((rc = refine_args(o, brm, xrm, rhs, &ra))) return rc;
        const bool jac = o.inner == SPTRSV_SCHED_JACOBI;
        if ((rc = launch_refine_init(ra, true))) return rc;
        if ((rc = mark(SPTRSV_K_INIT))) return rc;
        for (int s = 0; s < o.max_refine; ++s) {
            if ((rc = launch_residual(ra, jac, 0))) return rc;
            if ((rc = mark(SPTRSV_K_RESIDUAL))) return rc;
            if ((rc = launch_check(ra, s, true))) return rc;
            if ((rc = mark(SPTRSV_K_CHECK))) return rc;
            if (jac) {
                int src = 0;
                if (o.inner_sweeps <= 1) {
                    if ((rc = launch_axpy_pending(ra, 0))) return rc;
                    if ((rc = mark(SPTRSV_K_AXPY))) return rc;
                } else {
                    for (int q = 1; q < o.inner_sweeps; ++q) {
                        if ((rc = launch_jacobi_sweep(ra, src, q == o.inner_sweeps - 1, false))) return rc;
                        if ((rc = mark(SPTRSV_K_JACOBI))) return rc;
                        src ^= 1;
                    }
                }
            } else if (o.inner == SPTRSV_SCHED_SUPERNODAL) {
                if (!have_supernodes) return SPTRSV_ERR_SUPERNODES;
                if ((rc = launch_sn_solve(*this, true, ra.r32, ra.d32[0], rhs, o.spin_budget_ns, &launches))) return rc;
                if ((rc = mark(SPTRSV_K_SUPERNODAL))) return rc;
                if ((rc = launch_axpy_pending(ra, 0))) return rc;
                if ((rc = mark(SPTRSV_K_AXPY))) return rc;
            } else {
                if ((rc = launch_exact_inner(ra, o.inner, o.rows_per_warp, 0, max_level, level_ptr.as<int>(),
                                             level_rows.as<int>(),
                                             o.inner == SPTRSV_SCHED_LEVELSET ? levelset_warps(o) : resident_warps(o))))
                    return rc;
                if ((rc = mark(SPTRSV_K_INNER))) return rc;
                if ((rc = launch_axpy_pending(ra, 0))) return rc;
                if ((rc = mark(SPTRSV_K_AXPY))) return rc;
            }
        }
        if ((rc = launch_residual(ra, false, 1))) return rc;
        if ((rc = mark(SPTRSV_K_RESIDUAL))) return rc;
        if ((rc = launch_check(ra, o.max_refine, false))) return rc;
        if ((rc = mark(SPTRSV_K_CHECK))) return rc;
    }
    if (conv) {
        if ((rc = launch_transpose(false, xrm, x, n, rhs, st, &launches))) return rc;
        if ((rc = mark(SPTRSV_K_TRANSPOSE))) return rc;
    }
    return 0;
}

// Warps of a level-set launch: the caller's or tuner's choice, else one CTA (32 warps) when the
// level widths favour it, else the rows model below.
int Handle::levelset_warps(const sptrsv_opts& o) const {
    if (o.resident_warps > 0 || warps_override > 0) return resident_warps(o);
    return levelset_one_cta ? 32 : resident_warps(o);
}

int Handle::resident_warps(const sptrsv_opts& o) const {
    if (o.resident_warps > 0) return o.resident_warps;
    if (warps_override > 0) return warps_override;
    // enough rows in flight to cover ~32 levels of the DAG; more warps only add spin traffic
    const double width = levels_ready && max_level > 0 ? (double)n / max_level : 64.0;
    const int rows = (int)std::min(1.0e9, std::max(256.0, width * 32.0));
    const int rpw = o.rows_per_warp > 0 ? o.rows_per_warp : 1;
    return std::max(64, rows / rpw);
}

int Handle::ensure_offdiag() {
    if (have_offdiag) return 0;
    int rc;
    if (sweep_kernel == 6) {
        // SELL slices
        const int nslices = sell_slices(n);
        if ((rc = sell_perm.ensure(sizeof(int) * (size_t)nslices * 32))) return rc;
        if ((rc = sell_len.ensure(sizeof(int) * (size_t)nslices))) return rc;
        if ((rc = sell_ptr.ensure(sizeof(int) * ((size_t)nslices + 1)))) return rc;
        if ((rc = scratch.ensure(sizeof(int) * (size_t)(scan_partials_needed(nslices) + 64)))) return rc;
        int total = 0;
        if ((rc = sell_prepare(n, rp, sell_perm.as<int>(), sell_len.as<int>(), sell_ptr.as<int>(), (int*)scratch.p,
                               sm_count, st, &launches, &total)))
            return rc;
        if ((rc = sell.ensure(sizeof(int2) * ((size_t)total + 32)))) return rc;
        if ((rc = sell_fill(n, rp, col, val, sell_perm.as<int>(), sell_len.as<int>(), sell_ptr.as<int>(),
                            sell.as<int2>(), sm_count, st, &launches)))
            return rc;
        CUDA_TRY(cudaStreamSynchronize(st));
        sell_nslices = nslices;
        have_offdiag = true;
        return 0;
    }
    if (sweep_kernel == 9) {
        // the group-jagged layout (32-row groups, jagged diagonals)
        const int ngroups = (n + 31) / 32;
        if ((rc = jbase.ensure(sizeof(int) * ((size_t)ngroups + 2)))) return rc;
        if ((rc = jmeta.ensure(sizeof(int) * (size_t)ngroups * 32))) return rc;
        if ((rc = scratch.ensure(sizeof(int) * ((size_t)ngroups + scan_partials_needed(ngroups) + 64)))) return rc;
        int* gsize = scratch.as<int>();
        int* part = gsize + ngroups + 32;
        int* overflow = jbase.as<int>() + ngroups + 1;
        CUDA_TRY(cudaMemsetAsync(overflow, 0, sizeof(int), st));
        if ((rc = launch_jds_sizes(n, rp, gsize, overflow, sm_count, st, &launches))) return rc;
        if ((rc = scan_exclusive(gsize, jbase.as<int>(), ngroups, part, st, &launches))) return rc;
        int tail[2] = {0, 0};
        CUDA_TRY(cudaMemcpyAsync(tail, jbase.as<int>() + ngroups, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        if (tail[1] == 0) {
            if ((rc = offdiag.ensure(sizeof(int2) * ((size_t)tail[0] + 4)))) return rc;
            if ((rc = launch_jds_fill(n, rp, col, val, jbase.as<int>(), jmeta.as<int>(), offdiag.as<int2>(), sm_count,
                                      st, &launches)))
                return rc;
            CUDA_TRY(cudaStreamSynchronize(st));
            off_jds = true;
            off_pairs = false;
            have_offdiag = true;
            return 0;
        }
        // a row too long for the group metadata: the paired layout instead
    }
    off_jds = false;
    const int kRoffPad = 64;
    if ((rc = roff.ensure(sizeof(int) * ((size_t)n + 1 + kRoffPad)))) return rc;
    if (sweep_kernel == 0 || sweep_kernel == 9) {
        // the paired layout of the default sweep: rows padded to an even slot count
        if ((rc = scratch.ensure(sizeof(int) * ((size_t)n + scan_partials_needed(n) + 64)))) return rc;
        int* len2 = scratch.as<int>();
        int* part = len2 + n + 32;
        if ((rc = launch_pair_offsets(n, rp, len2, roff.as<int>(), kRoffPad, part, sm_count, st, &launches)))
            return rc;
        int total = 0;
        CUDA_TRY(cudaMemcpyAsync(&total, roff.as<int>() + n, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        if ((rc = offdiag.ensure(sizeof(int2) * ((size_t)total + 4)))) return rc;
        CUDA_TRY(cudaMemsetAsync(offdiag.p, 0, sizeof(int2) * ((size_t)total + 4), st));
        if ((rc = launch_build_offdiag_pairs(n, rp, col, val, roff.as<int>(), offdiag.as<int2>(), sm_count, st,
                                             &launches)))
            return rc;
        CUDA_TRY(cudaStreamSynchronize(st));
        off_pairs = true;
        have_offdiag = true;
        return 0;
    }
    off_pairs = false;
    if ((rc = offdiag.ensure(sizeof(int2) * ((size_t)(nnz - n) + 4)))) return rc;
    CUDA_TRY(cudaMemsetAsync(offdiag.p, 0, sizeof(int2) * ((size_t)(nnz - n) + 4), st));
    if ((rc = launch_build_offdiag(n, rp, col, val, offdiag.as<int2>(), roff.as<int>(), kRoffPad, sm_count, st,
                                   &launches)))
        return rc;
    CUDA_TRY(cudaStreamSynchronize(st));
    have_offdiag = true;
    return 0;
}

int Handle::refine_args(const sptrsv_opts& o, const double* b, double* x, int rhs, RefineArgs* ra) {
    RefineArgs& r = *ra;
    r = RefineArgs{};
    r.n = n;
    r.nnz = nnz;
    r.rhs = rhs;
    r.rp = rp;
    r.col = col;
    r.val = val;
    r.val32 = val32.as<float>();
    r.invd = invd.as<double>();
    r.invd32 = invd32.as<float>();
    const bool sl = have_offdiag && rhs == 1 && sweep_kernel == 6;
    r.off = (have_offdiag && rhs == 1 && !sl) ? offdiag.as<int2>() : nullptr;
    r.roff = (have_offdiag && rhs == 1 && !sl) ? roff.as<int>() : nullptr;
    r.pairs = off_pairs ? 1 : 0;
    r.jmeta = (have_offdiag && rhs == 1 && off_jds) ? jmeta.as<int>() : nullptr;
    r.jbase = (have_offdiag && rhs == 1 && off_jds) ? jbase.as<int>() : nullptr;
    r.sweep_kernel = sweep_kernel;
    r.nslices = sl ? sell_nslices : 0;
    r.sell_perm = sl ? sell_perm.as<int>() : nullptr;
    r.sell_len = sl ? sell_len.as<int>() : nullptr;
    r.sell_ptr = sl ? sell_ptr.as<int>() : nullptr;
    r.sell = sl ? sell.as<int2>() : nullptr;
    r.b = b;
    r.x = x;
    r.r32 = r32.as<float>();
    r.d32[0] = d32a.as<float>();
    r.d32[1] = d32b.as<float>();
    r.rn2 = norms.as<double>();
    r.bn2 = norms.as<double>() + rhs;
    r.ctl = ctl;
    r.tol = o.tol;
    r.budget = o.spin_budget_ns;
    r.sm_count = sm_count;
    r.st = st;
    r.launches = &launches;
    return 0;
}

// Device-looped mixed solves: Jacobi inner sweeps run in conditional WHILE nodes, so the whole
// solve is one graph launch with no launches after convergence.
bool Handle::cond_eligible(const sptrsv_opts& o, int rhs) const {
    (void)rhs;
    return use_graphs && !profiling && o.precision == SPTRSV_PREC_MIXED && o.inner == SPTRSV_SCHED_JACOBI;
}

int Handle::build_cond_graph(const sptrsv_opts& o, const double* b, double* x, double* x_out, int rhs, int layout,
                             cudaGraphExec_t* out, int64_t* fixed_kernels) {
    *out = nullptr;
    const bool conv = rhs > 1 && layout == SPTRSV_COL_MAJOR;
    const double* brm = conv ? bw.as<double>() : b;
    double* xrm = conv ? xw.as<double>() : x;
    RefineArgs ra{};
    int rc = refine_args(o, brm, xrm, rhs, &ra);
    if (rc) return rc;
    ra.x_out = rhs == 1 ? x_out : nullptr;
    int64_t scratch_launches = 0;
    ra.launches = &scratch_launches;
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle ho = 0, hi = 0;
    cudaError_t e = cudaGraphConditionalHandleCreate(&ho, g, 1, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hi, g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return set_cuda_error(e, "conditional handle"); }
    cudaGraph_t obody = nullptr, ibody = nullptr;
    const float eps = powf(10.f, -(float)o.inner_tol_exp);
    const int max_sweeps = 200;  // per correction; the change test normally stops far earlier
    auto add_while = [&](cudaGraph_t parent, cudaGraphConditionalHandle h, cudaGraph_t* body) -> cudaError_t {
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        cudaError_t er = cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd);
        if (er != cudaSuccess) return er;
        // cudaGraphNodeParams has no usable default constructor: build it in zeroed storage
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
    // top level: [transpose b] memset ctl, init, WHILE(outer), [transpose x]
    e = cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
        if (!rc && conv) rc = launch_transpose(true, b, bw.as<double>(), n, rhs, st, &scratch_launches);
        if (!rc && cudaMemsetAsync(ctl, 0, sizeof(Ctl), st) != cudaSuccess) rc = SPTRSV_ERR_CUDA;
        if (!rc) rc = launch_refine_init(ra, true);
        if (!rc && add_while(g, ho, &obody) != cudaSuccess) rc = SPTRSV_ERR_CUDA;
        if (!rc && conv) rc = launch_transpose(false, xrm, x, n, rhs, st, &scratch_launches);
        cudaGraph_t g2 = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(st, &g2);
        if (!rc && e2 != cudaSuccess) rc = set_cuda_error(e2, "capture top");
    } else {
        rc = set_cuda_error(e, "begin capture top");
    }
    const int64_t fixed = scratch_launches;
    // outer body: residual (seeds d0), test, WHILE(inner), x += d
    if (!rc) {
        e = cudaStreamBeginCaptureToGraph(st, obody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            rc = launch_residual(ra, true, 0);
            if (!rc) rc = launch_check_outer(ra, o.max_refine, ho, hi);
            if (!rc && add_while(obody, hi, &ibody) != cudaSuccess) rc = SPTRSV_ERR_CUDA;
            if (!rc) rc = launch_axpy_pending(ra, 0);
            cudaGraph_t g2 = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(st, &g2);
            if (!rc && e2 != cudaSuccess) rc = set_cuda_error(e2, "capture outer");
        } else {
            rc = set_cuda_error(e, "begin capture outer");
        }
    }
    // inner body: two sweeps (d0 -> d1 -> d0), the second measuring its change, then the test
    if (!rc) {
        e = cudaStreamBeginCaptureToGraph(st, ibody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            rc = launch_jacobi_sweep(ra, 0, false, false);
            if (!rc) rc = launch_jacobi_sweep(ra, 1, false, true);
            if (!rc) rc = launch_check_inner(ra, eps, max_sweeps, hi);
            cudaGraph_t g2 = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(st, &g2);
            if (!rc && e2 != cudaSuccess) rc = set_cuda_error(e2, "capture inner");
        } else {
            rc = set_cuda_error(e, "begin capture inner");
        }
    }
    if (!rc) {
        e = cudaGraphInstantiate(out, g, 0);
        if (e != cudaSuccess) rc = set_cuda_error(e, "instantiate conditional");
    }
    cudaGraphDestroy(g);
    (void)cudaGetLastError();
    *fixed_kernels = fixed;
    return rc;
}

int Handle::solve(const sptrsv_opts* o_in, const double* b, double* x, int rhs, int layout) {
    if (!analysed) return SPTRSV_ERR_NO_ANALYSIS;
    if (rhs < 1 || !b || !x || (layout != SPTRSV_COL_MAJOR && layout != SPTRSV_ROW_MAJOR)) return SPTRSV_ERR_INVALID_ARG;
    if ((size_t)n * rhs > (size_t)0x7fffffff) return SPTRSV_ERR_TOO_LARGE;
    sptrsv_opts o = resolve(o_in, rhs);
    if (o.precision == SPTRSV_PREC_MIXED && rhs > 1024) return SPTRSV_ERR_UNSUPPORTED;
    int rc;
    if ((rc = prepare(o, rhs, layout))) return rc;
    last_mixed = o.precision == SPTRSV_PREC_MIXED;
    last_cond = false;
    last_mirrored = false;
    // profiled solves launch directly: their per-step events are timed from the host stream
    if (!use_graphs || profiling) return enqueue(o, b, x, rhs, layout);
    const bool cond = cond_eligible(o, rhs);
    GraphKey key;
    key.o = o;
    key.b = b;
    key.x = x;
    key.xo = (cond && rhs == 1) ? x_mirror : nullptr;
    key.rhs = rhs;
    key.layout = layout;
    key.warps = warps_override;
    key.prof = profiling;
    for (auto& g : graphs) {
        if (g.key.same(key)) {
            CUDA_TRY(cudaGraphLaunch(g.exec, st));
            launches += g.kernels;
            last_cond = cond;
            last_mirrored = key.xo != nullptr;
            cond_fixed_kernels = g.kernels;
            return 0;
        }
    }
    if (cond) {
        cudaGraphExec_t exec = nullptr;
        int64_t fixed = 0;
        rc = build_cond_graph(o, b, x, key.xo, rhs, layout, &exec, &fixed);
        if (!rc && exec) {
            GraphEntry ge;
            ge.key = key;
            ge.exec = exec;
            ge.kernels = fixed;
            if (graphs.size() >= 16) {
                cudaGraphExecDestroy(graphs.front().exec);
                graphs.erase(graphs.begin());
            }
            graphs.push_back(ge);
            CUDA_TRY(cudaGraphLaunch(exec, st));
            launches += fixed;
            last_cond = true;
            last_mirrored = key.xo != nullptr;
            cond_fixed_kernels = fixed;
            return 0;
        }
        // conditional nodes unavailable: fall through to the flat graph (which writes no mirror)
        (void)cudaGetLastError();
        key.xo = nullptr;
    }
    const int64_t before = launches;
    CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    rc = enqueue(o, b, x, rhs, layout);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    cudaGraphExec_t exec = nullptr;
    if (!rc && e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (rc || e != cudaSuccess || !exec) {
        // capture not possible for this sequence: run it directly on the stream
        (void)cudaGetLastError();
        launches = before;
        return enqueue(o, b, x, rhs, layout);
    }
    GraphEntry ge;
    ge.key = key;
    ge.exec = exec;
    ge.kernels = launches - before;
    launches = before;
    if (graphs.size() >= 16) {
        cudaGraphExecDestroy(graphs.front().exec);
        graphs.erase(graphs.begin());
    }
    graphs.push_back(ge);
    CUDA_TRY(cudaGraphLaunch(exec, st));
    launches += ge.kernels;
    return 0;
}

int Handle::sync() {
    CUDA_TRY(cudaStreamSynchronize(st));
    Ctl c{};
    int rc = read_ctl(&c);
    if (rc) return rc;
    if (c.status) return c.status;
    if (last_mixed) {
        last_steps = c.steps;
        last_sweeps = c.inner_total;
        last_res = c.rel_res;
        if (last_cond) {
            // per outer iteration: residual, test, axpy; per inner pair: two sweeps + test
            launches += 3ll * (c.steps + 1) + c.inner_total + c.inner_total / 2;
            last_cond = false;
        }
        if (!c.done) return SPTRSV_ERR_NOT_CONVERGED;
    }
    return 0;
}

int Handle::set_matrix_host(int n_, int64_t nnz_, const int64_t* rp_h, const int* col_h, const double* val_h) {
    if (n_ <= 0 || nnz_ < n_ || !rp_h || !col_h || !val_h) return SPTRSV_ERR_INVALID_ARG;
    if (nnz_ > 0x7fffffffll) return SPTRSV_ERR_TOO_LARGE;
    drop_matrix();
    int rc;
    n = n_;
    nnz = (int)nnz_;
    if ((rc = own_rp.ensure(sizeof(int) * (size_t)(n + 1)))) return rc;
    if ((rc = own_col.ensure(sizeof(int) * (size_t)nnz))) return rc;
    if ((rc = own_val.ensure(sizeof(double) * (size_t)nnz))) return rc;
    if ((rc = scratch.ensure(sizeof(int64_t) * (size_t)(n + 1)))) return rc;
    CUDA_TRY(cudaMemcpyAsync(scratch.p, rp_h, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(own_col.p, col_h, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(own_val.p, val_h, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, st));
    if ((rc = reset_ctl())) return rc;
    k_narrow_rp<<<sm_count * 4, 256, 0, st>>>(n + 1, (const int64_t*)scratch.p, own_rp.as<int>(), ctl);
    ++launches;
    CUDA_TRY(cudaGetLastError());
    Ctl c{};
    if ((rc = read_ctl(&c))) return rc;
    if (c.status) return c.status;
    rp = own_rp.as<int>();
    col = own_col.as<int>();
    val = own_val.as<double>();
    return 0;
}

Handle::~Handle() {
    if (cancel_st) cudaStreamDestroy(cancel_st);
    if (cancel_flag) cudaFreeHost(cancel_flag);
    drop_graphs();
    for (cudaEvent_t e : prof_ev) cudaEventDestroy(e);
    if (prof0) cudaEventDestroy(prof0);
    DevBuf* bufs[] = {&own_rp, &own_col, &own_val, &val32, &invd, &invd32, &in_degree, &levels, &level_ptr,
                      &level_rows, &stats, &csc_ptr, &csc_row, &csc_val, &scratch, &xw, &bw, &r32, &d32a, &d32b,
                      &norms, &indeg_work, &left, &db, &dx, &flush, &offdiag, &roff, &jmeta, &jbase, &sell, &sell_perm, &sell_len, &sell_ptr,
                      &sn_start, &sn_m, &sn_roff, &sn_rect, &sn_goff, &sn_ld, &sn_colbase, &sn_outbase, &sn_items,
                      &sn_G, &sn_Ghi, &sn_Glo, &sn_pan, &sn_pitems, &sn_pcnt, &sn_ppart, &sn_gtc, &sn_tcrec, &sn_ghl, &sn_gexp, &tune_b, &tune_x};
    for (DevBuf* b : bufs) b->release();
    if (ctl) cudaFree(ctl);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (st) cudaStreamDestroy(st);
}

}  // namespace sptrsv

using sptrsv::Handle;

extern "C" {

void sptrsv_default_opts(sptrsv_opts* o) {
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->schedule = SPTRSV_SCHED_AUTO;
    o->precision = SPTRSV_PREC_FP64;
    o->rows_per_warp = 0;
    o->rhs_tile = 0;
    o->inner = SPTRSV_SCHED_AUTO;
    o->inner_sweeps = 0;
    o->max_refine = 8;
    o->tol = 1e-12;
    o->spin_budget_ns = sptrsv::kDefaultBudgetNs;
    o->resident_warps = 0;
    o->inner_tol_exp = 6;
}

const char* sptrsv_status_string(int s) {
    switch (s) {
        case SPTRSV_OK: return "ok";
        case SPTRSV_ERR_NOT_SQUARE: return "matrix is not square";
        case SPTRSV_ERR_INVALID_ARG: return "invalid argument";
        case SPTRSV_ERR_CUDA: return "CUDA runtime error";
        case SPTRSV_ERR_ROW_PTR: return "row pointer not monotone or not starting at 0";
        case SPTRSV_ERR_MISSING_DIAG: return "row empty or diagonal not its first entry";
        case SPTRSV_ERR_NOT_UPPER: return "entry at or left of the diagonal";
        case SPTRSV_ERR_COL_RANGE: return "column index out of range";
        case SPTRSV_ERR_ZERO_PIVOT: return "zero or non-finite diagonal";
        case SPTRSV_ERR_TIMEOUT: return "device wait exceeded its budget";
        case SPTRSV_ERR_NOT_CONVERGED: return "refinement did not reach the tolerance";
        case SPTRSV_ERR_TOO_LARGE: return "size above the supported maximum";
        case SPTRSV_ERR_NO_DEVICE: return "no CUDA device";
        case SPTRSV_ERR_NO_ANALYSIS: return "solve before analyse";
        case SPTRSV_ERR_SUPERNODES: return "supernode partition inconsistent with the matrix";
        case SPTRSV_ERR_UNSUPPORTED: return "unsupported combination of options";
        case SPTRSV_ERR_IO: return "file unreadable or malformed";
        default: return "unknown status";
    }
}

int sptrsv_last_status(void) { return sptrsv::t_last_status; }

int sptrsv_create(sptrsv_handle* out, int device) {
    if (!out) return SPTRSV_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        (void)cudaGetLastError();
        return SPTRSV_ERR_NO_DEVICE;
    }
    if (device < 0) CUDA_TRY(cudaGetDevice(&device));
    if (device >= count) return SPTRSV_ERR_INVALID_ARG;
    CUDA_TRY(cudaSetDevice(device));
    Handle* h = new Handle;
    h->device = device;
    int rc = 0;
    do {
        cudaError_t er;
        if ((er = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking)) != cudaSuccess) { rc = sptrsv::set_cuda_error(er, "stream"); break; }
        if ((er = cudaEventCreate(&h->ev0)) != cudaSuccess) { rc = sptrsv::set_cuda_error(er, "event"); break; }
        if ((er = cudaEventCreate(&h->ev1)) != cudaSuccess) { rc = sptrsv::set_cuda_error(er, "event"); break; }
        if ((er = cudaMalloc(&h->ctl, sizeof(sptrsv::Ctl))) != cudaSuccess) { rc = sptrsv::set_cuda_error(er, "ctl"); break; }
        // a new control block reports no status until a solve or analysis writes one
        if ((er = cudaMemsetAsync(h->ctl, 0, sizeof(sptrsv::Ctl), h->st)) != cudaSuccess ||
            (er = cudaStreamSynchronize(h->st)) != cudaSuccess) { rc = sptrsv::set_cuda_error(er, "ctl"); break; }
        if ((er = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) { rc = sptrsv::set_cuda_error(er, "attr"); break; }
    } while (0);
    if (rc) { delete h; return rc; }
    const char* g = getenv("SPTRSV_NO_GRAPH");
    h->use_graphs = !(g && g[0] == '1');
    // tuning override of the Jacobi sweep kernel (default: lane per row over entry pairs): jds,
    // batch8, batch4, direct, tile, tile8, direct2, tma, sell
    const char* sk = getenv("SPTRSV_SWEEP_KERNEL");
    h->sweep_kernel = 0;
    if (sk && strcmp(sk, "sell") == 0) h->sweep_kernel = 6;
    if (sk && strcmp(sk, "jds") == 0) h->sweep_kernel = 9;
    if (sk && strcmp(sk, "batch4") == 0) h->sweep_kernel = 7;
    if (sk && strcmp(sk, "batch8") == 0) h->sweep_kernel = 8;
    if (sk && strcmp(sk, "tile") == 0) h->sweep_kernel = 1;
    if (sk && strcmp(sk, "direct") == 0) h->sweep_kernel = 2;
    if (sk && strcmp(sk, "tile8") == 0) h->sweep_kernel = 3;
    if (sk && strcmp(sk, "direct2") == 0) h->sweep_kernel = 4;
    if (sk && strcmp(sk, "tma") == 0) h->sweep_kernel = 5;
    *out = reinterpret_cast<sptrsv_handle>(h);
    return 0;
}

int sptrsv_destroy(sptrsv_handle hh) {
    Handle* h = reinterpret_cast<Handle*>(hh);
    if (!h) return SPTRSV_ERR_INVALID_ARG;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->st);
    delete h;
    return 0;
}

#define H() Handle* h = reinterpret_cast<Handle*>(hh); if (!h) return SPTRSV_ERR_INVALID_ARG; \
    if (cudaSetDevice(h->device) != cudaSuccess) return SPTRSV_ERR_CUDA

int sptrsv_analyse_host(sptrsv_handle hh, int n, int64_t nnz, const int64_t* row_ptr, const int* col, const double* val) {
    H();
    int rc = h->set_matrix_host(n, nnz, row_ptr, col, val);
    if (rc) return rc;
    if ((rc = h->analyse())) return rc;
    return h->ensure_levels();
}

int sptrsv_analyse_device(sptrsv_handle hh, int n, int nnz, const int* d_row_ptr, const int* d_col, const double* d_val) {
    H();
    if (n <= 0 || nnz < n || !d_row_ptr || !d_col || !d_val) return SPTRSV_ERR_INVALID_ARG;
    h->drop_matrix();
    h->n = n;
    h->nnz = nnz;
    h->rp = d_row_ptr;
    h->col = d_col;
    h->val = d_val;
    int rc = h->analyse();
    if (rc) return rc;
    return h->ensure_levels();
}

int sptrsv_set_supernodes(sptrsv_handle hh, int sn, const int* supernodes) {
    H();
    return h->set_supernodes(sn, supernodes);
}

int sptrsv_info(sptrsv_handle hh, int* n, int* nnz, int* max_level) {
    H();
    if (!h->analysed) return SPTRSV_ERR_NO_ANALYSIS;
    int rc = h->ensure_levels();
    if (rc) return rc;
    if (n) *n = h->n;
    if (nnz) *nnz = h->nnz;
    if (max_level) *max_level = h->max_level;
    return 0;
}

__global__ void k_widen_u64(int n, const int* __restrict__ a, uint64_t* __restrict__ b) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = (uint64_t)a[i];
}

int sptrsv_get_levels(sptrsv_handle hh, uint64_t* levels) {
    H();
    if (!h->analysed) return SPTRSV_ERR_NO_ANALYSIS;
    if (int rc0 = h->ensure_levels()) return rc0;
    if (!levels) return SPTRSV_ERR_INVALID_ARG;
    int rc;
    if ((rc = h->scratch.ensure(sizeof(uint64_t) * (size_t)h->n))) return rc;
    k_widen_u64<<<h->sm_count * 4, 256, 0, h->st>>>(h->n, h->levels.as<int>(), (uint64_t*)h->scratch.p);
    h->launches++;
    CUDA_TRY(cudaMemcpyAsync(levels, h->scratch.p, sizeof(uint64_t) * (size_t)h->n, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    return 0;
}

int sptrsv_get_in_degree(sptrsv_handle hh, int* in_degree) {
    H();
    if (!h->analysed) return SPTRSV_ERR_NO_ANALYSIS;
    if (!in_degree) return SPTRSV_ERR_INVALID_ARG;
    CUDA_TRY(cudaMemcpyAsync(in_degree, h->in_degree.p, sizeof(int) * (size_t)h->n, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    return 0;
}

// The device CSC of U (utils.cpp:128-159 layout), built on first need, copied to host arrays
// of n+1, nnz and nnz entries; any of them may be NULL.
int sptrsv_get_csc(sptrsv_handle hh, int* col_ptr, int* row_idx, double* val) {
    H();
    if (!h->analysed) return SPTRSV_ERR_NO_ANALYSIS;
    if (int rc0 = h->build_csc()) return rc0;
    if (col_ptr)
        CUDA_TRY(cudaMemcpyAsync(col_ptr, h->csc_ptr.p, sizeof(int) * (size_t)(h->n + 1), cudaMemcpyDeviceToHost, h->st));
    if (row_idx)
        CUDA_TRY(cudaMemcpyAsync(row_idx, h->csc_row.p, sizeof(int) * (size_t)h->nnz, cudaMemcpyDeviceToHost, h->st));
    if (val) CUDA_TRY(cudaMemcpyAsync(val, h->csc_val.p, sizeof(double) * (size_t)h->nnz, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    return 0;
}

int sptrsv_get_level_buckets(sptrsv_handle hh, int* level_ptr, int* level_rows) {
    H();
    if (!h->analysed) return SPTRSV_ERR_NO_ANALYSIS;
    if (int rc0 = h->ensure_levels()) return rc0;
    if (level_ptr)
        CUDA_TRY(cudaMemcpyAsync(level_ptr, h->level_ptr.p, sizeof(int) * (size_t)(h->max_level + 2),
                                 cudaMemcpyDeviceToHost, h->st));
    if (level_rows)
        CUDA_TRY(cudaMemcpyAsync(level_rows, h->level_rows.p, sizeof(int) * (size_t)h->n, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    return 0;
}

int sptrsv_get_level_tasks(sptrsv_handle hh, int num_threads, int* tasks) {
    H();
    if (!h->analysed) return SPTRSV_ERR_NO_ANALYSIS;
    if (int rc0 = h->ensure_levels()) return rc0;
    if (num_threads < 1 || !tasks) return SPTRSV_ERR_INVALID_ARG;
    const size_t count = (size_t)(h->max_level + 1) * (num_threads + 1);
    int rc;
    if ((rc = h->scratch.ensure(sizeof(int) * count))) return rc;
    sptrsv::k_level_tasks<<<(h->max_level + 256) / 256, 256, 0, h->st>>>(
        h->max_level, h->level_ptr.as<int>(), h->level_rows.as<int>(), h->rp, num_threads, (int*)h->scratch.p);
    h->launches++;
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(tasks, h->scratch.p, sizeof(int) * count, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    return 0;
}

int sptrsv_solve(sptrsv_handle hh, const sptrsv_opts* o, const double* d_b, double* d_x, int rhs, int layout) {
    H();
    return h->solve(o, d_b, d_x, rhs, layout);
}

int sptrsv_solve_host(sptrsv_handle hh, const sptrsv_opts* o, const double* b, double* x, int rhs, int layout) {
    H();
    if (!h->analysed) return SPTRSV_ERR_NO_ANALYSIS;
    if (!b || !x || rhs < 1) return SPTRSV_ERR_INVALID_ARG;
    const size_t bytes = sizeof(double) * (size_t)h->n * rhs;
    int rc;
    if ((rc = h->db.ensure(bytes))) return rc;
    if ((rc = h->dx.ensure(bytes))) return rc;
    CUDA_TRY(cudaMemcpyAsync(h->db.p, b, bytes, cudaMemcpyHostToDevice, h->st));
    // Pinned (or registered) host x with one right-hand side: the refinement's FP64 residual
    // kernels, which read all of x anyway, write it straight to the host over the C2C link, so
    // the converged x needs no device-to-host copy after the last residual.
    h->x_mirror = nullptr;
    if (rhs == 1) {
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, x) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer)
            h->x_mirror = static_cast<double*>(pa.devicePointer);
        else
            (void)cudaGetLastError();
    }
    rc = h->solve(o, h->db.as<double>(), h->dx.as<double>(), rhs, layout);
    h->x_mirror = nullptr;
    if (rc) return rc;
    if (h->last_mirrored) {
        rc = h->sync();
        // complete when the solve converged after at least one residual of a nonzero x; a zero
        // right-hand side (x = 0 from the start) or an unconverged solve takes the copy below
        if (rc == 0 && h->last_steps >= 1) return 0;
        if (rc != 0 && rc != SPTRSV_ERR_NOT_CONVERGED) return rc;
        CUDA_TRY(cudaMemcpyAsync(x, h->dx.p, bytes, cudaMemcpyDeviceToHost, h->st));
        CUDA_TRY(cudaStreamSynchronize(h->st));
        return rc;
    }
    CUDA_TRY(cudaMemcpyAsync(x, h->dx.p, bytes, cudaMemcpyDeviceToHost, h->st));
    return h->sync();
}

int sptrsv_sync(sptrsv_handle hh) {
    H();
    return h->sync();
}

int sptrsv_last_refine(sptrsv_handle hh, int* steps, int* inner_sweeps, double* rel_residual) {
    H();
    if (steps) *steps = h->last_steps;
    if (inner_sweeps) *inner_sweeps = h->last_sweeps;
    if (rel_residual) *rel_residual = h->last_res;
    return 0;
}

int sptrsv_device_alloc(sptrsv_handle hh, size_t bytes, void** ptr) {
    H();
    if (!ptr) return SPTRSV_ERR_INVALID_ARG;
    CUDA_TRY(cudaMalloc(ptr, bytes ? bytes : 1));
    return 0;
}
int sptrsv_device_free(sptrsv_handle hh, void* ptr) {
    H();
    CUDA_TRY(cudaFree(ptr));
    return 0;
}
int sptrsv_host_alloc(sptrsv_handle hh, size_t bytes, void** ptr) {
    H();
    if (!ptr) return SPTRSV_ERR_INVALID_ARG;
    CUDA_TRY(cudaMallocHost(ptr, bytes ? bytes : 1));
    return 0;
}
int sptrsv_host_free(sptrsv_handle hh, void* ptr) {
    H();
    CUDA_TRY(cudaFreeHost(ptr));
    return 0;
}
int sptrsv_copy_h2d(sptrsv_handle hh, void* dst, const void* src, size_t bytes) {
    H();
    CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->st));
    return 0;
}
int sptrsv_copy_d2h(sptrsv_handle hh, void* dst, const void* src, size_t bytes) {
    H();
    CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->st));
    return 0;
}
int sptrsv_timer_begin(sptrsv_handle hh) {
    H();
    CUDA_TRY(cudaEventRecord(h->ev0, h->st));
    return 0;
}
int sptrsv_timer_end(sptrsv_handle hh, float* ms) {
    H();
    CUDA_TRY(cudaEventRecord(h->ev1, h->st));
    CUDA_TRY(cudaEventSynchronize(h->ev1));
    float t = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&t, h->ev0, h->ev1));
    if (ms) *ms = t;
    return 0;
}
int sptrsv_flush_l2(sptrsv_handle hh) {
    H();
    const size_t bytes = (size_t)512 << 20;
    int rc;
    if ((rc = h->flush.ensure(bytes))) return rc;
    CUDA_TRY(cudaMemsetAsync(h->flush.p, h->flush_byte++ & 0xff, bytes, h->st));
    return 0;
}
int64_t sptrsv_kernel_launches(sptrsv_handle hh) {
    Handle* h = reinterpret_cast<Handle*>(hh);
    return h ? h->launches : -1;
}
int sptrsv_profile_enable(sptrsv_handle hh, int enable) {
    H();
    h->profiling = enable != 0;
    return 0;
}

int sptrsv_profile_read(sptrsv_handle hh, int* kinds, float* ms, int cap) {
    H();
    if (!h->profiling || !h->prof0) return 0;
    CUDA_TRY(cudaStreamSynchronize(h->st));
    int n = std::min(cap, h->prof_n);
    cudaEvent_t prev = h->prof0;
    for (int i = 0; i < n; ++i) {
        float t = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&t, prev, h->prof_ev[i]));
        if (kinds) kinds[i] = h->prof_kind[i];
        if (ms) ms[i] = t;
        prev = h->prof_ev[i];
    }
    return n;
}

int sptrsv_device_sm_count(sptrsv_handle hh) {
    Handle* h = reinterpret_cast<Handle*>(hh);
    return h ? h->sm_count : -1;
}

}  // extern "C"
