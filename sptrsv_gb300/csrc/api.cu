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
    if ((rc = stats.ensure(2 * sizeof(unsigned long long)))) return rc;
    const int sgrid = sm_count * 4;
    k_validate<<<sgrid, 256, 0, st>>>(n, nnz, rp, col, val, in_degree.as<int>(), invd.as<double>(),
                                      invd32.as<float>(), ctl);
    ++launches;
    CUDA_TRY(cudaGetLastError());
    if ((rc = read_ctl(&c))) return rc;
    if (c.status) return c.status;
    k_to_f32<<<sgrid, 256, 0, st>>>((size_t)nnz, val, val32.as<float>());
    CUDA_TRY(cudaMemsetAsync(stats.p, 0, 2 * sizeof(unsigned long long), st));
    k_row_stats<<<sgrid, 256, 0, st>>>(n, rp, val, stats.as<unsigned long long>(), stats.as<unsigned long long>() + 1);
    launches += 2;
    CUDA_TRY(cudaGetLastError());
    unsigned long long hs[2];
    CUDA_TRY(cudaMemcpyAsync(hs, stats.p, sizeof(hs), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    double mr;
    memcpy(&mr, &hs[0], sizeof(double));
    max_ratio = mr;
    mean_len = (double)nnz / n;
    const double ex2 = (double)hs[1] / n;
    std_len = std::sqrt(std::fmax(0.0, ex2 - mean_len * mean_len));
    analysed = true;
    return 0;
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
    k_levels<<<sm_count * 2, 256, 0, st>>>(n, rp, col, levels.as<int>(), ctl, kDefaultBudgetNs);
    ++launches;
    CUDA_TRY(cudaGetLastError());
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
    CUDA_TRY(cudaStreamSynchronize(st));
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

// Schedule choice from the analysis features (the autotuner overrides it).
sptrsv_opts Handle::resolve(const sptrsv_opts* o, int rhs) const {
    sptrsv_opts r;
    sptrsv_default_opts(&r);
    if (o) r = *o;
    if (r.spin_budget_ns <= 0) r.spin_budget_ns = kDefaultBudgetNs;
    if (r.tol <= 0) r.tol = 1e-12;
    if (r.max_refine <= 0) r.max_refine = 8;
    const double width = (double)n / (max_level > 0 ? max_level : 1);
    if (r.schedule == SPTRSV_SCHED_AUTO) {
        if (r.precision == SPTRSV_PREC_MIXED) {
            r.schedule = SPTRSV_SCHED_JACOBI;
        } else {
            r.schedule = (levels_ready && width >= 2048.0 && max_level <= 2000) ? SPTRSV_SCHED_LEVELSET
                                                                                  : SPTRSV_SCHED_SYNCFREE_WARP;
        }
    }
    if (r.precision == SPTRSV_PREC_MIXED) {
        if (r.schedule == SPTRSV_SCHED_JACOBI) {
            r.inner = SPTRSV_SCHED_JACOBI;
        } else {
            r.inner = r.schedule;
        }
        if (r.inner == SPTRSV_SCHED_JACOBI && max_ratio >= 1.0) r.inner = SPTRSV_SCHED_SYNCFREE_WARP;
        if (r.inner == SPTRSV_SCHED_SYNCFREE_CSC) r.inner = SPTRSV_SCHED_SYNCFREE_WARP;
        if (r.inner_sweeps <= 0) {
            // sweeps so that max_ratio^s <= 1e-6 (FP32 correction accuracy), clamped
            int s = 12;
            if (max_ratio > 0 && max_ratio < 1.0) s = (int)std::ceil(std::log(1e-6) / std::log(max_ratio));
            r.inner_sweeps = std::max(2, std::min(s, 64));
        }
    }
    if (r.rows_per_warp <= 0) {
        const double m = mean_len;
        r.rows_per_warp = m <= 6 ? 8 : (m <= 12 ? 4 : (m <= 24 ? 2 : 1));
    }
    (void)rhs;
    return r;
}

int Handle::prepare(const sptrsv_opts& o, int rhs, int layout) {
    int rc;
    if (o.schedule == SPTRSV_SCHED_LEVELSET || (o.precision == SPTRSV_PREC_MIXED && o.inner == SPTRSV_SCHED_LEVELSET))
        if ((rc = ensure_levels())) return rc;
    const size_t nr = (size_t)n * rhs;
    if (rhs > 1 && layout == SPTRSV_COL_MAJOR) {
        if ((rc = bw.ensure(sizeof(double) * nr))) return rc;
        if ((rc = xw.ensure(sizeof(double) * nr))) return rc;
    }
    if (o.precision == SPTRSV_PREC_MIXED) {
        if ((rc = r32.ensure(sizeof(float) * nr))) return rc;
        if ((rc = d32a.ensure(sizeof(float) * nr))) return rc;
        if ((rc = d32b.ensure(sizeof(float) * nr))) return rc;
        if ((rc = norms.ensure(sizeof(double) * 2 * (size_t)rhs))) return rc;
    }
    if (o.schedule == SPTRSV_SCHED_SYNCFREE_CSC && o.precision == SPTRSV_PREC_FP64) {
        if ((rc = build_csc())) return rc;
        if ((rc = indeg_work.ensure(sizeof(int) * (size_t)n))) return rc;
        if ((rc = left.ensure(sizeof(double) * nr))) return rc;
    }
    return 0;
}

// Only stream work (captured into a graph).
int Handle::enqueue(const sptrsv_opts& o, const double* b, double* x, int rhs, int layout) {
    int rc;
    const double* brm = b;
    double* xrm = x;
    const bool conv = rhs > 1 && layout == SPTRSV_COL_MAJOR;
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
    a.warps = warps_override;
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
            case SPTRSV_SCHED_SYNCFREE_CSC:
                CUDA_TRY(cudaMemcpyAsync(indeg_work.p, in_degree.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, st));
                CUDA_TRY(cudaMemsetAsync(left.p, 0, sizeof(double) * (size_t)n * rhs, st));
                if ((rc = launch_push_csc(a, csc_ptr.as<int>(), csc_row.as<int>(), csc_val.as<double>(),
                                          indeg_work.as<int>(), left.as<double>())))
                    return rc;
                if ((rc = mark(SPTRSV_K_PUSH_CSC))) return rc;
                break;
            case SPTRSV_SCHED_LEVELSET:
                if ((rc = launch_levelset(false, a, max_level, level_ptr.as<int>(), level_rows.as<int>()))) return rc;
                if ((rc = mark(SPTRSV_K_LEVELSET))) return rc;
                break;
            default:
                return SPTRSV_ERR_UNSUPPORTED;
        }
    } else {
        RefineArgs ra{};
        ra.n = n;
        ra.nnz = nnz;
        ra.rhs = rhs;
        ra.rp = rp;
        ra.col = col;
        ra.val = val;
        ra.val32 = val32.as<float>();
        ra.invd = invd.as<double>();
        ra.invd32 = invd32.as<float>();
        ra.b = brm;
        ra.x = xrm;
        ra.r32 = r32.as<float>();
        ra.d32[0] = d32a.as<float>();
        ra.d32[1] = d32b.as<float>();
        ra.rn2 = norms.as<double>();
        ra.bn2 = norms.as<double>() + rhs;
        ra.ctl = ctl;
        ra.tol = o.tol;
        ra.budget = o.spin_budget_ns;
        ra.sm_count = sm_count;
        ra.st = st;
        ra.launches = &launches;
        const bool jac = o.inner == SPTRSV_SCHED_JACOBI;
        if ((rc = launch_refine_init(ra))) return rc;
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
                        if ((rc = launch_jacobi_sweep(ra, src, q == o.inner_sweeps - 1))) return rc;
                        if ((rc = mark(SPTRSV_K_JACOBI))) return rc;
                        src ^= 1;
                    }
                }
            } else {
                if ((rc = launch_exact_inner(ra, o.inner, o.rows_per_warp, 0, max_level, level_ptr.as<int>(),
                                             level_rows.as<int>())))
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

int Handle::solve(const sptrsv_opts* o_in, const double* b, double* x, int rhs, int layout) {
    if (!analysed) return SPTRSV_ERR_NO_ANALYSIS;
    if (rhs < 1 || !b || !x || (layout != SPTRSV_COL_MAJOR && layout != SPTRSV_ROW_MAJOR)) return SPTRSV_ERR_INVALID_ARG;
    if ((size_t)n * rhs > (size_t)0x7fffffff) return SPTRSV_ERR_TOO_LARGE;
    sptrsv_opts o = resolve(o_in, rhs);
    if (o.precision == SPTRSV_PREC_MIXED && rhs > 1024) return SPTRSV_ERR_UNSUPPORTED;
    int rc;
    if ((rc = prepare(o, rhs, layout))) return rc;
    last_mixed = o.precision == SPTRSV_PREC_MIXED;
    // profiled solves launch directly: their per-step events are timed from the host stream
    if (!use_graphs || profiling) return enqueue(o, b, x, rhs, layout);
    GraphKey key;
    key.o = o;
    key.b = b;
    key.x = x;
    key.rhs = rhs;
    key.layout = layout;
    key.warps = warps_override;
    key.prof = profiling;
    for (auto& g : graphs) {
        if (g.key.same(key)) {
            CUDA_TRY(cudaGraphLaunch(g.exec, st));
            launches += g.kernels;
            return 0;
        }
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
        last_res = c.rel_res;
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
    drop_graphs();
    for (cudaEvent_t e : prof_ev) cudaEventDestroy(e);
    if (prof0) cudaEventDestroy(prof0);
    DevBuf* bufs[] = {&own_rp, &own_col, &own_val, &val32, &invd, &invd32, &in_degree, &levels, &level_ptr,
                      &level_rows, &stats, &csc_ptr, &csc_row, &csc_val, &scratch, &xw, &bw, &r32, &d32a, &d32b,
                      &norms, &indeg_work, &left, &db, &dx, &flush};
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
        if ((er = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) { rc = sptrsv::set_cuda_error(er, "attr"); break; }
    } while (0);
    if (rc) { delete h; return rc; }
    const char* g = getenv("SPTRSV_NO_GRAPH");
    h->use_graphs = !(g && g[0] == '1');
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
    if ((rc = h->solve(o, h->db.as<double>(), h->dx.as<double>(), rhs, layout))) return rc;
    CUDA_TRY(cudaMemcpyAsync(x, h->dx.p, bytes, cudaMemcpyDeviceToHost, h->st));
    return h->sync();
}

int sptrsv_sync(sptrsv_handle hh) {
    H();
    return h->sync();
}

int sptrsv_last_refine(sptrsv_handle hh, int* steps, double* rel_residual) {
    H();
    if (steps) *steps = h->last_steps;
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
