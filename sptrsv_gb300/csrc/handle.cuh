// handle.cuh -- the state behind an sptrsv_handle: one device, one stream, one resident
// matrix with its analysis, grow-only work buffers and a small cache of solve graphs.
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>
#include "common.cuh"
#include "kernels.cuh"

namespace sptrsv {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes);
    void release();
    template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

// Relative residual the FP64 + JACOBI form refines to: an exact FP64 solve of the measured
// systems lands at 1e-16 - 2e-16.
constexpr double kFp64RefineTol = 1e-15;
// Mean row length from which FP64 solves of several column-major right-hand sides run the block
// sync-free kernel once per column rather than the RHS-tiled warp kernel (whose lanes walk a long
// row's entries one after another): on the 40^3 nested-dissection factor (385 entries per row)
// 114 ms against 1,558 ms at 8 RHS; on 8.6-entry rows the warp kernel stays 3.5x faster.
constexpr double kBlockPerColumnLen = 64.0;

// Rows per chunk of the partition prepare() builds for a skyline matrix: the widest chunk the
// supernodal solve takes.  A banded matrix's chunks form one dependency chain, and G = T^-1 [..]
// leaves no dependency inside a chunk, so wider chunks mean fewer hops (64 x 64 grid factor:
// 0.253 / 0.147 / 0.109 / 0.081 ms at 64 / 128 / 192 / 256 rows).
constexpr int kAutoChunkRows = 256;

struct GraphKey {
    sptrsv_opts o;
    const double* b;
    double* x;
    double* xo;  // host mirror of x written by the residual kernels (RefineArgs::x_out), or nullptr
    int rhs;
    int layout;
    int warps;
    bool prof;
    bool same(const GraphKey& k) const {
        return o.schedule == k.o.schedule && o.precision == k.o.precision && o.rows_per_warp == k.o.rows_per_warp &&
               o.rhs_tile == k.o.rhs_tile && o.inner == k.o.inner && o.inner_sweeps == k.o.inner_sweeps &&
               o.max_refine == k.o.max_refine && o.tol == k.o.tol && o.spin_budget_ns == k.o.spin_budget_ns &&
               o.resident_warps == k.o.resident_warps && o.inner_tol_exp == k.o.inner_tol_exp &&
               b == k.b && x == k.x && xo == k.xo && rhs == k.rhs && layout == k.layout && warps == k.warps && prof == k.prof;
    }
};

struct GraphEntry {
    GraphKey key;
    cudaGraphExec_t exec = nullptr;
    int64_t kernels = 0;
};

struct Handle {
    int device = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int sm_count = 0;
    int64_t launches = 0;
    Ctl* ctl = nullptr;
    bool use_graphs = true;
    int sweep_kernel = 0;   // 0 bulk-copy pipelined sweeps, 1 warp tiles with plain loads
    int warps_override = 0;

    // matrix (device; either owned copies or caller-owned pointers)
    int n = 0, nnz = 0;
    bool analysed = false;
    bool levels_ready = false;
    bool levelset_one_cta = false;  // the level-set solve's grid: one CTA (narrow levels) or the rows model
    const int* rp = nullptr;
    const int* col = nullptr;
    const double* val = nullptr;
    DevBuf own_rp, own_col, own_val;

    // analysis
    DevBuf val32, invd, invd32, in_degree, levels, level_ptr, level_rows, stats;
    int max_level = 0;
    double max_ratio = 0.0, mean_len = 0.0, std_len = 0.0;
    double depth_est = 0.0;  // analysis: sum over rows of 1 / (distance to the nearest dependency)
    bool skyline = false;    // analysis: every row is one contiguous column range from its diagonal
    bool auto_supernodes = false;  // the supernode partition was built by prepare(), not the caller
    // FP64 AUTO solves dense skyline matrices (rows of similar length, so the dense panels stay
    // about the size of the matrix) on exact FP64 panels over uniform chunks
    bool dense_skyline() const { return skyline && mean_len >= 16.0 && std_len <= 0.5 * mean_len; }
    // FP64 block sync-free solve of several column-major right-hand sides, one column at a time
    bool block_per_column(const sptrsv_opts& o, int rhs, int layout) const {
        if (o.precision != SPTRSV_PREC_FP64 || rhs <= 1 || layout != SPTRSV_COL_MAJOR) return false;
        return o.schedule == SPTRSV_SCHED_SYNCFREE_WINDOW ||
               (o.schedule == SPTRSV_SCHED_SYNCFREE_BLOCK && mean_len >= kBlockPerColumnLen);
    }
    DevBuf csc_ptr, csc_row, csc_val;
    bool have_csc = false;
    DevBuf offdiag;        // interleaved FP32 off-diagonals for the Jacobi sweeps
    DevBuf roff;           // per-row first off-diagonal slot, padded by kRoffPad
    bool off_pairs = false;  // offdiag/roff in the paired layout (rows padded to an even count)
    DevBuf jmeta;          // group-jagged layout: per 32-row group, lane R -> (row << 27) | count
    DevBuf jbase;          // group-jagged layout: first entry of every group (+ total, overflow flag)
    bool off_jds = false;  // offdiag holds the group-jagged entries
    DevBuf sell, sell_perm, sell_len, sell_ptr;  // SELL-32-256 copy of the off-diagonals
    int sell_nslices = 0;
    // supernode partition and its dense panels (supernodal.cu)
    DevBuf sn_start, sn_m, sn_roff, sn_rect, sn_goff, sn_ld, sn_colbase, sn_outbase, sn_items, sn_G, sn_Ghi, sn_Glo;
    int sn_count = 0, sn_nitems = 0;
    // the FP64 solve's 64-row panels split into column blocks (panels64.cu): panel records,
    // (panel, block) items, per-panel completion counters, partial sums (sn_prows per column)
    DevBuf sn_pan, sn_pitems, sn_pcnt, sn_ppart;
    DevBuf sn_gtc, sn_tcrec;  // tensor-core schedule: digit-slice G records of every panel block
    DevBuf sn_ghl, sn_gexp;   // double-FP32 schedule: G as scaled FP32 pairs, row exponents
    bool sn_tc = false;       // the records are built
    bool build_tc = true;     // set_supernodes builds them (off for the batch's scratch handle)
    int sn_npan = 0;
    unsigned sn_npitems = 0;
    long long sn_prows = 0;
    bool have_supernodes = false;
    bool have_offdiag = false;

    // work
    DevBuf scratch, xw, bw, r32, d32a, d32b, norms, indeg_work, left, db, dx, flush;
    unsigned flush_byte = 1;
    bool last_mixed = false;
    bool last_cond = false;       // the last solve ran the conditional (device-looped) graph
    double* x_mirror = nullptr;   // set by sptrsv_solve_host around solve(): pinned host x for the residuals
    bool last_mirrored = false;   // the last solve's residual kernels wrote x_mirror
    int64_t cond_fixed_kernels = 0;
    int last_steps = 0;
    int last_sweeps = 0;
    double last_res = 0.0;
    std::vector<GraphEntry> graphs;

    // per-launch profiling: an event after every kernel step of a solve (captured into the
    // graph as event-record nodes); durations are read after the solve completes
    bool profiling = false;
    cudaEvent_t prof0 = nullptr;
    std::vector<cudaEvent_t> prof_ev;
    std::vector<int> prof_kind;
    int prof_n = 0;
    int mark(int kind);

    ~Handle();
    int read_ctl(Ctl* out);
    int reset_ctl();
    void drop_graphs();
    void drop_matrix();
    int set_matrix_host(int n, int64_t nnz, const int64_t* rp, const int* col, const double* val);
    int analyse();
    int ensure_levels();
    int build_csc();
    sptrsv_opts resolve(const sptrsv_opts* o, int rhs) const;
    int prepare(const sptrsv_opts& o, int rhs, int layout);
    int enqueue(const sptrsv_opts& o, const double* b, double* x, int rhs, int layout);
    int ensure_offdiag();
    bool cond_eligible(const sptrsv_opts& o, int rhs) const;
    int refine_args(const sptrsv_opts& o, const double* b, double* x, int rhs, RefineArgs* ra);
    int build_cond_graph(const sptrsv_opts& o, const double* b, double* x, double* x_out, int rhs, int layout,
                         cudaGraphExec_t* out, int64_t* fixed_kernels);
    int resident_warps(const sptrsv_opts& o) const;
    int levelset_warps(const sptrsv_opts& o) const;
    int set_supernodes(int sn, const int* snodes_host);
    SnArgs sn_args() const;
    // autotuner state (tune.cu)
    DevBuf tune_b, tune_x;
    sptrsv_opts tuned[4];
    bool tuned_valid[4] = {false, false, false, false};
    bool applicable(const sptrsv_opts& o, int rhs) const;
    int autotune(int rhs, float cap_ms, int reps, float abort_ms, float* ms_out, int* censored_out, int* best_id);
    int timed_candidate(const sptrsv_opts& o, int rhs, float abort_ms, float* ms, bool* censored);
    int cancel_until_idle();
    cudaStream_t cancel_st = nullptr;
    int* cancel_flag = nullptr;  // pinned host 1
    int features(float* f, int rhs);
    int solve(const sptrsv_opts* o, const double* b, double* x, int rhs, int layout);
    int sync();
};

void set_last_status(int s);
int rhs_class(int rhs);
const sptrsv_opts* tune_candidates(int* count);
int launch_sn_solve(const Handle& h, bool mixed, const void* b, void* x, int rhs, int64_t budget, int64_t* launches);

}  // namespace sptrsv
