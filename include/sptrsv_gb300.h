/*
 * sptrsv_gb300.h -- C ABI of the GB300 sparse upper-triangular solver.
 *
 * Plain C types only (no CUDA or torch types), so that ctypes, cgo, JNI or any C caller can
 * bind it.  Two layers:
 *   1. the reference's own entry points, re-implemented on the GPU with identical C++
 *      signatures: include/core.h and include/sptrsv_syncfree_opencl.h;
 *   2. the handle API below, which keeps one matrix and its analysis resident on the
 *      device, solves many right-hand sides against it, and exposes the schedules.
 *
 * Matrix convention (the reference's, core.cpp:18-32): CSR of an upper-triangular U, the
 * diagonal FIRST in every row, every other column index in (i, n).  Values FP64.
 * Errors: every function returns an sptrsv_status (0 = success, negative = failure); the
 * reference-signature functions return the negative status cast to double instead of
 * their elapsed seconds, and never exit the process.
 */
#ifndef SPTRSV_GB300_H
#define SPTRSV_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifndef SPTRSV_API
#define SPTRSV_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  -1 keeps the reference's "not a square matrix" return
 * (sptrsv_syncfree_opencl.cpp:17-21). */
enum sptrsv_status {
    SPTRSV_OK = 0,
    SPTRSV_ERR_NOT_SQUARE = -1,
    SPTRSV_ERR_INVALID_ARG = -2,
    SPTRSV_ERR_CUDA = -3,
    SPTRSV_ERR_ROW_PTR = -4,        /* row pointer not monotone, or does not start at 0 */
    SPTRSV_ERR_MISSING_DIAG = -5,   /* a row is empty or its first entry is not the diagonal */
    SPTRSV_ERR_NOT_UPPER = -6,      /* an off-diagonal entry at or left of the diagonal */
    SPTRSV_ERR_COL_RANGE = -7,      /* a column index >= n */
    SPTRSV_ERR_ZERO_PIVOT = -8,     /* a zero or non-finite diagonal */
    SPTRSV_ERR_TIMEOUT = -9,        /* a device wait ran out of its budget */
    SPTRSV_ERR_NOT_CONVERGED = -10, /* refinement stopped above its tolerance */
    SPTRSV_ERR_TOO_LARGE = -11,     /* nnz >= 2^31 or a size above a fixed maximum */
    SPTRSV_ERR_NO_DEVICE = -12,
    SPTRSV_ERR_NO_ANALYSIS = -13,   /* solve before analyse */
    SPTRSV_ERR_SUPERNODES = -14,    /* supernode partition inconsistent with the matrix */
    SPTRSV_ERR_UNSUPPORTED = -15,
    SPTRSV_ERR_IO = -16
};

/* Solve schedules (kernel families). */
enum sptrsv_schedule {
    SPTRSV_SCHED_AUTO = 0,          /* pick from the matrix features */
    SPTRSV_SCHED_SYNCFREE_WARP = 1, /* CSR pull, warps per row, self-flagging x, bounded spins */
    SPTRSV_SCHED_SYNCFREE_THREAD = 2, /* CSR pull, one lane per row (kernel_full3.cl family) */
    SPTRSV_SCHED_SYNCFREE_CSC = 3,  /* CSC push with per-row in-degree counters (kernel_full.cl family) */
    SPTRSV_SCHED_LEVELSET = 4,      /* persistent kernel, one grid barrier per level */
    SPTRSV_SCHED_JACOBI = 5,        /* iterative FP32 sweeps x <- D^-1 (b - N x) inside FP64 refinement; with
                                       SPTRSV_PREC_FP64 the refinement runs to a relative residual of
                                       min(tol, 1e-15), the accuracy of the exact FP64 schedules */
    SPTRSV_SCHED_SUPERNODAL = 6,    /* dense supernode blocks on tensor cores */
    SPTRSV_SCHED_SYNCFREE_BLOCK = 7, /* CSR pull, 512-row blocks per CTA with their x in shared memory */
    SPTRSV_SCHED_SYNCFREE_WINDOW = 8 /* CSR pull by one CTA walking 32-row blocks, recent x in a shared-memory
                                        ring (one RHS; column-major RHS one column at a time) */
};

enum sptrsv_precision {
    SPTRSV_PREC_FP64 = 0,   /* direct FP64 solve */
    SPTRSV_PREC_MIXED = 1   /* FP32 inner solves + FP64 residual / update (iterative refinement) */
};

enum sptrsv_layout {
    SPTRSV_COL_MAJOR = 0,   /* x[i + r*n]  (core.h solvers, core.cpp:26-28) */
    SPTRSV_ROW_MAJOR = 1    /* x[i*rhs + r] (sptrsv_syncfree_opencl, kernel_full.cl:163) */
};

/* Kernel steps reported by sptrsv_profile_read. */
enum sptrsv_kernel_kind {
    SPTRSV_K_FILL = 1,         /* x <- pending sentinel */
    SPTRSV_K_PULL_WARP = 2,    /* sync-free CSR pull, warps per row */
    SPTRSV_K_PULL_THREAD = 3,  /* sync-free CSR pull, one lane per row */
    SPTRSV_K_PUSH_CSC = 4,     /* sync-free CSC push */
    SPTRSV_K_LEVELSET = 5,     /* persistent level-set kernel */
    SPTRSV_K_INIT = 6,         /* refinement set-up (x = 0, ||b||) */
    SPTRSV_K_RESIDUAL = 7,     /* r = b - U x in FP64 */
    SPTRSV_K_CHECK = 8,        /* convergence test */
    SPTRSV_K_JACOBI = 9,       /* FP32 Jacobi sweep */
    SPTRSV_K_INNER = 10,       /* exact FP32 inner solve */
    SPTRSV_K_AXPY = 11,        /* x += d */
    SPTRSV_K_TRANSPOSE = 12,   /* column-major <-> row-major */
    SPTRSV_K_PULL_BLOCK = 13,  /* sync-free CSR pull, shared-memory blocks */
    SPTRSV_K_SUPERNODAL = 14,  /* supernode panel products (FP64, or BF16x3 tensor cores) */
    SPTRSV_K_WINDOW = 15       /* sync-free CSR pull by one CTA over a shared-memory ring */
};

typedef struct sptrsv_opts {
    int schedule;           /* enum sptrsv_schedule */
    int precision;          /* enum sptrsv_precision */
    int rows_per_warp;      /* SYNCFREE_WARP: 1, 2, 4, 8 (lanes per row = 32 / rows_per_warp) */
    int rhs_tile;           /* columns handled per warp pass (0 = min(rhs, 32)) */
    int inner;              /* MIXED: inner FP32 schedule (enum sptrsv_schedule) */
    int inner_sweeps;       /* MIXED + JACOBI: sweeps per step in unlooped (profiled / graph-less)
                               solves; device-looped solves stop on the change test (cap 200) */
    int max_refine;         /* MIXED: maximum refinement steps */
    double tol;             /* MIXED: target ||b - U x||_2 / ||b||_2 */
    int64_t spin_budget_ns; /* per-wait limit of every device spin (0 = 2 s) */
    int resident_warps;     /* sync-free kernels: warps launched (0 = chosen from the level width) */
    int inner_tol_exp;      /* MIXED + JACOBI: inner sweeps stop when max|change| <= eps max|d|, eps =
                               max(10^-e, 0.1 tol / last relative residual) (0: e = 6) */
} sptrsv_opts;

typedef struct sptrsv_ctx* sptrsv_handle;

/* Fill *o with the defaults (AUTO schedule, FP64, tol 1e-12, 2 s spin budget). */
SPTRSV_API void sptrsv_default_opts(sptrsv_opts* o);
SPTRSV_API const char* sptrsv_status_string(int status);
/* Status of the last reference-signature call made on this host thread. */
SPTRSV_API int sptrsv_last_status(void);

SPTRSV_API int sptrsv_create(sptrsv_handle* out, int device);
SPTRSV_API int sptrsv_destroy(sptrsv_handle h);

/* Upload a host CSR (int64 row pointer) and analyse it: validation, in-degree, levels,
 * level buckets, FP32 copy and reciprocal diagonal.  Replaces the setup and analyser
 * stages of sptrsv_syncfree_opencl.cpp:96-267. */
SPTRSV_API int sptrsv_analyse_host(sptrsv_handle h, int n, int64_t nnz, const int64_t* row_ptr, const int* col,
                        const double* val);
/* Same on caller-owned device arrays (int32 row pointer); the handle keeps the pointers. */
SPTRSV_API int sptrsv_analyse_device(sptrsv_handle h, int n, int nnz, const int* d_row_ptr, const int* d_col,
                          const double* d_val);

/* Supernode partition of the analysed matrix (host array of sn+1 row boundaries, 0 ... n), as in
 * supernodal_upper (core.h:12, core.cpp:80-92): every row of a supernode holds the dense upper
 * triangle of the supernode followed by one column set shared by the whole supernode.  Builds
 * the dense panels [T^-1 | -T^-1 Rect] (FP64 and BF16 hi/lo) for SPTRSV_SCHED_SUPERNODAL; AUTO then
 * picks that schedule.  SPTRSV_ERR_SUPERNODES when the matrix does not have the layout. */
SPTRSV_API int sptrsv_set_supernodes(sptrsv_handle h, int sn, const int* supernodes);

/* Autotuner: times every applicable candidate schedule (table indices 0 .. SPTRSV_TUNE_CANDIDATES-1,
 * see sptrsv_candidate) on the resident matrix with a seeded random right-hand side of `rhs`
 * columns (device buffers, CUDA events), each run capped at cap_ms after its first run and
 * repeated `reps` times otherwise; writes every candidate's best time in ms (INFINITY when not
 * applicable or failed) to cand_ms[SPTRSV_TUNE_CANDIDATES], the winner's index and options, and
 * caches the winner for the RHS class (1, 2-8, 9-32, >32), where SPTRSV_SCHED_AUTO uses it. */
#define SPTRSV_TUNE_CANDIDATES 16
#define SPTRSV_FEATURES 24
SPTRSV_API int sptrsv_autotune(sptrsv_handle h, int rhs, float cap_ms, int reps, float* cand_ms, int* best_id,
                               sptrsv_opts* best);
/* As sptrsv_autotune, and once one candidate has finished, a later one still running after
 * max(abort_ms, 20 x the best time so far) is cancelled (its spins see the abort flag and
 * return): its time is then a lower bound and censored[id] = 1.  abort_ms = 0 never cancels. */
SPTRSV_API int sptrsv_autotune_bounded(sptrsv_handle h, int rhs, float cap_ms, int reps, float abort_ms,
                                       float* cand_ms, int* censored, int* best_id, sptrsv_opts* best);
/* Options of candidate `id` of the autotuner's table. */
SPTRSV_API int sptrsv_candidate(int id, sptrsv_opts* o);
/* 1 when candidate `id` can run on the resident matrix with `rhs` columns. */
SPTRSV_API int sptrsv_candidate_applicable(sptrsv_handle h, int id, int rhs);
/* The SPTRSV_FEATURES features the learned selector reads: the resident matrix's (sizes
 * log2-scaled, level-width and supernode-width histograms, row-length moments, dominance) and
 * log2(rhs) last. */
SPTRSV_API int sptrsv_features(sptrsv_handle h, int rhs, float* features);
/* Cache a schedule for the RHS class of `rhs` (what the selector does with its pick). */
SPTRSV_API int sptrsv_set_tuned(sptrsv_handle h, int rhs, const sptrsv_opts* o);

/* Analysis results copied to host memory. */
SPTRSV_API int sptrsv_info(sptrsv_handle h, int* n, int* nnz, int* max_level);
SPTRSV_API int sptrsv_get_levels(sptrsv_handle h, uint64_t* levels);       /* core.cpp:244-270 values */
SPTRSV_API int sptrsv_get_in_degree(sptrsv_handle h, int* in_degree);      /* kernel_full.cl:40-52 values */
SPTRSV_API int sptrsv_get_level_buckets(sptrsv_handle h, int* level_ptr, int* level_rows); /* core.cpp:282-288 */
SPTRSV_API int sptrsv_get_level_tasks(sptrsv_handle h, int num_threads, int* tasks);      /* core.cpp:289-332 */
/* CSR -> CSC of U as utils.cpp:128-159 lays it out (column pointer, rows ascending within a column so
 * the diagonal is last, values), built on the device; host arrays of n+1 / nnz / nnz, any may be NULL. */
SPTRSV_API int sptrsv_get_csc(sptrsv_handle h, int* col_ptr, int* row_idx, double* val);

/* Solve U X = B with device-resident B and X (rhs columns, layout enum sptrsv_layout),
 * enqueued on the handle's stream.  Returns after the enqueue; the device status is read by
 * sptrsv_sync. */
SPTRSV_API int sptrsv_solve(sptrsv_handle h, const sptrsv_opts* o, const double* d_b, double* d_x, int rhs, int layout);
/* Same with host B and X: H2D, solve, D2H on the handle's stream, then synchronise. */
SPTRSV_API int sptrsv_solve_host(sptrsv_handle h, const sptrsv_opts* o, const double* b, double* x, int rhs, int layout);
/* Wait for the handle's stream; returns the first device error of the enqueued work. */
SPTRSV_API int sptrsv_sync(sptrsv_handle h);
/* Refinement steps, total inner Jacobi sweeps and final relative residual of the last MIXED
 * solve (valid after sptrsv_sync or a host-buffer solve). */
SPTRSV_API int sptrsv_last_refine(sptrsv_handle h, int* steps, int* inner_sweeps, double* rel_residual);

/* Device and pinned-host memory, copies and timing on the handle's stream. */
SPTRSV_API int sptrsv_device_alloc(sptrsv_handle h, size_t bytes, void** ptr);
SPTRSV_API int sptrsv_device_free(sptrsv_handle h, void* ptr);
SPTRSV_API int sptrsv_host_alloc(sptrsv_handle h, size_t bytes, void** ptr); /* pinned */
SPTRSV_API int sptrsv_host_free(sptrsv_handle h, void* ptr);
SPTRSV_API int sptrsv_copy_h2d(sptrsv_handle h, void* dst, const void* src, size_t bytes);
SPTRSV_API int sptrsv_copy_d2h(sptrsv_handle h, void* dst, const void* src, size_t bytes);
SPTRSV_API int sptrsv_timer_begin(sptrsv_handle h);
SPTRSV_API int sptrsv_timer_end(sptrsv_handle h, float* ms);     /* synchronises */
SPTRSV_API int sptrsv_flush_l2(sptrsv_handle h);                 /* writes 512 MiB of scratch */
SPTRSV_API int64_t sptrsv_kernel_launches(sptrsv_handle h);      /* kernels this handle has launched */
SPTRSV_API int sptrsv_device_sm_count(sptrsv_handle h);
/* No counterpart in the reference: the FP64 pipe of `device`, measured -- fused multiply-adds per
 * second over every SM (independent chains, CUDA events) and SM cycles per dependent FMA (one
 * chain, clock64).  The first bounds the FP64 kernels' throughput, the second every dependency
 * hop of an exact FP64 solve.  Allocates a few bytes of scratch; synchronises the device. */
SPTRSV_API int sptrsv_measure_fp64(int device, double* gfma_per_s, double* dep_fma_cycles);
/* No counterpart in the reference: the panel products of the exact FP64 supernodal and batched
 * schedules -- 0 = FP64 FMAs (the default), 1 = the tensor cores (tcgen05: BF16 digit slices of
 * G and of the right-hand side, exact FP32 accumulation in TMEM, FP64 combination; FP64-accurate),
 * 2 = double-FP32 on the FP32 pipes (G and the right-hand side as scaled FP32 pairs, error-free
 * products and compensated sums; FP64-accurate).  Applies to partitions and batches built
 * afterwards; returns the previous mode. */
SPTRSV_API int sptrsv_set_panels_mode(int mode);

/* No counterpart in the reference, whose factors come from an external sparse Cholesky: the step
 * upstream of the solve, a multifrontal supernodal Cholesky A = U^T U of a symmetric positive
 * definite n x n matrix on the GPU.  A is host CSR (int64 row pointer) already in the elimination
 * order; every row must hold its entries at and right of the diagonal (a full symmetric pattern
 * or the upper triangle).  The elimination is given as nf fronts in a postorder: front t pivots
 * rows front_start[t] .. front_start[t+1]-1 (the ranges tile 0 .. n-1 in order) and hands its
 * update matrix to front_parent[t] > t (-1 for a root).  The host finds every front's row set;
 * the GPU assembles each front (A's entries, its children's update matrices), factors its pivot
 * columns and forms its update matrix in FP64 (blocked in 64-column panels), every front of one
 * tree height in the same launches.  Trailing updates with at least 256 rows go to the tensor
 * cores as FP64-accurate BF16 digit products (environment SPTRSV_FACTOR_UPDATE=fp64: FP64 FMAs).  On success *factor holds U on the device in the solver's CSR
 * layout (diagonal first, columns ascending), its row pointer on the host, and the supernode
 * partition: each front's pivots in pieces of at most max_width rows, each piece a dense triangle
 * plus one shared set of columns, as sptrsv_set_supernodes takes it.  SPTRSV_ERR_ZERO_PIVOT when a
 * pivot is not positive (A not positive definite); SPTRSV_ERR_INVALID_ARG for a tree whose
 * updates reach rows no later front pivots. */
SPTRSV_API int sptrsv_factor_multifrontal(int device, int n, const int64_t* a_row_ptr, const int* a_col,
                                          const double* a_val, int nf, const int* front_start,
                                          const int* front_parent, int max_width, void** factor);
/* Sizes of a factor: n, entries of U, supernodes. */
SPTRSV_API int sptrsv_factor_info(void* factor, int* n, int64_t* nnz, int* num_supernodes);
/* Copies U (row_ptr[n+1], col[nnz], val[nnz]) and the partition (supernodes[num_supernodes+1]);
 * any pointer may be NULL.  U lives on the device: col and val are copied from there. */
SPTRSV_API int sptrsv_factor_copy(void* factor, int64_t* row_ptr, int* col, double* val, int* supernodes);
/* U where the factor keeps it on its device: int32 row pointer, columns, values, valid until
 * sptrsv_factor_free -- what sptrsv_analyse_device takes, so the solve can follow the factor
 * without a trip through host memory.  SPTRSV_ERR_TOO_LARGE when U has 2^31 entries or more. */
SPTRSV_API int sptrsv_factor_device(void* factor, const int** d_row_ptr, const int** d_col, const double** d_val);
/* Host wall time of the factor's two steps in seconds: the symbolic step on the host and the
 * numeric step on the GPU (uploads, every front's kernels, the copy of U back); either may be NULL. */
SPTRSV_API int sptrsv_factor_times(void* factor, double* symbolic_s, double* numeric_s);
SPTRSV_API void sptrsv_factor_free(void* factor);
/* Largest n accepted by sptrsv_solve_noalloc (its reciprocal diagonal lives in a fixed array). */
#define SPTRSV_NOALLOC_MAX_ROWS (1 << 20)

/* No counterpart in the reference.  The FP64 sync-free warp solve of U x = b (one RHS) for
 * callers that cannot allocate device memory: programs that give the whole GPU to their own
 * memory pool and forbid any other allocation, and latency-critical loops that cannot pay for
 * cudaMalloc / cudaFree (which synchronise the device and may fail at run time).  The caller
 * passes device arrays only -- CSR of U with an int32 row pointer and the diagonal first in
 * every row, b and x -- and an optional stream (NULL = the legacy default stream).  No memory
 * is allocated: the spin control block and the reciprocal diagonal live in one fixed device
 * array of SPTRSV_NOALLOC_MAX_ROWS * 8 + 256 bytes that every GPU loading this library holds
 * until the process exits.  n above SPTRSV_NOALLOC_MAX_ROWS returns SPTRSV_ERR_TOO_LARGE.
 * The matrix is checked first (same statuses as sptrsv_analyse_*).  The call is synchronous: it
 * returns the solve's status after the stream has drained, so it cannot be captured into a CUDA
 * graph.  All calls in a process share the array and each rewrites it: the
 * library holds one lock for the whole of each call, so calls made from several host threads
 * run one after another whatever stream they name.  The array keeps the last call's contents;
 * each call clears what must start at zero. */
SPTRSV_API int sptrsv_solve_noalloc(int n, int nnz, const int* d_row_ptr, const int* d_col, const double* d_val,
                                    const double* d_b, double* d_x, void* stream);

/* Record a CUDA event after every kernel step of later solves (also inside their graphs). */
SPTRSV_API int sptrsv_profile_enable(sptrsv_handle h, int enable);
/* After a profiled solve: per-step kinds (enum sptrsv_kernel_kind) and device times in ms, in
 * launch order; returns the number of steps written (at most cap).  Synchronises. */
SPTRSV_API int sptrsv_profile_read(sptrsv_handle h, int* kinds, float* ms, int cap);

/* ---------------------------------------------------------------------------------------
 * Batched systems (no counterpart in the reference, which solves one system per call):
 * `count` independent upper-triangular systems of uneven n and RHS count in one packed arena.
 * Host input: n[s], rhs[s]; row_ptr = each system's local row pointer (n[s]+1 entries starting at
 * 0) one after another; col (indices local to the system) and val likewise.  The same CSR rules
 * as sptrsv_analyse_host apply per system.  Right-hand sides and solutions are row-major
 * n[s] x rhs[s] per system, one system after another (sum n[s] rhs[s] doubles).
 * Schedules per system: SPTRSV_BATCH_PLAIN (exact FP64 sync-free), _JACOBI (FP32 Jacobi inside
 * the FP64 refinement), _PANEL (BF16x3 tensor-core dense 64-row panels inside the refinement;
 * rows must form skyline or supernode chunks), _SF32 (FP32 sync-free inside the refinement),
 * _PANEL64 (exact FP64 on the same dense panels, each panel's product split over CTAs).
 * Mode 0 solves every system with the plain FP64 schedule in one persistent launch; mode 1
 * solves each with its own schedule (set_schedule; the default comes from the analysis), the
 * mixed ones until ||b - U x||_F <= tol ||b||_F per system. */
typedef struct sptrsv_batch_s* sptrsv_batch;
#define SPTRSV_BATCH_PLAIN 0
#define SPTRSV_BATCH_JACOBI 1
#define SPTRSV_BATCH_PANEL 2
#define SPTRSV_BATCH_SF32 3
#define SPTRSV_BATCH_PANEL64 4
SPTRSV_API int sptrsv_batch_create(sptrsv_batch* out, int device, int count, const int* n, const int* rhs,
                                   const int64_t* row_ptr, const int* col, const double* val);
SPTRSV_API int sptrsv_batch_destroy(sptrsv_batch b);
SPTRSV_API int sptrsv_batch_get_schedule(sptrsv_batch b, int* sched);
/* sched[s] = -1 keeps system s's schedule; PANEL on a system without panel structure returns
 * SPTRSV_ERR_SUPERNODES, JACOBI on one without row dominance SPTRSV_ERR_UNSUPPORTED. */
SPTRSV_API int sptrsv_batch_set_schedule(sptrsv_batch b, const int* sched);
/* tol (default 1e-12), max refinement steps (20), inner change-test exponent (6), wait budget. */
SPTRSV_API int sptrsv_batch_set_options(sptrsv_batch b, double tol, int max_refine, int inner_tol_exp,
                                        int64_t spin_budget_ns);
/* Device arena vectors; enqueued on the batch's stream (one CUDA graph launch). */
SPTRSV_API int sptrsv_batch_solve(sptrsv_batch b, int mode, const double* d_b, double* d_x);
/* Host vectors (pinned for overlap): host->device copy, solve, device->host copy, enqueued. */
SPTRSV_API int sptrsv_batch_solve_host(sptrsv_batch b, int mode, const double* h_b, double* h_x);
/* Waits; returns the first error; *kernels = kernel launches of the last solve. */
SPTRSV_API int sptrsv_batch_sync(sptrsv_batch b, int64_t* kernels);
/* Per system, of the last chosen-mode solve: status, refinement steps, relative residual, sweeps. */
SPTRSV_API int sptrsv_batch_stats(sptrsv_batch b, int* status, int* steps, double* rel_res, int* sweeps);
/* totals[6] = {sum n, sum nnz, sum n*rhs, count, G entries of the exact FP64 panels, their FMAs
 * per solve} (the schedules' work lists are built first); ratio[s] = max row sum|off|/|diag|. */
SPTRSV_API int sptrsv_batch_info(sptrsv_batch b, int64_t* totals, float* ratio);
/* The selector's SPTRSV_FEATURES features of system s (with its own rhs). */
SPTRSV_API int sptrsv_batch_features(sptrsv_batch b, int s, float* features);
/* One solve driven from the host with CUDA events around every kernel (same kernels and loop
 * decisions as the graph, read back after each check); per kernel kind the summed device time
 * and launch count, and the time of its first launch (SPTRSV_BATCH_KINDS kinds: fill x, FP64
 * pull, state init, mixed init, step begin, fill d, panels, FP32 pull, Jacobi sweep, sweep check,
 * axpy, residual, step check, FP64 panels). */
#define SPTRSV_BATCH_KINDS 14
SPTRSV_API int sptrsv_batch_profile(sptrsv_batch b, int mode, const double* d_b, double* d_x, float* kind_ms,
                                    int* kind_launches, float* kind_first_ms);
SPTRSV_API int sptrsv_batch_timer_begin(sptrsv_batch b);
SPTRSV_API int sptrsv_batch_timer_end(sptrsv_batch b, float* ms);
SPTRSV_API int64_t sptrsv_batch_launches(sptrsv_batch b);

/* ---------------------------------------------------------------------------------------
 * The learned schedule selector's network (no counterpart in the reference): an FP32 MLP
 * in -> h1 -> h2 -> out with ReLU hidden layers that predicts each candidate schedule's log
 * runtime from the matrix features (sptrsv_features).  Trained on the GPU by the library's own
 * forward, backward and Adam kernels.  Parameters are one flat array: W1 (h1 x in, row-major),
 * b1, W2 (h2 x h1), b2, W3 (out x h2), b3.  Inputs are standardised as (x - mean) * scale.
 * Loss: sum mask (P - Y)^2 / sum mask over a batch (mask 0 = not measured).  All arrays are
 * host, row-major, one sample per row. */
typedef struct sptrsv_mlp_s* sptrsv_mlp;
SPTRSV_API int sptrsv_mlp_create(sptrsv_mlp* out, int device, int in, int h1, int h2, int nout, uint64_t seed);
SPTRSV_API int sptrsv_mlp_destroy(sptrsv_mlp m);
SPTRSV_API int sptrsv_mlp_num_params(sptrsv_mlp m);
SPTRSV_API int sptrsv_mlp_get_params(sptrsv_mlp m, float* params);
SPTRSV_API int sptrsv_mlp_set_params(sptrsv_mlp m, const float* params);
SPTRSV_API int sptrsv_mlp_set_norm(sptrsv_mlp m, const float* mean, const float* scale);
/* Full-batch loss and gradient (no update). */
SPTRSV_API int sptrsv_mlp_grad(sptrsv_mlp m, int n, const float* x, const float* y, const float* mask, float* grad,
                               float* loss);
/* Adam over `epochs` shuffled passes (mt19937_64(seed)) in mini-batches; loss_out[epochs]. */
SPTRSV_API int sptrsv_mlp_train(sptrsv_mlp m, int n, const float* x, const float* y, const float* mask, int epochs,
                                int batch, float lr, uint64_t seed, float* loss_out);
SPTRSV_API int sptrsv_mlp_predict(sptrsv_mlp m, int n, const float* x, float* y);
SPTRSV_API int64_t sptrsv_mlp_launches(sptrsv_mlp m);

/* ---------------------------------------------------------------------------------------
 * The reference's file formats (utils.cpp:9-109), host side.  By extension:
 *   .matrix binary  int32 n, uint64 nz, int32 col[nz], uint64 row_ptr[n+1], f64 val[nz];
 *   .txt            n nz / val[nz] / col[nz] / row_ptr[n+1];
 *   .mtx (read)     MatrixMarket entries of a lower factor in column order, read as the CSR of
 *                   its transpose (utils.cpp:32-60);
 *   .snodes binary  int32 sn, int32 snodes[sn+1];  .txt: sn / snodes[sn+1].
 * Arrays returned by the readers are malloc'd; release them with sptrsv_io_free.  Failures:
 * SPTRSV_ERR_IO (unreadable or malformed), SPTRSV_ERR_INVALID_ARG (unknown extension). */
SPTRSV_API int sptrsv_read_csr(const char* path, int* n, int64_t* nnz, int64_t** row_ptr, int** col, double** val);
SPTRSV_API int sptrsv_write_csr(const char* path, int n, int64_t nnz, const int64_t* row_ptr, const int* col,
                                const double* val);
SPTRSV_API int sptrsv_read_snodes(const char* path, int* sn, int** snodes);
SPTRSV_API int sptrsv_write_snodes(const char* path, int sn, const int* snodes);
SPTRSV_API void sptrsv_io_free(void* p);

#ifdef __cplusplus
}
#endif
#endif
