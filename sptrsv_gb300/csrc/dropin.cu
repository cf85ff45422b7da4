// dropin.cu -- the reference's entry points (include/core.h, include/sptrsv_syncfree_opencl.h)
// with their exact C++ signatures, running on the GPU through one process-wide handle.
//
// Each call follows the reference's contract: caller-owned host arrays in, result written
// to the caller's x, elapsed seconds returned.  The time is device time measured with CUDA
// events around the solve kernels (the reference's GPU drivers report kernel-only time,
// sptrsv_syncfree_opencl.cpp:335-360); barrier_upper's time includes its level analysis, as
// the reference's does (core.cpp:375).  Failures return the negative sptrsv_status as a
// double and record it for sptrsv_last_status(); nothing prints or exits.
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <vector>
#include "common.cuh"
#include "kernels.cuh"
#include "handle.cuh"
#include "../../include/core.h"
#include "../../include/sptrsv_syncfree_opencl.h"

namespace sptrsv {

static std::mutex g_mu;
static sptrsv_handle g_h = nullptr;

static int default_handle(Handle** out) {
    if (!g_h) {
        int rc = sptrsv_create(&g_h, -1);
        if (rc) { g_h = nullptr; return rc; }
    }
    Handle* h = reinterpret_cast<Handle*>(g_h);
    if (cudaSetDevice(h->device) != cudaSuccess) return SPTRSV_ERR_CUDA;
    *out = h;
    return 0;
}

static double fail(int rc) {
    set_last_status(rc);
    return (double)rc;
}

__global__ void k_fill_f64(size_t count, double v, double* __restrict__ p) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x) p[k] = v;
}

// Row -> first row of its supernode; checks the partition (0 = s_0 < s_1 < ... < s_sn = n).
__global__ void k_snode_start(int sn, const int* __restrict__ snodes, int n, int* __restrict__ start, Ctl* ctl) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < sn; s += gridDim.x * blockDim.x) {
        const int a = snodes[s], b = snodes[s + 1];
        if ((s == 0 && a != 0) || (s == sn - 1 && b != n) || b <= a || a < 0 || b > n) {
            record_error(ctl, SPTRSV_ERR_SUPERNODES);
            continue;
        }
        for (int i = a; i < b; ++i) start[i] = a;
    }
}

// ccs2ccs_pad (core.cpp:136-161): padded row length = row length + offset in supernode.
__global__ void k_pad_lengths(int n, const int* __restrict__ rp, const int* __restrict__ start, int* __restrict__ len) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        len[i] = rp[i + 1] - rp[i] + (i - start[i]);
}
__global__ void k_pad_fill(int n, const int* __restrict__ rp, const int* __restrict__ col, const double* __restrict__ val,
                           const int* __restrict__ start, const int* __restrict__ prp, double* __restrict__ pval,
                           uint64_t* __restrict__ pcol) {
    const int lane = threadIdx.x & 31;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += (gridDim.x * blockDim.x) >> 5) {
        const int s0 = start[i], d = i - s0;
        const int base = prp[i];
        const int c0 = col[rp[s0]];  // the reference pads with row[col_index[nodes[si]]] + ci
        for (int q = lane; q < d; q += 32) { pval[base + q] = 0.0; pcol[base + q] = (uint64_t)(c0 + q); }
        for (int k = rp[i] + lane; k < rp[i + 1]; k += 32) {
            pval[base + d + (k - rp[i])] = val[k];
            pcol[base + d + (k - rp[i])] = (uint64_t)col[k];
        }
    }
}
// Inverse: drop the `i - start` leading padding entries of every padded row.
__global__ void k_unpad_lengths(int n, int nz, const int* __restrict__ prp, const int* __restrict__ start,
                                int* __restrict__ len, Ctl* ctl) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && (prp[0] != 0 || prp[n] > nz)) record_error(ctl, SPTRSV_ERR_ROW_PTR);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int l = prp[i + 1] - prp[i] - (i - start[i]);
        if (l < 1 || prp[i + 1] < prp[i]) { record_error(ctl, SPTRSV_ERR_SUPERNODES); len[i] = 0; }
        else len[i] = l;
    }
}
__global__ void k_unpad_fill(int n, const int* __restrict__ prp, const uint64_t* __restrict__ pcol,
                             const double* __restrict__ pval, const int* __restrict__ start, const int* __restrict__ rp,
                             int* __restrict__ col, double* __restrict__ val) {
    const int lane = threadIdx.x & 31;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += (gridDim.x * blockDim.x) >> 5) {
        const int d = i - start[i];
        const int src = prp[i] + d, len = rp[i + 1] - rp[i];
        for (int q = lane; q < len; q += 32) {
            const uint64_t c = pcol[src + q];
            col[rp[i] + q] = c > 0x7fffffffull ? -1 : (int)c;
            val[rp[i] + q] = pval[src + q];
        }
    }
}

// Host CSR with a 32-bit row pointer (the OpenCL-side layout).
static int set_matrix_host32(Handle* h, int n, int nnz, const int* rp32, const int* col, const double* val) {
    if (n <= 0 || nnz < n || !rp32 || !col || !val) return SPTRSV_ERR_INVALID_ARG;
    h->drop_matrix();
    int rc;
    h->n = n;
    h->nnz = nnz;
    if ((rc = h->own_rp.ensure(sizeof(int) * (size_t)(n + 1)))) return rc;
    if ((rc = h->own_col.ensure(sizeof(int) * (size_t)nnz))) return rc;
    if ((rc = h->own_val.ensure(sizeof(double) * (size_t)nnz))) return rc;
    CUDA_TRY(cudaMemcpyAsync(h->own_rp.p, rp32, sizeof(int) * (size_t)(n + 1), cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(cudaMemcpyAsync(h->own_col.p, col, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, h->st));
    CUDA_TRY(cudaMemcpyAsync(h->own_val.p, val, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, h->st));
    h->rp = h->own_rp.as<int>();
    h->col = h->own_col.as<int>();
    h->val = h->own_val.as<double>();
    return 0;
}

// Solve with host b / x, timing only the enqueued solve with events.
static int solve_host_timed(Handle* h, const sptrsv_opts& o, const double* b, double* x, int rhs, int layout,
                            double* secs) {
    const size_t bytes = sizeof(double) * (size_t)h->n * rhs;
    int rc;
    if ((rc = h->db.ensure(bytes))) return rc;
    if ((rc = h->dx.ensure(bytes))) return rc;
    CUDA_TRY(cudaMemcpyAsync(h->db.p, b, bytes, cudaMemcpyHostToDevice, h->st));
    // warm the graph cache / allocations outside the timed region
    sptrsv_opts r = h->resolve(&o, rhs);
    if ((rc = h->prepare(r, rhs, layout))) return rc;
    CUDA_TRY(cudaEventRecord(h->ev0, h->st));
    if ((rc = h->solve(&o, h->db.as<double>(), h->dx.as<double>(), rhs, layout))) return rc;
    CUDA_TRY(cudaEventRecord(h->ev1, h->st));
    CUDA_TRY(cudaMemcpyAsync(x, h->dx.p, bytes, cudaMemcpyDeviceToHost, h->st));
    rc = h->sync();
    if (rc && rc != SPTRSV_ERR_NOT_CONVERGED) return rc;
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    *secs = ms * 1e-3;
    return rc;
}

// Whether FP64 accuracy through refinement (FP32 Jacobi sweeps, FP64 residuals) should beat the
// exact sync-free solve by a wide margin: the exact solve waits one dependent global-memory hop
// (~1 us on GB300) per level of the DAG (the analysis's depth estimate when the levels have not
// been computed); the refinement makes about 40 bandwidth-bound sweeps and 4 FP64 residual
// passes, and needs sweeps that contract (every row strictly dominant).
static bool refinement_pays(const Handle* h, int rhs) {
    // dense skyline rows go to the exact FP64 panels instead
    if (!(h->max_ratio < 1.0) || rhs > 1024 || h->dense_skyline()) return false;
    const double depth = h->levels_ready ? (double)h->max_level : h->depth_est;
    const double n = h->n, nnz = h->nnz;
    const double sweep_s = (8.0 * (nnz - n) + 16.0 * n * rhs) / 4.0e12 + 4.0e-6;
    const double resid_s = (12.0 * nnz + 24.0 * n * rhs) / 3.5e12 + 4.0e-6;
    const double refined_s = 40.0 * sweep_s + 4.0 * resid_s;
    const double exact_s = 1.0e-6 * depth;
    return refined_s < 0.25 * exact_s;
}

static sptrsv_opts fp64(int schedule) {
    sptrsv_opts o;
    sptrsv_default_opts(&o);
    o.schedule = schedule;
    return o;
}

// The FP64 solve of the serial-substitution entry points (any schedule whose result meets the
// serial solve's accuracy): for deep DAGs with dominant rows, FP64 accuracy through refinement
// with the exact AUTO solve if it stalls; otherwise the exact AUTO solve.  *secs: device time of
// the solves made.
static int solve_fp64_host(Handle* h, const double* b, double* x, int rhs, double* secs) {
    *secs = 0.0;
    int rc;
    if (refinement_pays(h, rhs)) {
        sptrsv_opts o = fp64(SPTRSV_SCHED_JACOBI);
        o.max_refine = 6;
        rc = solve_host_timed(h, o, b, x, rhs, SPTRSV_COL_MAJOR, secs);
        if (rc != SPTRSV_ERR_NOT_CONVERGED) return rc;
    }
    double exact = 0.0;
    rc = solve_host_timed(h, fp64(SPTRSV_SCHED_AUTO), b, x, rhs, SPTRSV_COL_MAJOR, &exact);
    *secs += exact;
    return rc;
}

static double gauss_upper(int n, double* val, uint64_t* row_index, int* col, double* x, double* b, int rhs) {
    std::lock_guard<std::mutex> lk(g_mu);
    Handle* h;
    int rc;
    if ((rc = default_handle(&h))) return fail(rc);
    if (n <= 0 || rhs < 1 || !val || !row_index || !col || !x || !b) return fail(SPTRSV_ERR_INVALID_ARG);
    if ((rc = h->set_matrix_host(n, (int64_t)row_index[n], (const int64_t*)row_index, col, val))) return fail(rc);
    if ((rc = h->analyse())) return fail(rc);
    double secs = 0;
    if ((rc = solve_fp64_host(h, b, x, rhs, &secs))) return fail(rc);
    set_last_status(0);
    return secs;
}

// Lower-triangular CSR (diagonal last in every row) -> the upper-triangular CSR of the same
// system with rows and columns in reverse order: U = P L P, P the reversal permutation.  Row r of
// U is row n-1-r of L read backwards, so the whole col/val arrays are reversed (columns mapped to
// n-1-c) and U's row pointer is nnz - L's taken from the end.  rp_l is a copy of L's row pointer.
__global__ void k_reverse_lower(int n, int nnz, const int* __restrict__ rp_l, int* __restrict__ rp_u, int* col,
                                double* val) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    for (int r = tid; r <= n; r += nth) rp_u[r] = nnz - rp_l[n - r];
    for (int k = tid; k < (nnz + 1) / 2; k += nth) {
        const int q = nnz - 1 - k;
        const int ck = col[k], cq = col[q];
        const double vk = val[k], vq = val[q];
        col[k] = n - 1 - cq;
        col[q] = n - 1 - ck;
        val[k] = vq;
        val[q] = vk;
    }
}

// core.cpp:4-16: forward substitution, solved as the reversed upper system on the GPU.
static double gauss_lower(int n, double* val, uint64_t* row_index, int* col, double* x, double* b) {
    std::lock_guard<std::mutex> lk(g_mu);
    Handle* h;
    int rc;
    if ((rc = default_handle(&h))) return fail(rc);
    if (n <= 0 || !val || !row_index || !col || !x || !b) return fail(SPTRSV_ERR_INVALID_ARG);
    const int64_t nnz = (int64_t)row_index[n];
    if ((rc = h->set_matrix_host(n, nnz, (const int64_t*)row_index, col, val))) return fail(rc);
    if ((rc = h->scratch.ensure(sizeof(int) * ((size_t)n + 1)))) return fail(rc);
    if (cudaMemcpyAsync(h->scratch.p, h->own_rp.p, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToDevice, h->st) !=
        cudaSuccess)
        return fail(SPTRSV_ERR_CUDA);
    k_reverse_lower<<<h->sm_count * 4, 256, 0, h->st>>>(n, (int)nnz, (const int*)h->scratch.p, h->own_rp.as<int>(),
                                                        h->own_col.as<int>(), h->own_val.as<double>());
    h->launches++;
    if (cudaGetLastError() != cudaSuccess) return fail(SPTRSV_ERR_CUDA);
    if ((rc = h->analyse())) return fail(rc);
    std::vector<double> br(b, b + n), xr(n);
    std::reverse(br.begin(), br.end());
    double secs = 0;
    if ((rc = solve_fp64_host(h, br.data(), xr.data(), 1, &secs))) return fail(rc);
    std::reverse_copy(xr.begin(), xr.end(), x);
    set_last_status(0);
    return secs;
}

// In-place supernodal solve (x holds b on entry).  Runs the supernode-blocked path when the
// partition is valid.
static double supernodal_inplace(size_t sn, int* supernodes, double* x, double* val, int* row, uint64_t* col_index,
                                 int n, int rhs) {
    std::lock_guard<std::mutex> lk(g_mu);
    Handle* h;
    int rc;
    if ((rc = default_handle(&h))) return fail(rc);
    if (n <= 0 || rhs < 1 || sn < 1 || !supernodes || !x || !val || !row || !col_index) return fail(SPTRSV_ERR_INVALID_ARG);
    if ((rc = h->set_matrix_host(n, (int64_t)col_index[n], (const int64_t*)col_index, row, val))) return fail(rc);
    if ((rc = h->analyse())) return fail(rc);
    // check the supernode partition on the device
    if ((rc = h->scratch.ensure(sizeof(int) * ((size_t)n + sn + 2)))) return fail(rc);
    int* d_sn = (int*)h->scratch.p;
    int* d_start = d_sn + sn + 1;
    if (cudaMemcpyAsync(d_sn, supernodes, sizeof(int) * (sn + 1), cudaMemcpyHostToDevice, h->st) != cudaSuccess)
        return fail(SPTRSV_ERR_CUDA);
    if ((rc = h->reset_ctl())) return fail(rc);
    k_snode_start<<<h->sm_count, 256, 0, h->st>>>((int)sn, d_sn, n, d_start, h->ctl);
    h->launches++;
    Ctl c{};
    if ((rc = h->read_ctl(&c))) return fail(rc);
    if (c.status) return fail(c.status);
    std::vector<double> bcopy(x, x + (size_t)n * rhs);
    double secs = 0;
    // dense supernode panels when every supernode's rows share one rectangle; otherwise (the
    // reference also accepts rows with their own rectangle entries) the general FP64 solve
    const int sched = h->set_supernodes((int)sn, supernodes) == 0 ? SPTRSV_SCHED_SUPERNODAL : SPTRSV_SCHED_AUTO;
    if ((rc = solve_host_timed(h, fp64(sched), bcopy.data(), x, rhs, SPTRSV_COL_MAJOR, &secs))) return fail(rc);
    set_last_status(0);
    return secs;
}

static double blas_padded(int n, int nz, size_t sn, int* supernodes, double* x, double* val, uint64_t* colidx_pad,
                          int* rowptr_pad, int rhs) {
    std::lock_guard<std::mutex> lk(g_mu);
    Handle* h;
    int rc;
    if ((rc = default_handle(&h))) return fail(rc);
    if (n <= 0 || nz < n || rhs < 1 || sn < 1 || !supernodes || !x || !val || !colidx_pad || !rowptr_pad)
        return fail(SPTRSV_ERR_INVALID_ARG);
    h->drop_matrix();
    // upload padded arrays into scratch, unpad on the device into the owned CSR buffers
    const size_t need = sizeof(uint64_t) * (size_t)nz + sizeof(double) * (size_t)nz +
                        sizeof(int) * ((size_t)3 * n + sn + 8) + sizeof(int) * (size_t)scan_partials_needed(n) + 4096;
    if ((rc = h->scratch.ensure(need))) return fail(rc);
    Scratch scr{(char*)h->scratch.p, h->scratch.cap, 0};
    uint64_t* pcol = scr.take<uint64_t>(nz);
    double* pval = scr.take<double>(nz);
    int* prp = scr.take<int>(n + 1);
    int* d_sn = scr.take<int>(sn + 1);
    int* start = scr.take<int>(n);
    int* len = scr.take<int>(n + 1);
    int* part = scr.take<int>(scan_partials_needed(n));
    if (cudaMemcpyAsync(pcol, colidx_pad, sizeof(uint64_t) * nz, cudaMemcpyHostToDevice, h->st) ||
        cudaMemcpyAsync(pval, val, sizeof(double) * nz, cudaMemcpyHostToDevice, h->st) ||
        cudaMemcpyAsync(prp, rowptr_pad, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, h->st) ||
        cudaMemcpyAsync(d_sn, supernodes, sizeof(int) * (sn + 1), cudaMemcpyHostToDevice, h->st))
        return fail(SPTRSV_ERR_CUDA);
    if ((rc = h->reset_ctl())) return fail(rc);
    k_snode_start<<<h->sm_count, 256, 0, h->st>>>((int)sn, d_sn, n, start, h->ctl);
    k_unpad_lengths<<<h->sm_count * 4, 256, 0, h->st>>>(n, nz, prp, start, len, h->ctl);
    h->launches += 2;
    if ((rc = scan_exclusive(len, len, n, part, h->st, &h->launches))) return fail(rc);
    Ctl c{};
    if ((rc = h->read_ctl(&c))) return fail(rc);
    if (c.status) return fail(c.status);
    int nnz = 0;
    if (cudaMemcpy(&nnz, len + n, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return fail(SPTRSV_ERR_CUDA);
    h->n = n;
    h->nnz = nnz;
    if ((rc = h->own_rp.ensure(sizeof(int) * (size_t)(n + 1)))) return fail(rc);
    if ((rc = h->own_col.ensure(sizeof(int) * (size_t)nnz))) return fail(rc);
    if ((rc = h->own_val.ensure(sizeof(double) * (size_t)nnz))) return fail(rc);
    if (cudaMemcpyAsync(h->own_rp.p, len, sizeof(int) * (n + 1), cudaMemcpyDeviceToDevice, h->st)) return fail(SPTRSV_ERR_CUDA);
    k_unpad_fill<<<h->sm_count * 8, 256, 0, h->st>>>(n, prp, pcol, pval, start, h->own_rp.as<int>(), h->own_col.as<int>(),
                                                     h->own_val.as<double>());
    h->launches++;
    h->rp = h->own_rp.as<int>();
    h->col = h->own_col.as<int>();
    h->val = h->own_val.as<double>();
    if ((rc = h->analyse())) return fail(rc);
    std::vector<double> bcopy(x, x + (size_t)n * rhs);
    double secs = 0;
    const int sched = h->set_supernodes((int)sn, supernodes) == 0 ? SPTRSV_SCHED_SUPERNODAL : SPTRSV_SCHED_AUTO;
    if ((rc = solve_host_timed(h, fp64(sched), bcopy.data(), x, rhs, SPTRSV_COL_MAJOR, &secs))) return fail(rc);
    set_last_status(0);
    return secs;
}

static double levelset_solve(int n, double* x, double* b, double* val, int* col, uint64_t* row, int rhs) {
    std::lock_guard<std::mutex> lk(g_mu);
    Handle* h;
    int rc;
    if ((rc = default_handle(&h))) return fail(rc);
    if (n <= 0 || rhs < 1 || !x || !b || !val || !col || !row) return fail(SPTRSV_ERR_INVALID_ARG);
    if ((rc = h->set_matrix_host(n, (int64_t)row[n], (const int64_t*)row, col, val))) return fail(rc);
    if (cudaEventRecord(h->ev0, h->st) != cudaSuccess) return fail(SPTRSV_ERR_CUDA);
    if ((rc = h->analyse())) return fail(rc);
    if ((rc = h->ensure_levels())) return fail(rc);
    const size_t bytes = sizeof(double) * (size_t)n * rhs;
    if ((rc = h->db.ensure(bytes)) || (rc = h->dx.ensure(bytes))) return fail(rc);
    if (cudaMemcpyAsync(h->db.p, b, bytes, cudaMemcpyHostToDevice, h->st) != cudaSuccess) return fail(SPTRSV_ERR_CUDA);
    sptrsv_opts o = fp64(SPTRSV_SCHED_LEVELSET);
    if ((rc = h->solve(&o, h->db.as<double>(), h->dx.as<double>(), rhs, SPTRSV_COL_MAJOR))) return fail(rc);
    if (cudaEventRecord(h->ev1, h->st) != cudaSuccess) return fail(SPTRSV_ERR_CUDA);
    if (cudaMemcpyAsync(x, h->dx.p, bytes, cudaMemcpyDeviceToHost, h->st) != cudaSuccess) return fail(SPTRSV_ERR_CUDA);
    if ((rc = h->sync())) return fail(rc);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    set_last_status(0);
    return ms * 1e-3;
}

// sptrsv_syncfree_opencl family on a CSC input: analyser (in-degree histogram) + push solve.
static double csc_push(int* cp, int* crow, const double* cval, int m, int n, int nnz, double* x, const double* b,
                       int rhs) {
    if (m != n) return fail(SPTRSV_ERR_NOT_SQUARE);
    std::lock_guard<std::mutex> lk(g_mu);
    Handle* h;
    int rc;
    if ((rc = default_handle(&h))) return fail(rc);
    if (n <= 0 || nnz < n || rhs < 1 || !cp || !crow || !cval || !x || !b) return fail(SPTRSV_ERR_INVALID_ARG);
    memset(x, 0, sizeof(double) * (size_t)m);  // sptrsv_syncfree_opencl.cpp:193
    h->drop_matrix();
    h->n = n;
    h->nnz = nnz;
    const size_t nr = (size_t)n * rhs;
    if ((rc = h->csc_ptr.ensure(sizeof(int) * (size_t)(n + 1))) || (rc = h->csc_row.ensure(sizeof(int) * (size_t)nnz)) ||
        (rc = h->csc_val.ensure(sizeof(double) * (size_t)nnz)) || (rc = h->invd.ensure(sizeof(double) * (size_t)n)) ||
        (rc = h->in_degree.ensure(sizeof(int) * (size_t)n)) || (rc = h->indeg_work.ensure(sizeof(int) * (size_t)n)) ||
        (rc = h->left.ensure(sizeof(double) * nr)) || (rc = h->db.ensure(sizeof(double) * nr)) ||
        (rc = h->dx.ensure(sizeof(double) * nr)))
        return fail(rc);
    if (cudaMemcpyAsync(h->csc_ptr.p, cp, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, h->st) ||
        cudaMemcpyAsync(h->csc_row.p, crow, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, h->st) ||
        cudaMemcpyAsync(h->csc_val.p, cval, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, h->st) ||
        cudaMemcpyAsync(h->db.p, b, sizeof(double) * nr, cudaMemcpyHostToDevice, h->st))
        return fail(SPTRSV_ERR_CUDA);
    if ((rc = h->reset_ctl())) return fail(rc);
    k_validate_csc<<<h->sm_count * 4, 256, 0, h->st>>>(n, nnz, h->csc_ptr.as<int>(), h->csc_row.as<int>(),
                                                       h->csc_val.as<double>(), h->invd.as<double>(), h->ctl);
    if (cudaMemsetAsync(h->in_degree.p, 0, sizeof(int) * (size_t)n, h->st)) return fail(SPTRSV_ERR_CUDA);
    h->launches++;
    Ctl c{};
    if ((rc = h->read_ctl(&c))) return fail(rc);
    if (c.status) return fail(c.status);
    k_in_degree_csc<<<h->sm_count * 4, 256, 0, h->st>>>(nnz, h->csc_row.as<int>(), h->in_degree.as<int>());
    h->launches++;
    if (cudaMemcpyAsync(h->indeg_work.p, h->in_degree.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, h->st) ||
        cudaMemsetAsync(h->left.p, 0, sizeof(double) * nr, h->st) || cudaMemsetAsync(h->ctl, 0, sizeof(Ctl), h->st))
        return fail(SPTRSV_ERR_CUDA);
    SolveArgs a{};
    a.n = n;
    a.invd = h->invd.p;
    a.b = h->db.p;
    a.x = h->dx.p;
    a.rhs = rhs;
    a.ctl = h->ctl;
    a.budget = kDefaultBudgetNs;
    a.sm_count = h->sm_count;
    a.st = h->st;
    a.launches = &h->launches;
    if (cudaEventRecord(h->ev0, h->st) != cudaSuccess) return fail(SPTRSV_ERR_CUDA);
    if ((rc = launch_push_csc(a, h->csc_ptr.as<int>(), h->csc_row.as<int>(), h->csc_val.as<double>(),
                              h->indeg_work.as<int>(), h->left.as<double>())))
        return fail(rc);
    if (cudaEventRecord(h->ev1, h->st) != cudaSuccess) return fail(SPTRSV_ERR_CUDA);
    if (cudaMemcpyAsync(x, h->dx.p, sizeof(double) * nr, cudaMemcpyDeviceToHost, h->st) != cudaSuccess)
        return fail(SPTRSV_ERR_CUDA);
    if ((rc = h->read_ctl(&c))) return fail(rc);
    if (c.status) return fail(c.status);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    set_last_status(0);
    return ms * 1e-3;
}

}  // namespace sptrsv

using namespace sptrsv;

double base_gauss_lower(int n, double* val, uint64_t* row_index, int* col, double* x, double* b) {
    return gauss_lower(n, val, row_index, col, x, b);
}

double base_gauss_upper(int n, double* val, uint64_t* row_index, int* col, double* x, double* b, int rhs) {
    return gauss_upper(n, val, row_index, col, x, b, rhs);
}

double base_gauss_upper_new(int n, double* val, uint64_t* row_index, int* col, double* x, double* b, int rhs) {
    return gauss_upper(n, val, row_index, col, x, b, rhs);
}

double supernodal_upper(size_t sn, int* supernodes, double* x, double* val, int* row, uint64_t* col_index, int n,
                        int rhs) {
    return supernodal_inplace(sn, supernodes, x, val, row, col_index, n, rhs);
}

double supernodal_upper_new(size_t sn, int* supernodes, double* x, double* val, int* row, uint64_t* col_index, int n,
                            int rhs) {
    return supernodal_inplace(sn, supernodes, x, val, row, col_index, n, rhs);
}

double supernodal_blas_upper(int n, int nz, size_t sn, int* supernodes, double* x, double* val, uint64_t* col_index,
                             int* row, int rhs) {
    return blas_padded(n, nz, sn, supernodes, x, val, col_index, row, rhs);
}

double supernodal_blas_upper_new(int n, int nz, size_t sn, int* supernodes, double* x, double* val,
                                 uint64_t* col_index, int* row, int rhs) {
    return blas_padded(n, nz, sn, supernodes, x, val, col_index, row, rhs);
}

double ccs2ccs_pad(double* val, int* row, uint64_t* col_index, double* val_pad, uint64_t* col_index_pad, int* row_pad,
                   int* nodes, int& sn, int& nnz) {
    std::lock_guard<std::mutex> lk(g_mu);
    Handle* h;
    int rc;
    if ((rc = default_handle(&h))) return fail(rc);
    if (sn < 1 || !val || !row || !col_index || !val_pad || !col_index_pad || !row_pad || !nodes)
        return fail(SPTRSV_ERR_INVALID_ARG);
    const int n = nodes[sn];
    if (n <= 0) return fail(SPTRSV_ERR_SUPERNODES);
    if ((rc = h->set_matrix_host(n, (int64_t)col_index[n], (const int64_t*)col_index, row, val))) return fail(rc);
    if ((rc = h->analyse())) return fail(rc);  // the pad kernels index through the checked CSR
    const int nz0 = h->nnz;
    h->drop_graphs();
    if (cudaEventRecord(h->ev0, h->st) != cudaSuccess) return fail(SPTRSV_ERR_CUDA);
    const size_t need = sizeof(int) * ((size_t)3 * n + sn + 8) + sizeof(int) * (size_t)scan_partials_needed(n) + 4096;
    if ((rc = h->scratch.ensure(need))) return fail(rc);
    Scratch scr{(char*)h->scratch.p, h->scratch.cap, 0};
    int* d_sn = scr.take<int>(sn + 1);
    int* start = scr.take<int>(n);
    int* len = scr.take<int>(n + 1);
    int* part = scr.take<int>(scan_partials_needed(n));
    if (cudaMemcpyAsync(d_sn, nodes, sizeof(int) * (sn + 1), cudaMemcpyHostToDevice, h->st)) return fail(SPTRSV_ERR_CUDA);
    if ((rc = h->reset_ctl())) return fail(rc);
    k_snode_start<<<h->sm_count, 256, 0, h->st>>>(sn, d_sn, n, start, h->ctl);
    k_pad_lengths<<<h->sm_count * 4, 256, 0, h->st>>>(n, h->rp, start, len);
    h->launches += 2;
    if ((rc = scan_exclusive(len, len, n, part, h->st, &h->launches))) return fail(rc);
    Ctl c{};
    if ((rc = h->read_ctl(&c))) return fail(rc);
    if (c.status) return fail(c.status);
    int total = 0;
    if (cudaMemcpy(&total, len + n, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return fail(SPTRSV_ERR_CUDA);
    // outputs: reuse the FP32/aux buffers as staging
    if ((rc = h->left.ensure(sizeof(double) * (size_t)total)) || (rc = h->dx.ensure(sizeof(uint64_t) * (size_t)total)))
        return fail(rc);
    k_pad_fill<<<h->sm_count * 8, 256, 0, h->st>>>(n, h->rp, h->col, h->val, start, len, h->left.as<double>(),
                                                   h->dx.as<uint64_t>());
    h->launches++;
    if (cudaEventRecord(h->ev1, h->st) != cudaSuccess) return fail(SPTRSV_ERR_CUDA);
    if (cudaMemcpyAsync(val_pad, h->left.p, sizeof(double) * (size_t)total, cudaMemcpyDeviceToHost, h->st) ||
        cudaMemcpyAsync(col_index_pad, h->dx.p, sizeof(uint64_t) * (size_t)total, cudaMemcpyDeviceToHost, h->st) ||
        cudaMemcpyAsync(row_pad, len, sizeof(int) * (size_t)(n + 1), cudaMemcpyDeviceToHost, h->st) ||
        cudaStreamSynchronize(h->st))
        return fail(SPTRSV_ERR_CUDA);
    (void)nz0;
    nnz = total;
    h->drop_matrix();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    set_last_status(0);
    return ms * 1e-3;
}

int setLevelUpAndGetMaxLevel(int n, int* col, uint64_t* row_index, uint64_t* levelsUp) {
    std::lock_guard<std::mutex> lk(g_mu);
    Handle* h;
    int rc;
    if ((rc = default_handle(&h))) { set_last_status(rc); return rc; }
    if (n <= 0 || !col || !row_index || !levelsUp) { set_last_status(SPTRSV_ERR_INVALID_ARG); return SPTRSV_ERR_INVALID_ARG; }
    const int64_t nnz = (int64_t)row_index[n];
    // the pattern alone defines the levels: upload it with unit values
    h->drop_matrix();
    if (nnz < n || nnz > 0x7fffffffll) { set_last_status(SPTRSV_ERR_TOO_LARGE); return SPTRSV_ERR_TOO_LARGE; }
    if ((rc = h->own_val.ensure(sizeof(double) * (size_t)nnz))) { set_last_status(rc); return rc; }
    k_fill_f64<<<h->sm_count * 4, 256, 0, h->st>>>((size_t)nnz, 1.0, h->own_val.as<double>());
    h->launches++;
    h->n = n;
    h->nnz = (int)nnz;
    if ((rc = h->own_rp.ensure(sizeof(int) * (size_t)(n + 1))) || (rc = h->own_col.ensure(sizeof(int) * (size_t)nnz)) ||
        (rc = h->scratch.ensure(sizeof(int64_t) * (size_t)(n + 1)))) { set_last_status(rc); return rc; }
    if (cudaMemcpyAsync(h->scratch.p, row_index, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyHostToDevice, h->st) ||
        cudaMemcpyAsync(h->own_col.p, col, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, h->st)) {
        set_last_status(SPTRSV_ERR_CUDA);
        return SPTRSV_ERR_CUDA;
    }
    if ((rc = h->reset_ctl())) { set_last_status(rc); return rc; }
    k_narrow_rp<<<h->sm_count * 4, 256, 0, h->st>>>(n + 1, (const int64_t*)h->scratch.p, h->own_rp.as<int>(), h->ctl);
    h->launches++;
    h->rp = h->own_rp.as<int>();
    h->col = h->own_col.as<int>();
    h->val = h->own_val.as<double>();
    if ((rc = h->analyse()) || (rc = h->ensure_levels())) { set_last_status(rc); return rc; }
    if ((rc = sptrsv_get_levels(reinterpret_cast<sptrsv_handle>(h), levelsUp))) { set_last_status(rc); return rc; }
    set_last_status(0);
    return h->max_level;
}

double barrier_upper(int n, double* x, double* b, double* val, int* col, uint64_t* row, int num_of_threads, int rhs) {
    (void)num_of_threads;
    return levelset_solve(n, x, b, val, col, row, rhs);
}

double barrier_upper_new(int n, double* x, double* b, double* val, int* col, uint64_t* row, int num_of_threads,
                         int rhs) {
    (void)num_of_threads;
    return levelset_solve(n, x, b, val, col, row, rhs);
}

double sptrsv_syncfree_opencl(int* cscColPtrTR, int* cscRowIdxTR, double* cscValTR, int m, int n, int nnzTR, double* x,
                              double* b, int rhs) {
    return csc_push(cscColPtrTR, cscRowIdxTR, cscValTR, m, n, nnzTR, x, b, rhs);
}

double sptrsv_syncfree2_opencl(int* cscColPtrTR, int* cscRowIdxTR, const double* cscValTR, const int m, const int n,
                               const int nnzTR, double* x, const double* b) {
    return csc_push(cscColPtrTR, cscRowIdxTR, cscValTR, m, n, nnzTR, x, b, 1);
}

double sptrsv_syncfree3_opencl(int* csrColIdx, int* csrRowPtr, const double* csrVal, const int m, const int n,
                               const int nnz, double* x, const double* b) {
    if (m != n) return fail(SPTRSV_ERR_NOT_SQUARE);
    std::lock_guard<std::mutex> lk(g_mu);
    Handle* h;
    int rc;
    if ((rc = default_handle(&h))) return fail(rc);
    if (!x || !b) return fail(SPTRSV_ERR_INVALID_ARG);
    memset(x, 0, sizeof(double) * (size_t)(m > 0 ? m : 0));  // sptrsv_syncfree3_opencl.cpp:193
    if ((rc = set_matrix_host32(h, n, nnz, csrRowPtr, csrColIdx, csrVal))) return fail(rc);
    if ((rc = h->analyse())) return fail(rc);
    double secs = 0;
    if ((rc = solve_host_timed(h, fp64(SPTRSV_SCHED_SYNCFREE_THREAD), b, x, 1, SPTRSV_COL_MAJOR, &secs))) return fail(rc);
    set_last_status(0);
    return secs;
}
