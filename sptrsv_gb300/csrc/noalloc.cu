// noalloc.cu -- sptrsv_solve_noalloc: the FP64 sync-free warp solve for callers that must not
// allocate device memory.
//
// Who needs it: applications that hand the whole GPU to their own memory pool and forbid any
// other allocation, and latency-critical loops that cannot afford cudaMalloc / cudaFree (they
// synchronise the device and can fail at run time).  Such callers own the matrix, b and x;
// everything else this solve needs lives in the file-scope array below:
//   * the control block of the spins (row ticket, status word, abort flag), and
//   * the reciprocal diagonal, one double per row, for at most SPTRSV_NOALLOC_MAX_ROWS rows.
// The array is part of the library image: every GPU that loads the library holds it
// (SPTRSV_NOALLOC_MAX_ROWS * 8 bytes + 256) until the process exits.
//
// Host code must not pass `g_noalloc_scratch` itself to a kernel -- on the host that name is
// only a stand-in, not a device address.  Every call looks the device address up with
// cudaGetSymbolAddress on the current device.  The call synchronises its stream, so it cannot be
// captured into a CUDA graph.  All calls share
// the one array and it keeps the previous call's contents: each call clears the control block
// and rewrites the reciprocal diagonal for its rows before the solve.  A call runs in two
// phases on its stream (checks, then the solve), so every call in the process holds one lock
// from its first enqueue to its return: calls from several host threads run one after another,
// whatever streams they use.  Work the caller enqueues itself cannot be ordered by that lock,
// so calls that overlap on the GPU with another use of the array (another process's calls
// never do: each process has its own copy) must not be made.
#include <mutex>
#include "common.cuh"
#include "kernels.cuh"

namespace sptrsv {

struct NoallocScratch {
    Ctl ctl;
    char pad[256 - sizeof(Ctl) % 256];
    double invd[SPTRSV_NOALLOC_MAX_ROWS];
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// Row checks (the same rules as the analysis: row pointer monotone from 0 to nnz, diagonal
// first, other columns in (i, n), finite non-zero pivot) and the reciprocal diagonal.
__global__ void k_noalloc_prepare(int n, int nnz, const int* __restrict__ rp, const int* __restrict__ col,
                                  const double* __restrict__ val, NoallocScratch* s) {
    Ctl* ctl = &s->ctl;
    if (blockIdx.x == 0 && threadIdx.x == 0 && (rp[0] != 0 || rp[n] != nnz)) record_error(ctl, SPTRSV_ERR_ROW_PTR);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int b = rp[i], e = rp[i + 1];
        if (e < b || b < 0 || e > nnz) { record_error(ctl, SPTRSV_ERR_ROW_PTR); continue; }
        if (e == b || col[b] != i) { record_error(ctl, SPTRSV_ERR_MISSING_DIAG); continue; }
        const double d = val[b];
        if (d == 0.0 || !isfinite(d)) record_error(ctl, SPTRSV_ERR_ZERO_PIVOT);
        s->invd[i] = 1.0 / d;
        for (int k = b + 1; k < e; ++k) {
            const int c = col[k];
            if (c < 0 || c >= n) { record_error(ctl, SPTRSV_ERR_COL_RANGE); break; }
            if (c <= i) { record_error(ctl, SPTRSV_ERR_NOT_UPPER); break; }
        }
    }
}

static std::mutex g_noalloc_mu;

// The array's device address on the current device, looked up on every call (cheap next to the
// call's two stream synchronisations, and never stale after a cudaDeviceReset reloads the module).
static int noalloc_scratch(NoallocScratch** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return set_cuda_error(e, "cudaGetSymbolAddress");
    *out = static_cast<NoallocScratch*>(p);
    return 0;
}

}  // namespace sptrsv

extern "C" int sptrsv_solve_noalloc(int n, int nnz, const int* d_row_ptr, const int* d_col, const double* d_val,
                                    const double* d_b, double* d_x, void* stream) {
    using namespace sptrsv;
    if (n <= 0 || nnz < n || !d_row_ptr || !d_col || !d_val || !d_b || !d_x) return SPTRSV_ERR_INVALID_ARG;
    if (n > SPTRSV_NOALLOC_MAX_ROWS) return SPTRSV_ERR_TOO_LARGE;
    int device = 0;
    CUDA_TRY(cudaGetDevice(&device));
    // one call at a time in this process: the checks and the solve both use the shared array
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoallocScratch* s = nullptr;
    int rc = noalloc_scratch(&s);
    if (rc) return rc;
    int sm_count = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int64_t launches = 0;
    CUDA_TRY(cudaMemsetAsync(&s->ctl, 0, sizeof(Ctl), st));
    k_noalloc_prepare<<<sm_count * 4, 256, 0, st>>>(n, nnz, d_row_ptr, d_col, d_val, s);
    CUDA_TRY(cudaGetLastError());
    int status = 0;
    CUDA_TRY(cudaMemcpyAsync(&status, &s->ctl.status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (status) return status;
    if ((rc = launch_fill_pending(false, d_x, (size_t)n, st, &launches))) return rc;
    SolveArgs a{};
    a.n = n;
    a.rp = d_row_ptr;
    a.col = d_col;
    a.val = d_val;
    a.invd = s->invd;
    a.b = d_b;
    a.x = d_x;
    a.rhs = 1;
    a.ctl = &s->ctl;
    a.budget = kDefaultBudgetNs;
    a.sm_count = sm_count;
    a.warps = 0;
    a.st = st;
    a.launches = &launches;
    const double mean = (double)nnz / n;
    const int rows_per_warp = mean <= 6 ? 8 : (mean <= 12 ? 4 : (mean <= 24 ? 2 : 1));
    if ((rc = launch_pull_warp(false, a, rows_per_warp, 0))) return rc;
    CUDA_TRY(cudaMemcpyAsync(&status, &s->ctl.status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return status;
}
