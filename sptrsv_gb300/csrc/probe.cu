// probe.cu -- measurements of the FP64 pipe that bound the FP64 kernels here, taken on the GPU
// that runs them (no counterpart in the reference).
//
//   * throughput: every SM runs independent FMA chains (eight per thread, a full grid), timed
//     with CUDA events; the result is fused multiply-adds per second;
//   * latency: one thread runs one dependent FMA chain, timed with clock64; the result is SM
//     cycles per FMA.  One dependency hop of an exact FP64 triangular solve costs at least this.
#include "common.cuh"

namespace sptrsv {

constexpr int kRateChains = 8;
constexpr int kRateIters = 4096;
constexpr int kLatIters = 4096;

__global__ void __launch_bounds__(256) k_fp64_rate(double a, double c, double* sink) {
    double v[kRateChains];
#pragma unroll
    for (int q = 0; q < kRateChains; ++q) v[q] = (threadIdx.x + q) * 1e-3;
    for (int it = 0; it < kRateIters; ++it) {
#pragma unroll
        for (int q = 0; q < kRateChains; ++q) v[q] = fma(v[q], a, c);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < kRateChains; ++q) s += v[q];
    if (s == 12345.678) sink[threadIdx.x] = s;  // keeps the chains live; never true for these inputs
}

__global__ void k_fp64_latency(double a, double c, double* sink, long long* cycles) {
    double v = threadIdx.x * 1e-3;
    const long long t0 = clock64();
#pragma unroll 1
    for (int it = 0; it < kLatIters; ++it) v = fma(v, a, c);
    const long long t1 = clock64();
    sink[threadIdx.x] = v;
    if (threadIdx.x == 0) *cycles = t1 - t0;
}

}  // namespace sptrsv

extern "C" int sptrsv_measure_fp64(int device, double* gfma_per_s, double* dep_fma_cycles) {
    using namespace sptrsv;
    if (!gfma_per_s || !dep_fma_cycles) return SPTRSV_ERR_INVALID_ARG;
    int prev = 0;
    CUDA_TRY(cudaGetDevice(&prev));
    CUDA_TRY(cudaSetDevice(device));
    int sms = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    double* sink = nullptr;
    long long* cyc = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = 0;
    float best = 1e30f;
    long long hc = 0;
    const int grid = sms * 8;
    if (cudaMalloc(&sink, 1024 * sizeof(double)) != cudaSuccess || cudaMalloc(&cyc, sizeof(long long)) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        rc = set_cuda_error(cudaGetLastError(), "sptrsv_measure_fp64 setup");
        goto out;
    }
    for (int rep = 0; rep < 4; ++rep) {  // the first run warms the clocks up
        cudaEventRecord(e0, 0);
        k_fp64_rate<<<grid, 256>>>(0.999999, 1e-9, sink);
        cudaEventRecord(e1, 0);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            rc = set_cuda_error(cudaGetLastError(), "k_fp64_rate");
            goto out;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    k_fp64_latency<<<1, 32>>>(0.999999, 1e-9, sink, cyc);
    if (cudaMemcpy(&hc, cyc, sizeof(hc), cudaMemcpyDeviceToHost) != cudaSuccess) {
        rc = set_cuda_error(cudaGetLastError(), "k_fp64_latency");
        goto out;
    }
    *gfma_per_s = (double)grid * 256 * kRateChains * kRateIters / (best * 1e-3) / 1e9;
    *dep_fma_cycles = (double)hc / kLatIters;
out:
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (sink) cudaFree(sink);
    if (cyc) cudaFree(cyc);
    cudaSetDevice(prev);
    return rc;
}
