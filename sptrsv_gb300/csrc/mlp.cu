// mlp.cu -- the learned schedule selector's network: a small FP32 MLP
//     in -> h1 -> h2 -> out,  ReLU after the two hidden layers,
// that predicts every candidate schedule's log runtime from a matrix's features.  It is trained
// on the GPU by the kernels of this file (tiled GEMMs with fused bias / ReLU / ReLU-gradient
// epilogues, the masked mean-squared-error gradient, column sums for the bias gradients, Adam)
// and never touches a solve's arithmetic: its only output is which schedule to run.
//
// Parameters live in one flat FP32 array: W1 (h1 x in, row-major), b1, W2 (h2 x h1), b2,
// W3 (out x h2), b3.  Inputs are standardised with a stored per-feature mean and scale.
// Loss over a batch: sum_{r,k} mask[r,k] (P[r,k] - Y[r,k])^2 / sum mask (targets that were not
// measured carry mask 0).
#include <cmath>
#include <cstring>
#include <random>
#include <vector>
#include "common.cuh"
#include "handle.cuh"

namespace sptrsv {

constexpr int kT = 16;  // GEMM tile

// C[m][n] = sum_k A(m,k) B(k,n), A(m,k) = TA ? A[k*lda+m] : A[m*lda+k], B(k,n) = TB ? B[n*ldb+k] : B[k*ldb+n];
// epilogue: 0 store, 1 + bias[n], 2 relu(. + bias[n]), 3 . * (R[m*ldr+n] > 0)
template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(kT* kT) k_mlp_gemm(int M, int N, int K, const float* __restrict__ A, int lda,
                                                     const float* __restrict__ B, int ldb, float* __restrict__ C,
                                                     int ldc, const float* __restrict__ bias,
                                                     const float* __restrict__ R, int ldr) {
    __shared__ float As[kT][kT + 1];
    __shared__ float Bs[kT][kT + 1];
    const int tx = threadIdx.x % kT, ty = threadIdx.x / kT;
    const int m = blockIdx.y * kT + ty, n = blockIdx.x * kT + tx;
    float acc = 0.f;
    for (int k0 = 0; k0 < K; k0 += kT) {
        {
            const int am = blockIdx.y * kT + ty, ak = k0 + tx;
            As[ty][tx] = (am < M && ak < K) ? (TA ? A[(size_t)ak * lda + am] : A[(size_t)am * lda + ak]) : 0.f;
            const int bk = k0 + ty, bn = blockIdx.x * kT + tx;
            Bs[ty][tx] = (bk < K && bn < N) ? (TB ? B[(size_t)bn * ldb + bk] : B[(size_t)bk * ldb + bn]) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kT; ++k) acc = fmaf(As[ty][k], Bs[k][tx], acc);
        __syncthreads();
    }
    if (m < M && n < N) {
        float v = acc;
        if (EPI == 1) v += bias[n];
        if (EPI == 2) v = fmaxf(v + bias[n], 0.f);
        if (EPI == 3) v = R[(size_t)m * ldr + n] > 0.f ? v : 0.f;
        C[(size_t)m * ldc + n] = v;
    }
}

// rows idx[r] of (X standardised, Y, mask) into the batch buffers
__global__ void k_mlp_gather(int n, int in, int out, const int* __restrict__ idx, const float* __restrict__ X,
                             const float* __restrict__ Y, const float* __restrict__ Mk, const float* __restrict__ mean,
                             const float* __restrict__ scale, float* __restrict__ Xb, float* __restrict__ Yb,
                             float* __restrict__ Mb) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * (in + out); e += gridDim.x * blockDim.x) {
        const int r = e / (in + out), c = e % (in + out);
        const int src = idx ? idx[r] : r;
        if (c < in) {
            Xb[(size_t)r * in + c] = (X[(size_t)src * in + c] - mean[c]) * scale[c];
        } else if (Y) {
            const int k = c - in;
            Yb[(size_t)r * out + k] = Y[(size_t)src * out + k];
            Mb[(size_t)r * out + k] = Mk[(size_t)src * out + k];
        }
    }
}

// dP = 2 mask (P - Y) / count, loss += mask (P - Y)^2 / count
__global__ void k_mlp_loss(int total, const float* __restrict__ P, const float* __restrict__ Y,
                           const float* __restrict__ Mk, float inv_count, float* __restrict__ dP, float* loss) {
    float l = 0.f;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const float d = Mk[e] != 0.f ? P[e] - Y[e] : 0.f;
        dP[e] = 2.f * d * inv_count;
        l += d * d * inv_count;
    }
    l = warp_sum(l);
    if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, l);
}

// db[c] = sum_r dY[r][c]
__global__ void k_mlp_colsum(int n, int cols, const float* __restrict__ dY, float* __restrict__ db) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.f;
    for (int r = 0; r < n; ++r) s += dY[(size_t)r * cols + c];
    db[c] = s;
}

// Adam (bias-corrected first and second moments)
__global__ void k_mlp_adam(int np, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                           float* __restrict__ m2, float lr, float beta1, float beta2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = beta1 * m1[i] + (1.f - beta1) * gi;
        const float b = beta2 * m2[i] + (1.f - beta2) * gi * gi;
        m1[i] = a;
        m2[i] = b;
        p[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
    }
}

struct Mlp {
    int device = 0;
    cudaStream_t st = nullptr;
    int in = 0, h1 = 0, h2 = 0, out = 0;
    int np = 0;
    int oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0;
    DevBuf params, grads, mom1, mom2, mean, scale;
    DevBuf X, Y, Mk, idx, Xb, Yb, Mb, H1, H2, P, dP, dH2, dH1, loss;
    int cap_data = 0, cap_batch = 0;
    long long step = 0;
    int64_t launches = 0;

    ~Mlp() {
        if (device >= 0) cudaSetDevice(device);
        DevBuf* b[] = {&params, &grads, &mom1, &mom2, &mean, &scale, &X, &Y, &Mk, &idx, &Xb, &Yb, &Mb,
                       &H1, &H2, &P, &dP, &dH2, &dH1, &loss};
        for (DevBuf* d : b) d->release();
        if (st) cudaStreamDestroy(st);
    }

    int ensure_batch(int n) {
        if (n <= cap_batch) return 0;
        int rc;
        if ((rc = Xb.ensure(sizeof(float) * (size_t)n * in)) || (rc = Yb.ensure(sizeof(float) * (size_t)n * out)) ||
            (rc = Mb.ensure(sizeof(float) * (size_t)n * out)) || (rc = H1.ensure(sizeof(float) * (size_t)n * h1)) ||
            (rc = H2.ensure(sizeof(float) * (size_t)n * h2)) || (rc = P.ensure(sizeof(float) * (size_t)n * out)) ||
            (rc = dP.ensure(sizeof(float) * (size_t)n * out)) || (rc = dH2.ensure(sizeof(float) * (size_t)n * h2)) ||
            (rc = dH1.ensure(sizeof(float) * (size_t)n * h1)))
            return rc;
        cap_batch = n;
        return 0;
    }

    int upload_data(int n, const float* x, const float* y, const float* mk) {
        int rc;
        if ((rc = X.ensure(sizeof(float) * (size_t)n * in))) return rc;
        CUDA_TRY(cudaMemcpyAsync(X.p, x, sizeof(float) * (size_t)n * in, cudaMemcpyHostToDevice, st));
        if (y) {
            if ((rc = Y.ensure(sizeof(float) * (size_t)n * out)) || (rc = Mk.ensure(sizeof(float) * (size_t)n * out)))
                return rc;
            CUDA_TRY(cudaMemcpyAsync(Y.p, y, sizeof(float) * (size_t)n * out, cudaMemcpyHostToDevice, st));
            CUDA_TRY(cudaMemcpyAsync(Mk.p, mk, sizeof(float) * (size_t)n * out, cudaMemcpyHostToDevice, st));
        }
        return 0;
    }

    template <bool TA, bool TB, int EPI>
    void gemm(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
              const float* bias = nullptr, const float* R = nullptr, int ldr = 0) {
        dim3 grid((N + kT - 1) / kT, (M + kT - 1) / kT);
        k_mlp_gemm<TA, TB, EPI><<<grid, kT * kT, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, R, ldr);
        ++launches;
    }

    // batch buffers hold n standardised rows: forward into H1, H2, P
    void forward(int n) {
        const float* p = params.as<float>();
        gemm<false, true, 2>(n, h1, in, Xb.as<float>(), in, p + oW1, in, H1.as<float>(), h1, p + ob1);
        gemm<false, true, 2>(n, h2, h1, H1.as<float>(), h1, p + oW2, h1, H2.as<float>(), h2, p + ob2);
        gemm<false, true, 1>(n, out, h2, H2.as<float>(), h2, p + oW3, h2, P.as<float>(), out, p + ob3);
    }

    // loss gradient and backward pass into `grads`; loss accumulated into loss[slot]
    void backward(int n, float inv_count, int slot) {
        const float* p = params.as<float>();
        float* g = grads.as<float>();
        const int tot = n * out;
        k_mlp_loss<<<std::max(1, std::min(256, (tot + 255) / 256)), 256, 0, st>>>(
            tot, P.as<float>(), Yb.as<float>(), Mb.as<float>(), inv_count, dP.as<float>(), loss.as<float>() + slot);
        ++launches;
        gemm<true, false, 0>(out, h2, n, dP.as<float>(), out, H2.as<float>(), h2, g + oW3, h2);
        k_mlp_colsum<<<(out + 127) / 128, 128, 0, st>>>(n, out, dP.as<float>(), g + ob3);
        gemm<false, false, 3>(n, h2, out, dP.as<float>(), out, p + oW3, h2, dH2.as<float>(), h2, nullptr,
                              H2.as<float>(), h2);
        gemm<true, false, 0>(h2, h1, n, dH2.as<float>(), h2, H1.as<float>(), h1, g + oW2, h1);
        k_mlp_colsum<<<(h2 + 127) / 128, 128, 0, st>>>(n, h2, dH2.as<float>(), g + ob2);
        gemm<false, false, 3>(n, h1, h2, dH2.as<float>(), h2, p + oW2, h1, dH1.as<float>(), h1, nullptr,
                              H1.as<float>(), h1);
        gemm<true, false, 0>(h1, in, n, dH1.as<float>(), h1, Xb.as<float>(), in, g + oW1, in);
        k_mlp_colsum<<<(h1 + 127) / 128, 128, 0, st>>>(n, h1, dH1.as<float>(), g + ob1);
        launches += 3;
    }

    void gather(int n, const int* d_idx, bool with_targets) {
        const int tot = n * (in + out);
        k_mlp_gather<<<std::max(1, std::min(1024, (tot + 255) / 256)), 256, 0, st>>>(
            n, in, out, d_idx, X.as<float>(), with_targets ? Y.as<float>() : nullptr, Mk.as<float>(),
            mean.as<float>(), scale.as<float>(), Xb.as<float>(), Yb.as<float>(), Mb.as<float>());
        ++launches;
    }
};

}  // namespace sptrsv

using sptrsv::Mlp;

extern "C" {

int sptrsv_mlp_create(sptrsv_mlp* out, int device, int in, int h1, int h2, int nout, uint64_t seed) {
    using namespace sptrsv;
    if (!out) return SPTRSV_ERR_INVALID_ARG;
    *out = nullptr;
    if (in < 1 || h1 < 1 || h2 < 1 || nout < 1 || in > 4096 || h1 > 4096 || h2 > 4096 || nout > 4096)
        return SPTRSV_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        (void)cudaGetLastError();
        return SPTRSV_ERR_NO_DEVICE;
    }
    if (device < 0) CUDA_TRY(cudaGetDevice(&device));
    if (device >= ndev) return SPTRSV_ERR_INVALID_ARG;
    CUDA_TRY(cudaSetDevice(device));
    Mlp* m = new Mlp;
    m->device = device;
    m->in = in;
    m->h1 = h1;
    m->h2 = h2;
    m->out = nout;
    m->oW1 = 0;
    m->ob1 = h1 * in;
    m->oW2 = m->ob1 + h1;
    m->ob2 = m->oW2 + h2 * h1;
    m->oW3 = m->ob2 + h2;
    m->ob3 = m->oW3 + nout * h2;
    m->np = m->ob3 + nout;
    // He-uniform weights from mt19937_64(seed): W ~ U(-sqrt(6/fan_in), sqrt(6/fan_in)), biases 0
    std::vector<float> p(m->np, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int rows, int fan_in) {
        const double a = std::sqrt(6.0 / fan_in);
        for (int k = 0; k < rows * fan_in; ++k)
            p[off + k] = (float)(-a + 2.0 * a * ((double)(rng() >> 11) * (1.0 / 9007199254740992.0)));
    };
    fill(m->oW1, h1, in);
    fill(m->oW2, h2, h1);
    fill(m->oW3, nout, h2);
    std::vector<float> mean(in, 0.f), scale(in, 1.f);
    int rc = 0;
    cudaError_t er = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
    if (er != cudaSuccess) rc = set_cuda_error(er, "mlp stream");
    if (!rc && ((rc = m->params.ensure(sizeof(float) * m->np)) || (rc = m->grads.ensure(sizeof(float) * m->np)) ||
                (rc = m->mom1.ensure(sizeof(float) * m->np)) || (rc = m->mom2.ensure(sizeof(float) * m->np)) ||
                (rc = m->mean.ensure(sizeof(float) * in)) || (rc = m->scale.ensure(sizeof(float) * in)) ||
                (rc = m->loss.ensure(sizeof(float) * 4096))))
        ;
    if (!rc) {
        // stream-ordered: every later kernel runs on the network's non-blocking stream
        if (cudaMemcpyAsync(m->params.p, p.data(), sizeof(float) * m->np, cudaMemcpyHostToDevice, m->st) !=
                cudaSuccess ||
            cudaMemsetAsync(m->mom1.p, 0, sizeof(float) * m->np, m->st) != cudaSuccess ||
            cudaMemsetAsync(m->mom2.p, 0, sizeof(float) * m->np, m->st) != cudaSuccess ||
            cudaMemsetAsync(m->grads.p, 0, sizeof(float) * m->np, m->st) != cudaSuccess ||
            cudaMemcpyAsync(m->mean.p, mean.data(), sizeof(float) * in, cudaMemcpyHostToDevice, m->st) != cudaSuccess ||
            cudaMemcpyAsync(m->scale.p, scale.data(), sizeof(float) * in, cudaMemcpyHostToDevice, m->st) !=
                cudaSuccess ||
            cudaStreamSynchronize(m->st) != cudaSuccess)
            rc = SPTRSV_ERR_CUDA;
    }
    if (rc) {
        delete m;
        return rc;
    }
    *out = reinterpret_cast<sptrsv_mlp>(m);
    return 0;
}

int sptrsv_mlp_destroy(sptrsv_mlp mh) {
    Mlp* m = reinterpret_cast<Mlp*>(mh);
    if (!m) return SPTRSV_ERR_INVALID_ARG;
    delete m;
    return 0;
}

#define MH()                                                 \
    Mlp* m = reinterpret_cast<Mlp*>(mh);                     \
    if (!m) return SPTRSV_ERR_INVALID_ARG;                   \
    if (cudaSetDevice(m->device) != cudaSuccess) return SPTRSV_ERR_CUDA

int sptrsv_mlp_num_params(sptrsv_mlp mh) {
    Mlp* m = reinterpret_cast<Mlp*>(mh);
    return m ? m->np : -1;
}

int sptrsv_mlp_get_params(sptrsv_mlp mh, float* p) {
    MH();
    if (!p) return SPTRSV_ERR_INVALID_ARG;
    CUDA_TRY(cudaStreamSynchronize(m->st));
    CUDA_TRY(cudaMemcpy(p, m->params.p, sizeof(float) * m->np, cudaMemcpyDeviceToHost));
    return 0;
}

int sptrsv_mlp_set_params(sptrsv_mlp mh, const float* p) {
    MH();
    if (!p) return SPTRSV_ERR_INVALID_ARG;
    CUDA_TRY(cudaStreamSynchronize(m->st));
    CUDA_TRY(cudaMemcpyAsync(m->params.p, p, sizeof(float) * m->np, cudaMemcpyHostToDevice, m->st));
    CUDA_TRY(cudaMemsetAsync(m->mom1.p, 0, sizeof(float) * m->np, m->st));
    CUDA_TRY(cudaMemsetAsync(m->mom2.p, 0, sizeof(float) * m->np, m->st));
    CUDA_TRY(cudaStreamSynchronize(m->st));
    m->step = 0;
    return 0;
}

int sptrsv_mlp_set_norm(sptrsv_mlp mh, const float* mean, const float* scale) {
    MH();
    if (!mean || !scale) return SPTRSV_ERR_INVALID_ARG;
    CUDA_TRY(cudaStreamSynchronize(m->st));
    CUDA_TRY(cudaMemcpyAsync(m->mean.p, mean, sizeof(float) * m->in, cudaMemcpyHostToDevice, m->st));
    CUDA_TRY(cudaMemcpyAsync(m->scale.p, scale, sizeof(float) * m->in, cudaMemcpyHostToDevice, m->st));
    CUDA_TRY(cudaStreamSynchronize(m->st));
    return 0;
}

// One full-batch forward + backward on (x, y, mask) (host, row-major): the loss and the flat
// gradient of the parameters (no update).
int sptrsv_mlp_grad(sptrsv_mlp mh, int n, const float* x, const float* y, const float* mask, float* grad,
                    float* loss) {
    MH();
    if (n < 1 || !x || !y || !mask) return SPTRSV_ERR_INVALID_ARG;
    int rc;
    if ((rc = m->upload_data(n, x, y, mask)) || (rc = m->ensure_batch(n))) return rc;
    double cnt = 0.0;
    for (long long e = 0; e < (long long)n * m->out; ++e) cnt += mask[e] != 0.f;
    CUDA_TRY(cudaMemsetAsync(m->loss.p, 0, sizeof(float), m->st));
    m->gather(n, nullptr, true);
    m->forward(n);
    m->backward(n, cnt > 0 ? (float)(1.0 / cnt) : 0.f, 0);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(m->st));
    if (grad) CUDA_TRY(cudaMemcpy(grad, m->grads.p, sizeof(float) * m->np, cudaMemcpyDeviceToHost));
    if (loss) CUDA_TRY(cudaMemcpy(loss, m->loss.p, sizeof(float), cudaMemcpyDeviceToHost));
    return 0;
}

// Adam training on (x, y, mask) (host, row-major): `epochs` passes over a fresh mt19937_64(seed)
// shuffle each, mini-batches of `batch` rows; loss_out[e] = the mean batch loss of epoch e.
int sptrsv_mlp_train(sptrsv_mlp mh, int n, const float* x, const float* y, const float* mask, int epochs, int batch,
                     float lr, uint64_t seed, float* loss_out) {
    MH();
    if (n < 1 || !x || !y || !mask || epochs < 1 || epochs > 4096 || batch < 1) return SPTRSV_ERR_INVALID_ARG;
    batch = std::min(batch, n);
    int rc;
    if ((rc = m->upload_data(n, x, y, mask)) || (rc = m->ensure_batch(batch))) return rc;
    if ((rc = m->idx.ensure(sizeof(int) * (size_t)n * epochs))) return rc;
    // all epochs' shuffles up front (one upload), with every batch's inverse mask count
    std::mt19937_64 rng(seed);
    std::vector<int> perm((size_t)n * epochs);
    std::vector<int> cur(n);
    for (int i = 0; i < n; ++i) cur[i] = i;
    for (int e = 0; e < epochs; ++e) {
        for (int i = n - 1; i > 0; --i) std::swap(cur[i], cur[(size_t)(rng() % (uint64_t)(i + 1))]);
        std::memcpy(perm.data() + (size_t)e * n, cur.data(), sizeof(int) * n);
    }
    CUDA_TRY(cudaMemcpyAsync(m->idx.p, perm.data(), sizeof(int) * perm.size(), cudaMemcpyHostToDevice, m->st));
    CUDA_TRY(cudaMemsetAsync(m->loss.p, 0, sizeof(float) * epochs, m->st));
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    std::vector<int> nb(epochs, 0);
    for (int e = 0; e < epochs; ++e) {
        for (int r0 = 0; r0 < n; r0 += batch) {
            const int nbat = std::min(batch, n - r0);
            const int* id = perm.data() + (size_t)e * n + r0;
            double cnt = 0.0;
            for (int r = 0; r < nbat; ++r)
                for (int k = 0; k < m->out; ++k) cnt += mask[(size_t)id[r] * m->out + k] != 0.f;
            m->gather(nbat, m->idx.as<int>() + (size_t)e * n + r0, true);
            m->forward(nbat);
            m->backward(nbat, cnt > 0 ? (float)(1.0 / cnt) : 0.f, e);
            ++m->step;
            const float c1 = 1.f - powf(beta1, (float)m->step), c2 = 1.f - powf(beta2, (float)m->step);
            sptrsv::k_mlp_adam<<<std::max(1, std::min(256, (m->np + 255) / 256)), 256, 0, m->st>>>(
                m->np, m->params.as<float>(), m->grads.as<float>(), m->mom1.as<float>(), m->mom2.as<float>(), lr,
                beta1, beta2, eps, c1, c2);
            ++m->launches;
            ++nb[e];
        }
    }
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(m->st));
    if (loss_out) {
        CUDA_TRY(cudaMemcpy(loss_out, m->loss.p, sizeof(float) * epochs, cudaMemcpyDeviceToHost));
        for (int e = 0; e < epochs; ++e) loss_out[e] /= (float)std::max(1, nb[e]);
    }
    return 0;
}

// Predictions for n rows of x (host, row-major) into y (host, n x out).
int sptrsv_mlp_predict(sptrsv_mlp mh, int n, const float* x, float* y) {
    MH();
    if (n < 1 || !x || !y) return SPTRSV_ERR_INVALID_ARG;
    int rc;
    if ((rc = m->upload_data(n, x, nullptr, nullptr)) || (rc = m->ensure_batch(n))) return rc;
    m->gather(n, nullptr, false);
    m->forward(n);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(y, m->P.p, sizeof(float) * (size_t)n * m->out, cudaMemcpyDeviceToHost, m->st));
    CUDA_TRY(cudaStreamSynchronize(m->st));
    return 0;
}

int64_t sptrsv_mlp_launches(sptrsv_mlp mh) {
    Mlp* m = reinterpret_cast<Mlp*>(mh);
    return m ? m->launches : -1;
}

}  // extern "C"
