// gen.cpp -- seeded synthetic upper-triangular systems (host C++, no CUDA).
//
// The reference ships no generator: its factors came from an external Cholesky code and
// its right-hand sides are all ones (utils.cpp:113-126).  These generators produce the
// workloads the solver is measured on:
//   * laplace2d_cholesky: the exact upper Cholesky factor U (A = U^T U) of the 5-point
//     Laplacian (diag 4, off -1) on a g x g grid in natural ordering, stored as a full
//     band (bandwidth g, explicit zeros kept): nnz = n(g+1) - g(g+1)/2;
//   * random_upper: n rows; row i draws k ~ Poisson(mean) off-diagonals, each at
//     i + U{1..band} with probability p_near, else at U{i+1..n-1}; columns >= n dropped,
//     duplicates merged; values U[-1,1]; diagonal = 1 + sum |off-diagonals|.
// Random numbers: std::mt19937_64 (bit-identical on every platform) with this file's own
// transforms, so x86 and Arm hosts build the same matrices:
//   u01 = (r >> 11) * 2^-53, uniform int in [lo,hi] = lo + r % (hi-lo+1),
//   Poisson by Knuth's product-of-uniforms method.
// Rows are generated in ascending order from one stream; the values of a row are drawn
// after its columns are sorted and merged.  All CSR output has the diagonal first.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <thread>
#include <random>
#include <vector>

#define GEN_API extern "C" __attribute__((visibility("default")))

namespace {

struct Csr {
    int n = 0;
    std::vector<int64_t> row_ptr;
    std::vector<int> col;
    std::vector<double> val;
};

inline double u01(std::mt19937_64& g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }
inline int64_t uint_in(std::mt19937_64& g, int64_t lo, int64_t hi) {
    return lo + (int64_t)(g() % (uint64_t)(hi - lo + 1));
}
inline int poisson(std::mt19937_64& g, double mean) {
    const double L = std::exp(-mean);
    int k = 0;
    double p = 1.0;
    do { ++k; p *= u01(g); } while (p > L);
    return k - 1;
}

}  // namespace

namespace {

// Upper Cholesky factor of the 2D 5-point Laplacian on a g x g grid, row by row:
//     U(i, i+d) = (A(i, i+d) - sum_{k<i} U(k,i) U(k, i+d)) / U(i,i),   U(i,i)^2 = A(i,i) - sum_k U(k,i)^2,
// written as a full band of g+1 entries per row (explicit zeros kept, clipped at n) into
// col/val from offset 0; returns nnz.  Row i is accumulated as A's row minus one scaled band row
// U(k, .) per earlier row k in [i-g, i), every element's sum taken in increasing k.  Rows are
// produced in blocks of kGenBlock: the earlier rows' updates are applied to the whole block while
// each band row is in cache, then the block's rows finish one after another with the updates from
// inside the block, which keeps the increasing-k order.  The last g + kGenBlock rows live in a
// ring of contiguous band rows.  The file is compiled without floating-point contraction, so x86
// and Arm round identically.
constexpr int kGenBlock = 8;

// u[d] -= alpha * r[d] for d < len (u and r never overlap)
inline void axpy_neg(double* __restrict__ u, const double* __restrict__ r, double alpha, int len) {
    for (int d = 0; d < len; ++d) u[d] -= alpha * r[d];
}

int64_t laplace2d_into(int g, int64_t* row_ptr, int* col, double* val) {
    const int64_t n = (int64_t)g * g;
    const int w = g + 1;
    const int slots = w + kGenBlock;
    std::vector<double> ring((size_t)slots * w, 0.0);  // slot (k mod slots): U(k, k+d) at entry d
    std::vector<double> ub((size_t)kGenBlock * w);
    auto update = [&](double* __restrict__ u, int64_t i, int64_t k) {
        const double* __restrict__ rk = ring.data() + (size_t)(k % slots) * w + (i - k);  // U(k, i + d) at rk[d]
        axpy_neg(u, rk, rk[0], (int)(k + g - i) + 1);
    };
    int64_t nz = 0;
    row_ptr[0] = 0;
    for (int64_t i0 = 0; i0 < n; i0 += kGenBlock) {
        const int B = (int)std::min<int64_t>(kGenBlock, n - i0);
        for (int q = 0; q < B; ++q) {
            const int64_t i = i0 + q;
            double* u = ub.data() + (size_t)q * w;
            std::fill(u, u + w, 0.0);
            u[0] = 4.0;
            if (1 < w && (i % g) != g - 1 && i + 1 < n) u[1] = -1.0;
            if (i + g < n) u[g] += -1.0;
        }
        for (int64_t k = std::max<int64_t>(0, i0 - g); k < i0; ++k)
            for (int q = 0; q < B; ++q)
                if (k >= i0 + q - g) update(ub.data() + (size_t)q * w, i0 + q, k);
        for (int q = 0; q < B; ++q) {
            const int64_t i = i0 + q;
            double* u = ub.data() + (size_t)q * w;
            for (int64_t k = i0; k < i; ++k) update(u, i, k);
            const double uii = std::sqrt(u[0]);
            double* ri = ring.data() + (size_t)(i % slots) * w;
            ri[0] = uii;
            for (int d = 1; d < w; ++d) ri[d] = i + d < n ? u[d] / uii : 0.0;
            const int64_t jmax = std::min<int64_t>(i + g, n - 1);
            for (int64_t j = i; j <= jmax; ++j) {
                col[nz] = (int)j;
                val[nz] = ri[j - i];
                ++nz;
            }
            row_ptr[i + 1] = nz;
        }
    }
    return nz;
}

int64_t laplace2d_nnz(int g) {
    const int64_t n = (int64_t)g * g;
    return n * (g + 1) - (int64_t)g * (g + 1) / 2;
}

}  // namespace

GEN_API void* sptrsv_gen_laplace2d_cholesky(int g) {
    if (g <= 0) return nullptr;
    const int64_t n = (int64_t)g * g;
    Csr* m = new Csr;
    m->n = (int)n;
    m->row_ptr.resize(n + 1);
    const int64_t nnz = laplace2d_nnz(g);
    m->col.resize(nnz);
    m->val.resize(nnz);
    laplace2d_into(g, m->row_ptr.data(), m->col.data(), m->val.data());
    return m;
}

GEN_API void* sptrsv_gen_random_upper(int n, double mean, double p_near, int band, uint64_t seed) {
    if (n <= 0 || band <= 0) return nullptr;
    std::mt19937_64 rng(seed);
    Csr* m = new Csr;
    m->n = n;
    m->row_ptr.resize((size_t)n + 1);
    m->row_ptr[0] = 0;
    m->col.reserve((size_t)n * (size_t)(mean + 2));
    m->val.reserve((size_t)n * (size_t)(mean + 2));
    std::vector<int64_t> cols;
    for (int64_t i = 0; i < n; ++i) {
        int k = poisson(rng, mean);
        cols.clear();
        for (int t = 0; t < k; ++t) {
            double u = u01(rng);
            int64_t j;
            if (u < p_near) {
                j = i + uint_in(rng, 1, band);
            } else {
                if (i + 1 > n - 1) continue;
                j = uint_in(rng, i + 1, n - 1);
            }
            if (j >= n) continue;
            cols.push_back(j);
        }
        std::sort(cols.begin(), cols.end());
        cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
        size_t diag_pos = m->col.size();
        m->col.push_back((int)i);
        m->val.push_back(0.0);
        double s = 0.0;
        for (int64_t j : cols) {
            double v = 2.0 * u01(rng) - 1.0;
            m->col.push_back((int)j);
            m->val.push_back(v);
            s += std::fabs(v);
        }
        m->val[diag_pos] = 1.0 + s;
        m->row_ptr[i + 1] = (int64_t)m->col.size();
    }
    return m;
}

// Random U with true supernode structure: supernodes of width U{wmin..wmax}; supernode
// [a, a+w) has a dense upper triangle and one shared set of k ~ Poisson(mean_rect) columns
// to its right (p_near of them within `band` of the block, the rest uniform), so row a+t
// holds w-t triangle entries followed by the shared columns -- the layout core.cpp:53-78 and
// ccs2ccs_pad (core.cpp:136-161) expect.  Values U[-1,1]; diagonal = 1 + sum |off-diagonals|.
// The partition is written to *snodes_out (malloc'd, sn+1 entries); *sn_out receives sn.
GEN_API void* sptrsv_gen_supernodal_random(int n, int wmin, int wmax, double mean_rect, double p_near, int band,
                                           uint64_t seed, int** snodes_out, int* sn_out) {
    if (n <= 0 || wmin < 1 || wmax < wmin) return nullptr;
    std::mt19937_64 rng(seed);
    std::vector<int> nodes{0};
    while (nodes.back() < n) {
        int w = (int)uint_in(rng, wmin, wmax);
        nodes.push_back(std::min(n, nodes.back() + w));
    }
    Csr* m = new Csr;
    m->n = n;
    m->row_ptr.assign((size_t)n + 1, 0);
    std::vector<int64_t> rect;
    for (size_t s = 0; s + 1 < nodes.size(); ++s) {
        const int a = nodes[s], b = nodes[s + 1];
        const int k = poisson(rng, mean_rect);
        rect.clear();
        for (int t = 0; t < k; ++t) {
            int64_t j;
            if (u01(rng) < p_near) j = b - 1 + uint_in(rng, 1, band);
            else { if (b > n - 1) continue; j = uint_in(rng, b, n - 1); }
            if (j >= n) continue;
            rect.push_back(j);
        }
        std::sort(rect.begin(), rect.end());
        rect.erase(std::unique(rect.begin(), rect.end()), rect.end());
        for (int i = a; i < b; ++i) {
            size_t diag_pos = m->col.size();
            m->col.push_back(i);
            m->val.push_back(0.0);
            double sum = 0.0;
            for (int j = i + 1; j < b; ++j) {
                double v = 2.0 * u01(rng) - 1.0;
                m->col.push_back(j);
                m->val.push_back(v);
                sum += std::fabs(v);
            }
            for (int64_t j : rect) {
                double v = 2.0 * u01(rng) - 1.0;
                m->col.push_back((int)j);
                m->val.push_back(v);
                sum += std::fabs(v);
            }
            m->val[diag_pos] = 1.0 + sum;
            m->row_ptr[i + 1] = (int64_t)m->col.size();
        }
    }
    *sn_out = (int)nodes.size() - 1;
    *snodes_out = (int*)std::malloc(sizeof(int) * nodes.size());
    std::memcpy(*snodes_out, nodes.data(), sizeof(int) * nodes.size());
    return m;
}

GEN_API void sptrsv_gen_free_ints(int* p) { std::free(p); }

GEN_API int sptrsv_gen_n(void* h) { return h ? ((Csr*)h)->n : -1; }
GEN_API int64_t sptrsv_gen_nnz(void* h) { return h ? (int64_t)((Csr*)h)->col.size() : -1; }

GEN_API void sptrsv_gen_copy(void* h, int64_t* row_ptr, int* col, double* val) {
    Csr* m = (Csr*)h;
    std::memcpy(row_ptr, m->row_ptr.data(), sizeof(int64_t) * m->row_ptr.size());
    std::memcpy(col, m->col.data(), sizeof(int) * m->col.size());
    std::memcpy(val, m->val.data(), sizeof(double) * m->val.size());
}

GEN_API void sptrsv_gen_free(void* h) { delete (Csr*)h; }

// count values U[lo,hi] from mt19937_64(seed), in order.
GEN_API void sptrsv_gen_uniform(uint64_t seed, int64_t count, double lo, double hi, double* out) {
    std::mt19937_64 rng(seed);
    for (int64_t i = 0; i < count; ++i) out[i] = lo + (hi - lo) * u01(rng);
}

// b = U x for rhs column-major columns (FP64, CSR order of summation).
GEN_API void sptrsv_gen_spmv(int n, const int64_t* row_ptr, const int* col, const double* val, const double* x,
                             double* b, int rhs) {
    for (int r = 0; r < rhs; ++r) {
        const double* xr = x + (size_t)r * n;
        double* br = b + (size_t)r * n;
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) s += val[k] * xr[col[k]];
            br[i] = s;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// The batched uneven mix: `count` independent systems in one packed host arena.
// Per system s (drawn in order from one mt19937_64(seed) stream):
//   n    = round(exp(ln nmin + u (ln nmax - ln nmin)))            (log-uniform)
//   kind = s mod 2: 0 -> laplace2d_cholesky(g), g = round(sqrt(n)), n = g^2;
//                   1 -> random_upper(n, mean, 0.9, 64, sseed), mean = mlo + u (mhi - mlo)
//   rhs  = U{1..rhs_max};  sseed, xseed = the next two raw draws
// x* (row-major n x rhs) = U[-1,1] from mt19937_64(xseed); b = U x* in FP64 (CSR order).
// Packed layout: row_ptr holds each system's local row pointer (n+1 entries, from 0) one after
// another; col/val likewise; x*/b one system after another.  The matrices are built on
// `threads` host threads, largest first; the result does not depend on the thread count.
namespace {

struct Mix {
    std::vector<int> n, rhs, kind;
    std::vector<double> mean;
    std::vector<uint64_t> sseed, xseed;
    std::vector<int64_t> nnz, rp_off, nz_off, xb_off;
    std::vector<int64_t> row_ptr;
    std::vector<int> col;
    std::vector<double> val, xstar, b;
};

template <typename F>
void parallel_for(int count, int threads, const std::vector<int>& order, F f) {
    std::atomic<int> next{0};
    auto work = [&]() {
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= count) return;
            f(order[k]);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
}

}  // namespace

GEN_API void* sptrsv_gen_mix(int count, uint64_t seed, int nmin, int nmax, double mlo, double mhi, int rhs_max,
                             int threads) {
    if (count <= 0 || nmin < 4 || nmax < nmin || rhs_max < 1 || mlo < 0 || mhi < mlo) return nullptr;
    if (threads < 1) threads = 1;
    std::mt19937_64 rng(seed);
    Mix* M = new Mix;
    M->n.resize(count); M->rhs.resize(count); M->kind.resize(count); M->mean.assign(count, 0.0);
    M->sseed.assign(count, 0); M->xseed.resize(count);
    M->nnz.resize(count); M->rp_off.resize(count + 1); M->nz_off.resize(count + 1); M->xb_off.resize(count + 1);
    const double l0 = std::log((double)nmin), l1 = std::log((double)nmax);
    for (int s = 0; s < count; ++s) {
        int n = (int)std::llround(std::exp(l0 + u01(rng) * (l1 - l0)));
        M->kind[s] = s % 2;
        if (M->kind[s] == 0) {
            const int g = std::max(2, (int)std::llround(std::sqrt((double)n)));
            n = g * g;
        } else {
            M->mean[s] = mlo + u01(rng) * (mhi - mlo);
        }
        M->n[s] = n;
        M->rhs[s] = (int)uint_in(rng, 1, rhs_max);
        M->sseed[s] = rng();
        M->xseed[s] = rng();
    }
    // random systems first (their nnz is known only once built), each into its own Csr
    std::vector<Csr*> rnd(count, nullptr);
    std::vector<int> order(count);
    for (int s = 0; s < count; ++s) order[s] = s;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return M->n[a] > M->n[b]; });
    std::vector<int> rorder;
    for (int s : order) if (M->kind[s] == 1) rorder.push_back(s);
    parallel_for((int)rorder.size(), threads, rorder, [&](int s) {
        rnd[s] = (Csr*)sptrsv_gen_random_upper(M->n[s], M->mean[s], 0.9, 64, M->sseed[s]);
    });
    M->rp_off[0] = M->nz_off[0] = M->xb_off[0] = 0;
    for (int s = 0; s < count; ++s) {
        const int g = (int)std::llround(std::sqrt((double)M->n[s]));
        M->nnz[s] = M->kind[s] == 0 ? laplace2d_nnz(g) : (int64_t)rnd[s]->col.size();
        M->rp_off[s + 1] = M->rp_off[s] + M->n[s] + 1;
        M->nz_off[s + 1] = M->nz_off[s] + M->nnz[s];
        M->xb_off[s + 1] = M->xb_off[s] + (int64_t)M->n[s] * M->rhs[s];
    }
    M->row_ptr.resize(M->rp_off[count]);
    M->col.resize(M->nz_off[count]);
    M->val.resize(M->nz_off[count]);
    M->xstar.resize(M->xb_off[count]);
    M->b.resize(M->xb_off[count]);
    parallel_for(count, threads, order, [&](int s) {
        int64_t* rp = M->row_ptr.data() + M->rp_off[s];
        int* col = M->col.data() + M->nz_off[s];
        double* val = M->val.data() + M->nz_off[s];
        if (M->kind[s] == 0) {
            laplace2d_into((int)std::llround(std::sqrt((double)M->n[s])), rp, col, val);
        } else {
            Csr* c = rnd[s];
            std::memcpy(rp, c->row_ptr.data(), sizeof(int64_t) * c->row_ptr.size());
            std::memcpy(col, c->col.data(), sizeof(int) * c->col.size());
            std::memcpy(val, c->val.data(), sizeof(double) * c->val.size());
            delete c;
        }
        const int n = M->n[s], r = M->rhs[s];
        double* xs = M->xstar.data() + M->xb_off[s];
        double* bb = M->b.data() + M->xb_off[s];
        std::mt19937_64 xr(M->xseed[s]);
        for (int64_t k = 0; k < (int64_t)n * r; ++k) xs[k] = 2.0 * u01(xr) - 1.0;
        std::vector<double> acc(r);
        for (int i = 0; i < n; ++i) {
            std::fill(acc.begin(), acc.end(), 0.0);
            for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
                const double v = val[k];
                const double* xc = xs + (size_t)col[k] * r;
                for (int c = 0; c < r; ++c) acc[c] += v * xc[c];
            }
            for (int c = 0; c < r; ++c) bb[(size_t)i * r + c] = acc[c];
        }
    });
    return M;
}

// Pointers into the mix (owned by it) and their element counts:
// 0 n(int) 1 rhs(int) 2 kind(int) 3 nnz(int64) 4 rp_off 5 nz_off 6 xb_off (int64, count+1)
// 7 row_ptr(int64) 8 col(int) 9 val 10 xstar 11 b (double) 12 mean (double)
GEN_API int sptrsv_gen_mix_array(void* h, int which, void** ptr, int64_t* len) {
    Mix* M = (Mix*)h;
    if (!M || !ptr || !len) return -1;
    switch (which) {
        case 0: *ptr = M->n.data(); *len = (int64_t)M->n.size(); break;
        case 1: *ptr = M->rhs.data(); *len = (int64_t)M->rhs.size(); break;
        case 2: *ptr = M->kind.data(); *len = (int64_t)M->kind.size(); break;
        case 3: *ptr = M->nnz.data(); *len = (int64_t)M->nnz.size(); break;
        case 4: *ptr = M->rp_off.data(); *len = (int64_t)M->rp_off.size(); break;
        case 5: *ptr = M->nz_off.data(); *len = (int64_t)M->nz_off.size(); break;
        case 6: *ptr = M->xb_off.data(); *len = (int64_t)M->xb_off.size(); break;
        case 7: *ptr = M->row_ptr.data(); *len = (int64_t)M->row_ptr.size(); break;
        case 8: *ptr = M->col.data(); *len = (int64_t)M->col.size(); break;
        case 9: *ptr = M->val.data(); *len = (int64_t)M->val.size(); break;
        case 10: *ptr = M->xstar.data(); *len = (int64_t)M->xstar.size(); break;
        case 11: *ptr = M->b.data(); *len = (int64_t)M->b.size(); break;
        case 12: *ptr = M->mean.data(); *len = (int64_t)M->mean.size(); break;
        default: return -1;
    }
    return 0;
}

GEN_API void sptrsv_gen_mix_free(void* h) { delete (Mix*)h; }
