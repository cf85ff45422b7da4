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

// Upper Cholesky factor of the 2D 5-point Laplacian, band-by-band (row-oriented upper
// band Cholesky: U[i][j] = (A[i][j] - sum_k U[k][i] U[k][j]) / U[i][i]).
GEN_API void* sptrsv_gen_laplace2d_cholesky(int g) {
    if (g <= 0) return nullptr;
    const int64_t n = (int64_t)g * g;
    const int w = g + 1;  // band entries per row (diagonal included)
    std::vector<double> U((size_t)n * w, 0.0);  // U[i*w + d] = U(i, i+d)
    auto A = [&](int64_t i, int64_t j) -> double {
        if (i == j) return 4.0;
        int64_t d = j - i;
        if (d == 1 && (i % g) != g - 1) return -1.0;
        if (d == g) return -1.0;
        return 0.0;
    };
    for (int64_t i = 0; i < n; ++i) {
        int64_t jmax = std::min<int64_t>(i + g, n - 1);
        int64_t k0 = std::max<int64_t>(0, i - g);
        for (int64_t j = i; j <= jmax; ++j) {
            double s = A(i, j);
            // rows k with U(k,i) and U(k,j) both inside the band: k >= j - g
            for (int64_t k = std::max<int64_t>(k0, j - g); k < i; ++k)
                s -= U[(size_t)k * w + (i - k)] * U[(size_t)k * w + (j - k)];
            if (j == i) U[(size_t)i * w] = std::sqrt(s);
            else U[(size_t)i * w + (j - i)] = s / U[(size_t)i * w];
        }
    }
    Csr* m = new Csr;
    m->n = (int)n;
    m->row_ptr.resize(n + 1);
    m->row_ptr[0] = 0;
    for (int64_t i = 0; i < n; ++i) {
        int64_t jmax = std::min<int64_t>(i + g, n - 1);
        for (int64_t j = i; j <= jmax; ++j) {
            m->col.push_back((int)j);
            m->val.push_back(U[(size_t)i * w + (j - i)]);
        }
        m->row_ptr[i + 1] = (int64_t)m->col.size();
    }
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
