// A C++ caller written the way a program built against the reference's lib_SPTRSV calls it:
// it includes core.h and sptrsv_syncfree_opencl.h and links libsptrsv_gb300.so in their place.
// It builds a seeded upper-triangular CSR system (diagonal first in every row), solves it through
// base_gauss_upper (two column-major right-hand sides), barrier_upper, sptrsv_syncfree_opencl
// (CSC, row-major) and sptrsv_syncfree3_opencl (CSR), computes the levels, and checks every
// result against its own serial backward substitution and longest-path levels.
// Prints one line "dropin_caller ok ..." and exits 0, or names the failing call and exits 1.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

#include "core.h"
#include "sptrsv_syncfree_opencl.h"

static double max_rel(const std::vector<double>& x, const std::vector<double>& ref) {
    double scale = 0.0, worst = 0.0;
    for (double r : ref) scale = std::fmax(scale, std::fabs(r));
    for (size_t i = 0; i < x.size(); ++i)
        worst = std::fmax(worst, std::fabs(x[i] - ref[i]) / std::fmax(std::fabs(ref[i]), 1e-12 * scale));
    return worst;
}

int main() {
    const int n = 3000;
    std::mt19937_64 rng(11);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    std::uniform_int_distribution<int> near(1, 24);
    std::vector<uint64_t> rp(1, 0);
    std::vector<int> col;
    std::vector<double> val;
    for (int i = 0; i < n; ++i) {
        std::vector<int> cs;
        for (int k = 0; k < 5; ++k) {
            int c = i + near(rng);
            if (c < n) cs.push_back(c);
        }
        std::sort(cs.begin(), cs.end());
        cs.erase(std::unique(cs.begin(), cs.end()), cs.end());
        double off = 0.0;
        std::vector<double> vs;
        for (size_t k = 0; k < cs.size(); ++k) {
            vs.push_back(u(rng));
            off += std::fabs(vs.back());
        }
        col.push_back(i);
        val.push_back(1.0 + off);
        for (size_t k = 0; k < cs.size(); ++k) {
            col.push_back(cs[k]);
            val.push_back(vs[k]);
        }
        rp.push_back(col.size());
    }
    const int nnz = (int)col.size();
    const int rhs = 2;
    std::vector<double> b((size_t)n * rhs);
    for (double& v : b) v = u(rng);

    // serial backward substitution (column-major X) and longest-path levels
    std::vector<double> ref((size_t)n * rhs);
    for (int r = 0; r < rhs; ++r)
        for (int i = n - 1; i >= 0; --i) {
            double s = b[i + (size_t)r * n];
            for (uint64_t k = rp[i] + 1; k < rp[i + 1]; ++k) s -= val[k] * ref[col[k] + (size_t)r * n];
            ref[i + (size_t)r * n] = s / val[rp[i]];
        }
    std::vector<uint64_t> lv_ref(n);
    uint64_t ml_ref = 0;
    for (int i = n - 1; i >= 0; --i) {
        uint64_t m = 0;
        for (uint64_t k = rp[i] + 1; k < rp[i + 1]; ++k) m = std::max(m, lv_ref[col[k]]);
        lv_ref[i] = 1 + m;
        ml_ref = std::max(ml_ref, lv_ref[i]);
    }

    int fails = 0;
    double worst = 0.0;
    auto check = [&](const char* what, double secs, double err) {
        worst = std::fmax(worst, err);
        if (!(secs >= 0.0) || !(err <= 1e-10)) {
            std::printf("dropin_caller FAIL %s: returned %g, max elementwise error %g\n", what, secs, err);
            ++fails;
        }
    };

    std::vector<double> x((size_t)n * rhs, 0.0);
    check("base_gauss_upper", base_gauss_upper(n, val.data(), rp.data(), col.data(), x.data(), b.data(), rhs),
          max_rel(x, ref));
    std::fill(x.begin(), x.end(), 0.0);
    check("barrier_upper", barrier_upper(n, x.data(), b.data(), val.data(), col.data(), rp.data(), 4, rhs),
          max_rel(x, ref));

    std::vector<uint64_t> lv(n, 0);
    const int ml = setLevelUpAndGetMaxLevel(n, col.data(), rp.data(), lv.data());
    if (ml != (int)ml_ref || lv != lv_ref) {
        std::printf("dropin_caller FAIL setLevelUpAndGetMaxLevel: %d levels, expected %d\n", ml, (int)ml_ref);
        ++fails;
    }

    // CSC of U (rows ascending in each column, diagonal last) for the OpenCL-interface solve
    std::vector<int> cp(n + 1, 0), crow(nnz);
    std::vector<double> cval(nnz);
    for (int k = 0; k < nnz; ++k) cp[col[k] + 1]++;
    for (int j = 0; j < n; ++j) cp[j + 1] += cp[j];
    std::vector<int> fill(cp.begin(), cp.end() - 1);
    for (int i = 0; i < n; ++i)
        for (uint64_t k = rp[i]; k < rp[i + 1]; ++k) {
            const int d = fill[col[k]]++;
            crow[d] = i;
            cval[d] = val[k];
        }
    std::vector<double> b_rm((size_t)n * rhs), x_rm((size_t)n * rhs), ref_rm((size_t)n * rhs);
    for (int i = 0; i < n; ++i)
        for (int r = 0; r < rhs; ++r) {
            b_rm[(size_t)i * rhs + r] = b[i + (size_t)r * n];
            ref_rm[(size_t)i * rhs + r] = ref[i + (size_t)r * n];
        }
    check("sptrsv_syncfree_opencl",
          sptrsv_syncfree_opencl(cp.data(), crow.data(), cval.data(), n, n, nnz, x_rm.data(), b_rm.data(), rhs),
          max_rel(x_rm, ref_rm));
    if (sptrsv_syncfree_opencl(cp.data(), crow.data(), cval.data(), n, n + 1, nnz, x_rm.data(), b_rm.data(), rhs) != -1) {
        std::printf("dropin_caller FAIL sptrsv_syncfree_opencl: a non-square call did not return -1\n");
        ++fails;
    }

    std::vector<int> rp32(rp.begin(), rp.end());
    std::vector<double> x1(n), ref1(ref.begin(), ref.begin() + n);
    check("sptrsv_syncfree3_opencl",
          sptrsv_syncfree3_opencl(col.data(), rp32.data(), val.data(), n, n, nnz, x1.data(), b.data()),
          max_rel(x1, ref1));

    if (fails) return 1;
    std::printf("dropin_caller ok n=%d nnz=%d levels=%d max_elem_err=%.3g\n", n, nnz, ml, worst);
    return 0;
}
