/* Plain-loop dgemm / dtrsm for the row-major, no-transpose, left/upper/non-unit cases the
 * reference's core.cpp uses (core.cpp:186-194).  Test infrastructure only: it lets the
 * unmodified reference run as a CPU checker without MKL.  Any other case returns without
 * touching memory. */
#include "mkl.h"
void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n, int k,
                 double alpha, const double* a, int lda, const double* b, int ldb, double beta, double* c, int ldc) {
    if (layout != CblasRowMajor || ta != CblasNoTrans || tb != CblasNoTrans) return;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < n; ++j) {
            double acc = 0.0;
            for (int p = 0; p < k; ++p) acc += a[(long)i * lda + p] * b[(long)p * ldb + j];
            c[(long)i * ldc + j] = alpha * acc + beta * c[(long)i * ldc + j];
        }
}
void cblas_dtrsm(CBLAS_LAYOUT layout, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE ta, CBLAS_DIAG diag,
                 int m, int n, double alpha, const double* a, int lda, double* b, int ldb) {
    if (layout != CblasRowMajor || side != CblasLeft || uplo != CblasUpper || ta != CblasNoTrans) return;
    for (int j = 0; j < n; ++j)
        for (int i = m - 1; i >= 0; --i) {
            double s = alpha * b[(long)i * ldb + j];
            for (int p = i + 1; p < m; ++p) s -= a[(long)i * lda + p] * b[(long)p * ldb + j];
            b[(long)i * ldb + j] = (diag == CblasNonUnit) ? s / a[(long)i * lda + i] : s;
        }
}
