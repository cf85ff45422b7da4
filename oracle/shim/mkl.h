/* Minimal stand-in for MKL's CBLAS header, written for this project so that the
 * reference's src/core.cpp compiles unmodified into oracle/_ref.  Only the enums and the
 * two routines core.cpp calls (core.cpp:186, :193) are declared; cblas_naive.c defines
 * them with plain loops.  Test infrastructure only. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef enum { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;
void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n, int k,
                 double alpha, const double* a, int lda, const double* b, int ldb, double beta, double* c, int ldc);
void cblas_dtrsm(CBLAS_LAYOUT layout, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE ta, CBLAS_DIAG diag,
                 int m, int n, double alpha, const double* a, int lda, double* b, int ldb);
#ifdef __cplusplus
}
#endif
