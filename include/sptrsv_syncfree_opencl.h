/*
 * sptrsv_syncfree_opencl.h -- the reference's GPU sync-free entry points, re-implemented in
 * CUDA for sm_103a (no OpenCL).  Same names and parameter types as xnd-r/SPTRSV
 * include/sptrsv_syncfree_opencl.h:11-37 (C++ linkage).
 *
 * As in the reference: m must equal n (else -1 is returned, sptrsv_syncfree_opencl.cpp:17-21);
 * x is zeroed on entry; the return value is the solve kernel's device time in seconds
 * (sptrsv_syncfree_opencl.cpp:360).  Failures return a negative sptrsv_status as a double.
 * Unlike the reference, the device is the current CUDA device (not hard-coded id 1), the spins
 * are bounded, and nothing exits the process.
 */
#ifndef SPTRSV_GB300_SYNCFREE_OPENCL_H
#define SPTRSV_GB300_SYNCFREE_OPENCL_H
#ifndef SPTRSV_API
#define SPTRSV_API __attribute__((visibility("default")))
#endif

/* :11-19 -- CSC of U (diagonal last in each column), rhs >= 1, X/B row-major (j*rhs + k,
 * kernel_full.cl:163).  CSC push with per-row in-degree counters. */
SPTRSV_API double sptrsv_syncfree_opencl(int* cscColPtrTR, int* cscRowIdxTR, double* cscValTR, int m, int n, int nnzTR,
                              double* x, double* b, int rhs);
/* :21-28 -- same, one RHS. */
SPTRSV_API double sptrsv_syncfree2_opencl(int* cscColPtrTR, int* cscRowIdxTR, const double* cscValTR, const int m,
                               const int n, const int nnzTR, double* x, const double* b);
/* :30-37 -- CSR (diagonal first), one RHS, one lane per row (kernel_full3.cl family). */
SPTRSV_API double sptrsv_syncfree3_opencl(int* csrColIdx, int* csrRowPtr, const double* csrVal, const int m, const int n,
                               const int nnz, double* x, const double* b);
#endif
