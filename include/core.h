/*
 * core.h -- the reference's CPU solver entry points, re-implemented on the GB300.
 *
 * Same names, C++ linkage and parameter types as xnd-r/SPTRSV include/core.h:10-19, so a
 * program built against the reference links against libsptrsv_gb300.so in place of
 * lib_SPTRSV for these symbols.  Each call copies its host arrays to the GPU, runs the
 * CUDA path and copies the result back.  Return value: the solve's device time in seconds
 * (CUDA events), or a negative sptrsv_status cast to double on failure (see
 * sptrsv_last_status() in sptrsv_gb300.h).  Layouts follow the reference: CSR with uint64
 * row pointer and the diagonal first in every row; X/B column-major (x[i + r*n]).
 * base_gauss_lower (core.h:9) solves the lower system as the reversed upper one (rows and
 * columns in reverse order), on the same GPU path.
 */
#ifndef SPTRSV_GB300_CORE_H
#define SPTRSV_GB300_CORE_H
#include <cstddef>
#include <cstdint>
#ifndef SPTRSV_API
#define SPTRSV_API __attribute__((visibility("default")))
#endif

/* core.h:9, core.cpp:4-16 -- forward substitution, x = L^{-1} b, one RHS; lower CSR with the
 * diagonal LAST in every row. */
SPTRSV_API double base_gauss_lower(int n, double* val, uint64_t* row_index, int* col, double* x, double* b);
/* core.h:10, core.cpp:18-32 -- backward substitution, x = U^{-1} b. */
SPTRSV_API double base_gauss_upper(int n, double* val, uint64_t* row_index, int* col, double* x, double* b, int rhs);
/* core.h:11, core.cpp:34-51 -- same solve (the RHS loop order has no GPU meaning). */
SPTRSV_API double base_gauss_upper_new(int n, double* val, uint64_t* row_index, int* col, double* x, double* b, int rhs);
/* core.h:12, core.cpp:80-92 -- supernodal solve in place: x holds b on entry.  `row` is the
 * CSR column index array and `col_index` the uint64 row pointer (the reference's naming). */
SPTRSV_API double supernodal_upper(size_t sn, int* supernodes, double* x, double* val, int* row, uint64_t* col_index, int n,
                        int rhs);
/* core.h:13, core.cpp:94-133 */
SPTRSV_API double supernodal_upper_new(size_t sn, int* supernodes, double* x, double* val, int* row, uint64_t* col_index,
                            int n, int rhs);
/* core.h:14, core.cpp:164-201 -- solve on the padded format made by ccs2ccs_pad.  By
 * position: padded values, uint64 padded column indices, int padded row pointer. */
SPTRSV_API double supernodal_blas_upper(int n, int nz, size_t sn, int* supernodes, double* x, double* val,
                             uint64_t* col_index, int* row, int rhs);
/* core.h:15, core.cpp:203-242 (marked "DOESN'T WORK" there) -- provided with the meaning of
 * supernodal_blas_upper over every RHS column. */
SPTRSV_API double supernodal_blas_upper_new(int n, int nz, size_t sn, int* supernodes, double* x, double* val,
                                 uint64_t* col_index, int* row, int rhs);
/* core.h:16, core.cpp:136-161 -- pad every supernode's triangle to a dense block. */
SPTRSV_API double ccs2ccs_pad(double* val, int* row, uint64_t* col_index, double* val_pad, uint64_t* col_index_pad,
                   int* row_pad, int* nodes, int& sn, int& nnz);
/* core.h:17, core.cpp:244-270 -- levels, bit-exact; returns the largest level. */
SPTRSV_API int setLevelUpAndGetMaxLevel(int n, int* col, uint64_t* row_index, uint64_t* levelsUp);
/* core.h:18, core.cpp:273-376 -- level-set solve (persistent kernel, grid barrier per level).
 * num_of_threads is accepted and ignored: the GPU sizes its own grid. */
SPTRSV_API double barrier_upper(int n, double* x, double* b, double* val, int* col, uint64_t* row, int num_of_threads,
                     int rhs);
/* core.h:19, core.cpp:378-483 */
SPTRSV_API double barrier_upper_new(int n, double* x, double* b, double* val, int* col, uint64_t* row, int num_of_threads,
                         int rhs);
#endif
