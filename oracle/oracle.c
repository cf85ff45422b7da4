/*
 * oracle.c -- CPU restatement of the reference's sparse upper-triangular solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product: only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs load it.  The
 * shipped library (sptrsv_gb300/csrc) never links or calls it.
 *
 * Each function restates one routine of xnd-r/SPTRSV and cites the file:line it follows.
 * Conventions kept from the reference:
 *   - CSR of U with the diagonal FIRST in every row; row_index is uint64 (core.h:10);
 *   - X and B column-major, x[i + rh*n] (core.cpp:26-28);
 *   - CSC (for the sync-free interface) with the diagonal LAST in every column
 *     (kernel_full.cl:82).
 * Parity is pinned against the reference core.cpp compiled unmodified (oracle/_ref,
 * built by oracle/build_ref.sh) on the shipped txt fixtures and on seeded matrices;
 * tests/golden holds the vectors that build produced.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_API __attribute__((visibility("default")))

/* core.cpp:18-32  base_gauss_upper: serial backward substitution, RHS loop outermost.
 * The last row uses val[row_index[n]-1] (its only entry); every other row divides by the
 * first entry of its CSR row. */
ORC_API void orc_base_gauss_upper(int n, const double* val, const uint64_t* row_index, const int* col,
                                  double* x, const double* b, int rhs) {
    for (int rh = 0; rh < rhs; ++rh) {
        const size_t off = (size_t)rh * (size_t)n;
        x[off + n - 1] = b[off + n - 1] / val[row_index[n] - 1];
        for (int ir = n - 2; ir >= 0; --ir) {
            double sum = 0.0;
            for (uint64_t j = row_index[ir] + 1; j < row_index[ir + 1]; ++j)
                sum += val[j] * x[(size_t)col[j] + off];
            x[off + ir] = (b[off + ir] - sum) / val[row_index[ir]];
        }
    }
}

/* NOT a restatement of a reference routine: core.cpp:18-32 with every row sum taken in the
 * opposite order (largest column first).  Two correct FP64 solves that differ only in summation
 * order lie this far apart; the tests use it to measure that floor on a given system. */
ORC_API void orc_base_gauss_upper_rev(int n, const double* val, const uint64_t* row_index, const int* col,
                                      double* x, const double* b, int rhs) {
    for (int rh = 0; rh < rhs; ++rh) {
        const size_t off = (size_t)rh * (size_t)n;
        for (int ir = n - 1; ir >= 0; --ir) {
            double sum = 0.0;
            for (uint64_t j = row_index[ir + 1]; j-- > row_index[ir] + 1;) sum += val[j] * x[(size_t)col[j] + off];
            x[off + ir] = (b[off + ir] - sum) / val[row_index[ir]];
        }
    }
}

/* Elementwise error measured against the size of what each component is computed from:
 * max_i |x_i - x_ref_i| / max(|x_ref_i|, (|b_i| + sum_j |U_ij x_ref_j|) / |U_ii|), j over the
 * off-diagonals of row i, column-major RHS blocks.  Where x_ref_i is small because the row's
 * terms nearly cancel, rounding in any summation order is relative to the terms, not to
 * x_ref_i; this denominator follows that with no free constant. */
ORC_API double orc_term_rel_error(int n, const double* val, const uint64_t* row_index, const int* col,
                                  const double* x_ref, const double* x, const double* b, int rhs) {
    double worst = 0.0;
    for (int rh = 0; rh < rhs; ++rh) {
        const size_t off = (size_t)rh * (size_t)n;
        for (int i = 0; i < n; ++i) {
            double mag = fabs(b[off + i]);
            for (uint64_t j = row_index[i] + 1; j < row_index[i + 1]; ++j) mag += fabs(val[j] * x_ref[off + col[j]]);
            mag /= fabs(val[row_index[i]]);
            const double r = fabs(x_ref[off + i]);
            const double den = r > mag ? r : mag;
            const double e = fabs(x[off + i] - x_ref[off + i]) / (den > 1e-300 ? den : 1e-300);
            if (e > worst) worst = e;
        }
    }
    return worst;
}

/* core.cpp:4-16  base_gauss_lower: forward substitution for lower-triangular CSR with the
 * diagonal LAST in every row; one right-hand side.  Row 0 divides by val[col[0]] as the
 * reference does (its only entry when col[0] = 0). */
ORC_API void orc_base_gauss_lower(int n, const double* val, const uint64_t* row_index, const int* col, double* x,
                                  const double* b) {
    x[0] = b[0] / val[col[0]];
    for (int ir = 1; ir < n; ++ir) {
        double sum = 0.0;
        for (uint64_t j = row_index[ir]; j < row_index[ir + 1] - 1; ++j) sum += val[j] * x[col[j]];
        x[ir] = (b[ir] - sum) / val[row_index[ir + 1] - 1];
    }
}

/* core.cpp:34-51  base_gauss_upper_new: same arithmetic, RHS loop inside the row loop. */
ORC_API void orc_base_gauss_upper_new(int n, const double* val, const uint64_t* row_index, const int* col,
                                      double* x, const double* b, int rhs) {
    for (int rh = 0; rh < rhs; ++rh) {
        const size_t off = (size_t)rh * (size_t)n;
        x[off + n - 1] = b[off + n - 1] / val[row_index[n] - 1];
    }
    for (int ir = n - 2; ir >= 0; --ir) {
        for (int rh = 0; rh < rhs; ++rh) {
            const size_t off = (size_t)rh * (size_t)n;
            double sum = 0.0;
            for (uint64_t j = row_index[ir] + 1; j < row_index[ir + 1]; ++j)
                sum += val[j] * x[(size_t)col[j] + off];
            x[off + ir] = (b[off + ir] - sum) / val[row_index[ir]];
        }
    }
}

/* core.cpp:244-270  setLevelUpAndGetMaxLevel.  level[i] = 1 for a row holding only its
 * diagonal, else 1 + max(1, max_j level[col[j]]) over the row's off-diagonal entries.
 * Rows are scanned from n-1 down to 0; the return value is the largest level. */
ORC_API int orc_set_levels(int n, const int* col, const uint64_t* row_index, uint64_t* levels) {
    for (int i = 0; i < n; ++i) levels[i] = 1;
    int maxl = 1;
    for (int i = n - 1; i >= 0; --i) {
        uint64_t m = 1;
        if (row_index[i + 1] - row_index[i] > 1) {
            for (uint64_t j = row_index[i] + 1; j < row_index[i + 1]; ++j)
                if (levels[col[j]] > m) m = levels[col[j]];
            levels[i] += m;
        }
        if (levels[i] > (uint64_t)maxl) maxl = (int)levels[i];
    }
    return maxl;
}

/* core.cpp:282-288  rowsByLevel: rows bucketed by level, ascending inside a level.
 * Output is flattened: level_ptr[l] .. level_ptr[l+1] index level_rows for level l,
 * l = 0..max_level (level 0 is always empty). */
ORC_API void orc_level_buckets(int n, const uint64_t* levels, int max_level, int* level_ptr, int* level_rows) {
    memset(level_ptr, 0, sizeof(int) * (size_t)(max_level + 2));
    for (int i = 0; i < n; ++i) level_ptr[levels[i] + 1]++;
    for (int l = 0; l <= max_level; ++l) level_ptr[l + 1] += level_ptr[l];
    int* fill = (int*)malloc(sizeof(int) * (size_t)(max_level + 1));
    memcpy(fill, level_ptr, sizeof(int) * (size_t)(max_level + 1));
    for (int i = 0; i < n; ++i) level_rows[fill[levels[i]]++] = i;
    free(fill);
}

/* core.cpp:289-332  tasksByLevel: a greedy nnz-balanced split of each level's rows into
 * num_threads tasks, then prefix-summed.  tasks is (max_level+1) x (num_threads+1). */
ORC_API void orc_level_tasks(int max_level, const int* level_ptr, const int* level_rows,
                             const uint64_t* row_index, int num_threads, int* tasks) {
    for (int l = 0; l <= max_level; ++l) {
        int* t = tasks + (size_t)l * (size_t)(num_threads + 1);
        uint64_t level_nz = 0;
        for (int k = level_ptr[l]; k < level_ptr[l + 1]; ++k) {
            int v = level_rows[k];
            level_nz += row_index[v + 1] - row_index[v];
        }
        uint64_t limit = level_nz / (uint64_t)num_threads;
        int cur = 1;
        uint64_t cur_nz = 0;
        for (int j = 0; j <= num_threads; ++j) t[j] = 0;
        for (int k = level_ptr[l]; k < level_ptr[l + 1]; ++k) {
            int v = level_rows[k];
            uint64_t len = row_index[v + 1] - row_index[v];
            if (cur == num_threads) { t[cur] += 1; continue; }
            if (len + cur_nz > limit) { cur_nz = len; cur++; t[cur] += 1; }
            else { t[cur] += 1; cur_nz += len; }
        }
        for (int j = 1; j <= num_threads; ++j) t[j] += t[j - 1];
    }
}

/* core.cpp:273-376  barrier_upper: level-set solve.  Levels 1..max in order; inside a
 * level the rows of each task are solved by one OpenMP thread; the implicit barrier of
 * the `omp for` separates levels.  Each row's arithmetic equals base_gauss_upper's.
 * The analysis (levels, buckets, tasks) is done by the caller with the functions above. */
ORC_API void orc_barrier_solve(int n, double* x, const double* b, const double* val, const int* col,
                               const uint64_t* row, int max_level, const int* level_ptr,
                               const int* level_rows, const int* tasks, int num_threads, int rhs,
                               int rhs_inner) {
#ifdef _OPENMP
    omp_set_num_threads(num_threads);
#endif
    if (!rhs_inner) {
        for (int bi = 0; bi < rhs; ++bi) {
            const size_t off = (size_t)bi * (size_t)n;
#pragma omp parallel
            for (int l = 1; l <= max_level; ++l) {
                const int* t = tasks + (size_t)l * (size_t)(num_threads + 1);
                const int* rows = level_rows + level_ptr[l];
#pragma omp for schedule(static, 1)
                for (int tk = 0; tk < num_threads; ++tk) {
                    for (int j = t[tk]; j < t[tk + 1]; ++j) {
                        int v = rows[j];
                        double sum = 0.0;
                        for (uint64_t k = row[v] + 1; k < row[v + 1]; ++k) sum += val[k] * x[(size_t)col[k] + off];
                        x[(size_t)v + off] = (b[(size_t)v + off] - sum) / val[row[v]];
                    }
                }
            }
        }
    } else {
        /* core.cpp:378-483 barrier_upper_new: RHS loop inside the row. */
#pragma omp parallel
        for (int l = 1; l <= max_level; ++l) {
            const int* t = tasks + (size_t)l * (size_t)(num_threads + 1);
            const int* rows = level_rows + level_ptr[l];
#pragma omp for schedule(static, 1)
            for (int tk = 0; tk < num_threads; ++tk) {
                for (int j = t[tk]; j < t[tk + 1]; ++j) {
                    int v = rows[j];
                    for (int bi = 0; bi < rhs; ++bi) {
                        const size_t off = (size_t)bi * (size_t)n;
                        double sum = 0.0;
                        for (uint64_t k = row[v] + 1; k < row[v + 1]; ++k) sum += val[k] * x[(size_t)col[k] + off];
                        x[(size_t)v + off] = (b[(size_t)v + off] - sum) / val[row[v]];
                    }
                }
            }
        }
    }
}

/* kernel_full.cl:40-52  analyser: in_degree[rowidx[k]] += 1 over every CSC entry, the
 * diagonal included, so in_degree[i] equals the number of entries of row i. */
ORC_API void orc_in_degree_csc(int n, int nnz, const int* csc_row_idx, int* in_degree) {
    memset(in_degree, 0, sizeof(int) * (size_t)n);
    for (int k = 0; k < nnz; ++k) in_degree[csc_row_idx[k]]++;
}

/* utils.cpp:128-159  transpose: CSR -> CSC by count / prefix / scatter.  Column j of the
 * result lists its rows in ascending order, so the diagonal of U lands last. */
ORC_API void orc_transpose(int n, uint64_t nz, const double* val, const int* col, const uint64_t* row_index,
                           double* val_t, uint64_t* row_t, int* col_index_t) {
    memset(col_index_t, 0, sizeof(int) * (size_t)(n + 1));
    for (uint64_t i = 0; i < nz; ++i) col_index_t[col[i] + 1]++;
    int S = 0;
    for (int i = 1; i <= n; ++i) { int tmp = col_index_t[i]; col_index_t[i] = S; S += tmp; }
    for (int i = 0; i < n; ++i) {
        for (uint64_t j = row_index[i]; j < row_index[i + 1]; ++j) {
            int dst = col_index_t[col[j] + 1]++;
            val_t[dst] = val[j];
            row_t[dst] = (uint64_t)i;
        }
    }
}

/* kernel_full.cl:54-124 / :126-228 (sequential meaning)  Column-oriented backward
 * substitution on the CSC of U: columns in reverse; x_j = (b_j - left_sum_j) / U_jj with
 * U_jj the last entry of column j; then left_sum_i += x_j * U_ij for the column's other
 * entries.  X and B row-major (pos = j*rhs + k, kernel_full.cl:163). */
ORC_API void orc_syncfree_csc(int n, const int* col_ptr, const int* row_idx, const double* val,
                              double* x, const double* b, int rhs) {
    double* left = (double*)calloc((size_t)n * (size_t)rhs, sizeof(double));
    for (int j = n - 1; j >= 0; --j) {
        const int start = col_ptr[j], stop = col_ptr[j + 1] - 1;
        const double d = val[stop];
        for (int k = 0; k < rhs; ++k) {
            size_t p = (size_t)j * rhs + k;
            x[p] = (b[p] - left[p]) / d;
        }
        for (int e = stop - 1; e >= start; --e) {
            const int i = row_idx[e];
            for (int k = 0; k < rhs; ++k) left[(size_t)i * rhs + k] += x[(size_t)j * rhs + k] * val[e];
        }
    }
    free(left);
}

/* core.cpp:53-65  get_tr_part_upper: in-place solve of a supernode's dense triangle.
 * Row isn+dim-1 is divided by its diagonal; each earlier row j subtracts the `cnt+1`
 * entries right of its diagonal (the triangle part) and divides. */
static void tr_part(int isn, int dim, double* x, const double* val, const int* row, const uint64_t* colp, size_t gs) {
    x[gs + isn + dim - 1] = x[gs + isn + dim - 1] / val[colp[isn + dim - 1]];
    int cnt = 0;
    for (int j = isn + dim - 2; j >= isn; --j) {
        double sum = 0.0;
        for (uint64_t k = colp[j] + 1; k <= colp[j] + 1 + (uint64_t)cnt; ++k) sum += val[k] * x[gs + row[k]];
        x[gs + j] = (x[gs + j] - sum) / val[colp[j]];
        cnt++;
    }
}

/* core.cpp:67-78  get_rect_part_upper: x_s -= R_s x_rect, where row isn+cnt's rectangle
 * starts `dim-cnt` entries into the row (after its part of the triangle). */
static void rect_part(int isn, int dim, double* x, const double* val, const int* row, const uint64_t* colp, size_t gs) {
    int cnt = 0;
    for (int i = isn; i < isn + dim; ++i) {
        double sum = 0.0;
        for (uint64_t j = colp[i] + (uint64_t)(dim - cnt); j < colp[i + 1]; ++j) sum += val[j] * x[gs + row[j]];
        x[gs + i] -= sum;
        cnt++;
    }
}

/* core.cpp:80-92  supernodal_upper: per RHS, supernodes in reverse, rectangle update then
 * triangle solve, in place on x (x holds b on entry).  The reference passes the CSR column
 * indices as `row` and the uint64 row pointer as `col_index`. */
ORC_API void orc_supernodal_upper(size_t sn, const int* supernodes, double* x, const double* val,
                                  const int* row, const uint64_t* col_index, int n, int rhs) {
    for (int rh = 0; rh < rhs; ++rh) {
        size_t gs = (size_t)rh * (size_t)n;
        for (int i = (int)sn - 1; i >= 0; --i) {
            int isn = supernodes[i], dim = supernodes[i + 1] - supernodes[i];
            rect_part(isn, dim, x, val, row, col_index, gs);
            tr_part(isn, dim, x, val, row, col_index, gs);
        }
    }
}

/* core.cpp:94-133  supernodal_upper_new: supernode loop outermost, RHS loop inside. */
ORC_API void orc_supernodal_upper_new(size_t sn, const int* supernodes, double* x, const double* val,
                                      const int* row, const uint64_t* col_index, int n, int rhs) {
    for (int s = (int)sn - 1; s >= 0; --s) {
        int isn = supernodes[s], dim = supernodes[s + 1] - supernodes[s];
        int cnt = 0;
        for (int i = isn; i < isn + dim; ++i) {
            for (int rh = 0; rh < rhs; ++rh) {
                double sum = 0.0;
                for (uint64_t j = col_index[i] + (uint64_t)(dim - cnt); j < col_index[i + 1]; ++j)
                    sum += val[j] * x[(size_t)rh * n + row[j]];
                x[(size_t)rh * n + i] -= sum;
            }
            cnt++;
        }
        for (int rh = 0; rh < rhs; ++rh) {
            size_t p = (size_t)rh * n + isn + dim - 1;
            x[p] = x[p] / val[col_index[isn + dim - 1]];
        }
        cnt = 0;
        for (int j = isn + dim - 2; j >= isn; --j) {
            for (int rh = 0; rh < rhs; ++rh) {
                double sum = 0.0;
                for (uint64_t k = col_index[j] + 1; k <= col_index[j] + 1 + (uint64_t)cnt; ++k)
                    sum += val[k] * x[(size_t)rh * n + row[k]];
                x[(size_t)rh * n + j] = (x[(size_t)rh * n + j] - sum) / val[col_index[j]];
            }
            cnt++;
        }
    }
}

/* core.cpp:136-161  ccs2ccs_pad: pad every supernode's triangle to a full dim x rowlen
 * row-major block.  Row d of a supernode first gets d explicit zeros at columns
 * row[col_index[nodes[si]]] + 0..d-1, then its own entries.  row_pad[i+1] receives the
 * running entry count (row_pad[0] is left to the caller, who zeroes it).  Returns nnz. */
ORC_API int orc_ccs2ccs_pad(const double* val, const int* row, const uint64_t* col_index, double* val_pad,
                            uint64_t* col_index_pad, int* row_pad, const int* nodes, int sn) {
    int g = 0, cnt = 0;
    for (int si = 0; si < sn; ++si) {
        int pad = nodes[si + 1] - nodes[si];
        for (int d = 0; d < pad; ++d) {
            for (int ci = 0; ci < d; ++ci, ++g) {
                val_pad[g] = 0.0;
                col_index_pad[g] = (uint64_t)(row[col_index[nodes[si]]] + ci);
                cnt++;
            }
            for (uint64_t ci = col_index[nodes[si] + d]; ci < col_index[nodes[si] + d + 1]; ++ci, ++g) {
                val_pad[g] = val[ci];
                col_index_pad[g] = (uint64_t)row[ci];
                cnt++;
            }
            row_pad[nodes[si] + d + 1] = cnt;
        }
    }
    return cnt;
}

/* core.cpp:164-201  supernodal_blas_upper on the padded format: per RHS, supernodes in
 * reverse: gather x at the rectangle's columns, c = R x_rect (cblas_dgemm, row-major,
 * lda = padded row length), x_s -= c, x_s = T^{-1} x_s (cblas_dtrsm upper non-unit).
 * The two BLAS calls are restated as plain loops (row-major, unit ldb). */
ORC_API void orc_supernodal_blas_upper(int n, size_t sn, const int* supernodes, double* x, const double* val,
                                       const uint64_t* colidx_pad, const int* rowptr_pad, int rhs) {
    double* B = (double*)calloc((size_t)n, sizeof(double));
    double* c = (double*)calloc((size_t)n, sizeof(double));
    for (int rh = 0; rh < rhs; ++rh) {
        size_t gs = (size_t)rh * n;
        for (int i = (int)sn - 1; i >= 0; --i) {
            int tr = supernodes[i + 1] - supernodes[i];
            int shift = rowptr_pad[supernodes[i]];
            int lda = (rowptr_pad[supernodes[i + 1]] - rowptr_pad[supernodes[i]]) / tr;
            int rec = rowptr_pad[supernodes[i] + 1] - rowptr_pad[supernodes[i]] - tr;
            for (int k = 0; k < rec; ++k) B[k] = x[gs + colidx_pad[shift + tr + k]];
            for (int r = 0; r < tr; ++r) {
                double acc = 0.0;
                for (int k = 0; k < rec; ++k) acc += val[shift + tr + (size_t)r * lda + k] * B[k];
                c[r] = acc;
            }
            for (int k = 0; k < tr; ++k) { x[gs + supernodes[i] + k] -= c[k]; c[k] = 0.0; }
            double* xs = x + gs + supernodes[i];
            for (int r = tr - 1; r >= 0; --r) {
                double s = xs[r];
                for (int k = r + 1; k < tr; ++k) s -= val[shift + (size_t)r * lda + k] * xs[k];
                xs[r] = s / val[shift + (size_t)r * lda + r];
            }
        }
    }
    free(B);
    free(c);
}

/* core.cpp:164-201  supernodal_blas_upper with its two BLAS calls made through a CBLAS library
 * loaded at run time (ILP64 interface: 64-bit dimensions, e.g. the OpenBLAS that numpy bundles,
 * scipy_cblas_dgemm64_ / scipy_cblas_dtrsm64_), so that the CPU baseline times the reference's
 * algorithm on an optimised multithreaded BLAS where MKL is absent.  Same calls and arguments as
 * core.cpp:186-195: row-major dgemm (tr_dim x 1 x rec_dim, lda = padded row length, beta = 1 on a
 * zeroed c) and dtrsm (left, upper, no transpose, non-unit, tr_dim x 1, ldb = 1). */
typedef void (*orc_dgemm64_fn)(int, int, int, int64_t, int64_t, int64_t, double, const double*, int64_t, const double*,
                               int64_t, double, double*, int64_t);
typedef void (*orc_dtrsm64_fn)(int, int, int, int, int, int64_t, int64_t, double, const double*, int64_t, double*,
                               int64_t);
ORC_API void orc_supernodal_blas_upper_cblas(int n, size_t sn, const int* supernodes, double* x, const double* val,
                                             const uint64_t* colidx_pad, const int* rowptr_pad, int rhs, void* dgemm,
                                             void* dtrsm) {
    orc_dgemm64_fn gemm = (orc_dgemm64_fn)dgemm;
    orc_dtrsm64_fn trsm = (orc_dtrsm64_fn)dtrsm;
    double* B = (double*)calloc((size_t)n, sizeof(double));
    double* c = (double*)calloc((size_t)n, sizeof(double));
    for (int rh = 0; rh < rhs; ++rh) {
        size_t gs = (size_t)rh * n;
        for (int i = (int)sn - 1; i >= 0; --i) {
            int tr = supernodes[i + 1] - supernodes[i];
            int shift = rowptr_pad[supernodes[i]];
            int lda = (rowptr_pad[supernodes[i + 1]] - rowptr_pad[supernodes[i]]) / tr;
            int rec = rowptr_pad[supernodes[i] + 1] - rowptr_pad[supernodes[i]] - tr;
            for (int k = 0; k < rec; ++k) B[k] = x[gs + colidx_pad[shift + tr + k]];
            gemm(101 /* row-major */, 111, 111, tr, 1, rec, 1.0, val + shift + tr, lda, B, 1, 1.0, c, 1);
            for (int k = 0; k < tr; ++k) { x[gs + supernodes[i] + k] -= c[k]; c[k] = 0.0; }
            trsm(101, 141 /* left */, 121 /* upper */, 111, 131 /* non-unit */, tr, 1, 1.0, val + shift, lda,
                 x + gs + supernodes[i], 1);
        }
    }
    free(B);
    free(c);
}

/* utils.cpp:355-380  check_result (row-major branch): ||x1 - x2||_2 / ||x1||_2. */
ORC_API double orc_rel_error(size_t len, const double* x_ref, const double* x) {
    double s = 0.0, nrm = 0.0;
    for (size_t i = 0; i < len; ++i) { double d = x_ref[i] - x[i]; s += d * d; nrm += x_ref[i] * x_ref[i]; }
    return sqrt(s) / sqrt(nrm);
}

/* Relative residual ||b - U x||_2 / ||b||_2 of one column-major RHS block (FP64). */
ORC_API double orc_rel_residual(int n, const double* val, const uint64_t* row_index, const int* col,
                                const double* x, const double* b, int rhs) {
    double rr = 0.0, bb = 0.0;
    for (int rh = 0; rh < rhs; ++rh) {
        size_t off = (size_t)rh * n;
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for (uint64_t k = row_index[i]; k < row_index[i + 1]; ++k) s += val[k] * x[off + col[k]];
            double r = b[off + i] - s;
            rr += r * r;
            bb += b[off + i] * b[off + i];
        }
    }
    return sqrt(rr) / sqrt(bb);
}

ORC_API int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
