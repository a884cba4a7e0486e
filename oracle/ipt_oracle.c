/*
 * ipt_oracle.c - CPU restatement of the FJennie/BLOCK_IPT IPT path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA solver in
 * block_ipt_gb300/ and the timed CPU baseline of bench.py; the product never
 * links, loads or calls it.  Every function names the reference lines it
 * restates.  It is compiled with -ffp-contract=off so that x86-64 and aarch64
 * hosts produce bit-identical results, and the OpenMP loops split output
 * elements between threads without changing any element's summation order,
 * so the thread count never changes a result bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_API __attribute__((visibility("default")))

/* Hash used by the reference dense tests: IPT_C_GPU/test_temp/runtests.cu:46-58. */
ORACLE_API double oracle_deterministic_noise(int row, int col)
{
    uint32_t x = (uint32_t)(row + 1) * 747796405u;
    x ^= (uint32_t)(col + 1) * 2891336453u;
    x ^= x >> 16;
    x *= 2246822519u;
    x ^= x >> 13;
    x *= 3266489917u;
    x ^= x >> 16;
    return ((double)(x & 0x00ffffffu) / 16777216.0) - 0.5;
}

/* Dense test matrix: IPT_C_GPU/test_temp/runtests.cu:60-80
 * (eps = 1e-2 hash noise, optionally symmetrised, diagonal += row + 1). */
ORACLE_API void oracle_fill_perturbative_matrix(double *matrix, int n, int symmetric)
{
    const double eps = 1.0e-2;
    for (int col = 0; col < n; ++col) {
        for (int row = 0; row < n; ++row) {
            double noise = oracle_deterministic_noise(row, col);
            if (symmetric) {
                noise = 0.5 * (oracle_deterministic_noise(row, col) +
                               oracle_deterministic_noise(col, row));
            }
            matrix[(size_t)row + (size_t)col * (size_t)n] = eps * noise;
        }
    }
    for (int row = 0; row < n; ++row) {
        matrix[(size_t)row + (size_t)row * (size_t)n] += (double)(row + 1);
    }
}

/* Banded CSC test matrix: IPT_C_GPU/test/sparse/runtests_sparse.cu:224-268.
 * Arrays must hold n+1, 3n-2 and 3n-2 entries.  Returns nnz. */
ORACLE_API int oracle_build_banded_csc(int n, int *col_ptr, int *row_ind, double *values)
{
    int cursor = 0;
    for (int col = 0; col < n; ++col) {
        col_ptr[col] = cursor;
        if (col > 0) {
            int edge = col - 1;
            row_ind[cursor] = col - 1;
            values[cursor] = 1.0e-2 * (0.50 + 0.03 * (double)(edge % 7));
            ++cursor;
        }
        row_ind[cursor] = col;
        values[cursor] = (double)(col + 1);
        ++cursor;
        if (col + 1 < n) {
            int edge = col;
            row_ind[cursor] = col + 1;
            values[cursor] = 1.0e-2 * (0.50 + 0.03 * (double)(edge % 7));
            ++cursor;
        }
    }
    col_ptr[n] = cursor;
    return cursor;
}

/* out = a * x for column-major a (n x n) and x (n x k).  Each output element
 * sums inner = 0..n-1 in ascending order, exactly as
 * IPT_C_GPU/test_temp/runtests.cu:82-96; the loop nest is reordered (row
 * block, inner, col, row) so that every thread streams its slab of `a` once
 * per product, which keeps every element's summation order. */
static void oracle_dense_matmul(double *out, const double *a, const double *x, int n, int k)
{
    const int rb = 256;
    const int nblocks = (n + rb - 1) / rb;
#pragma omp parallel for schedule(dynamic, 1)
    for (int b = 0; b < nblocks; ++b) {
        const int r0 = b * rb;
        const int r1 = r0 + rb < n ? r0 + rb : n;
        for (int col = 0; col < k; ++col) {
            double *o = out + (size_t)col * (size_t)n;
            for (int row = r0; row < r1; ++row) {
                o[row] = 0.0;
            }
        }
        for (int inner = 0; inner < n; ++inner) {
            const double *ac = a + (size_t)inner * (size_t)n;
            for (int col = 0; col < k; ++col) {
                const double xv = x[(size_t)inner + (size_t)col * (size_t)n];
                double *o = out + (size_t)col * (size_t)n;
                for (int row = r0; row < r1; ++row) {
                    o[row] += ac[row] * xv;
                }
            }
        }
    }
}

ORACLE_API void oracle_matmul(double *out, const double *a, const double *x, int n, int k)
{
    oracle_dense_matmul(out, a, x, n, k);
}

static double oracle_sum_squares(const double *v, size_t count)
{
    double s = 0.0;
    for (size_t i = 0; i < count; ++i) {
        s += v[i] * v[i];
    }
    return s;
}

/* Plain IPT on a dense column-major matrix.
 *  - fixed-iteration mode (use_tol = 0): IPT_C_GPU/test_temp/runtests.cu:98-174;
 *  - tolerance mode (use_tol = 1): the stopping rule of
 *    IPT_C_GPU/src/ipt_cuda.cu:1883-1932 (||F(X)-X||_F / ||X||_F <= tol, the
 *    returned block is F(X) of the last step; unconverged after maxiter still
 *    returns the last block).
 * The map is X'_ij = (Y_ij - d_i X_ij - X_ij c_j) / (d_j - d_i) with
 * Y = H X, c_j = Y_jj - d_j X_jj, and X'_jj = 1 (runtests.cu:130-150).
 * Eigenvalues are (H X)_jj of the returned block (runtests.cu:160-164).
 * x0 may be NULL (identity start, runtests.cu:122-124).
 * Returns 0, or -1 on allocation failure, -2 on a zero/non-finite ||X||. */
ORACLE_API int oracle_ipt_dense(const double *matrix, int n, int k, int maxiter, double tol,
                                int use_tol, const double *x0, double *vectors_out,
                                double *values_out, int *iterations_out,
                                double *fixed_point_residual_out)
{
    size_t elems = (size_t)n * (size_t)k;
    double *x = (double *)calloc(elems, sizeof(double));
    double *y = (double *)calloc(elems, sizeof(double));
    double *diag = (double *)calloc((size_t)n, sizeof(double));
    double *cdiag = (double *)calloc((size_t)k, sizeof(double));
    int done = 0;
    int status = 0;
    double fpres = NAN;

    if (x == NULL || y == NULL || diag == NULL || cdiag == NULL) {
        free(x); free(y); free(diag); free(cdiag);
        return -1;
    }
    if (x0 != NULL) {
        memcpy(x, x0, elems * sizeof(double));
    } else {
        for (int col = 0; col < k; ++col) {
            x[(size_t)col + (size_t)col * (size_t)n] = 1.0;
        }
    }
    for (int row = 0; row < n; ++row) {
        diag[row] = matrix[(size_t)row + (size_t)row * (size_t)n];
    }

    for (int iter = 0; iter < maxiter; ++iter) {
        oracle_dense_matmul(y, matrix, x, n, k);
        for (int col = 0; col < k; ++col) {
            size_t di = (size_t)col + (size_t)col * (size_t)n;
            cdiag[col] = y[di] - diag[col] * x[di];
        }
#pragma omp parallel for schedule(static)
        for (int col = 0; col < k; ++col) {
            for (int row = 0; row < n; ++row) {
                size_t idx = (size_t)row + (size_t)col * (size_t)n;
                if (row == col) {
                    y[idx] = 1.0;
                } else {
                    double g = 1.0 / (diag[col] - diag[row]);
                    y[idx] = (y[idx] - diag[row] * x[idx] - x[idx] * cdiag[col]) * g;
                }
            }
        }
        done = iter + 1;
        if (use_tol) {
            double dsum = 0.0;
            double xsum = oracle_sum_squares(x, elems);
            for (size_t i = 0; i < elems; ++i) {
                double d = y[i] - x[i];
                dsum += d * d;
            }
            if (!(xsum > 0.0) || !isfinite(xsum)) {
                status = -2;
                break;
            }
            fpres = sqrt(dsum) / sqrt(xsum);
            {
                double *t = x; x = y; y = t;
            }
            if (fpres <= tol) {
                break;
            }
        } else {
            double *t = x; x = y; y = t;
        }
    }

    if (status == 0) {
        oracle_dense_matmul(y, matrix, x, n, k);
        for (int col = 0; col < k; ++col) {
            values_out[col] = y[(size_t)col + (size_t)col * (size_t)n];
        }
        memcpy(vectors_out, x, elems * sizeof(double));
        if (iterations_out != NULL) {
            *iterations_out = done;
        }
        if (fixed_point_residual_out != NULL) {
            *fixed_point_residual_out = fpres;
        }
    }
    free(x); free(y); free(diag); free(cdiag);
    return status;
}

/* Dense copy of a CSC matrix, duplicates summed:
 * IPT_C_GPU/test/sparse/runtests_sparse.cu:60-75. */
ORACLE_API void oracle_csc_to_dense(double *dense, const int *col_ptr, const int *row_ind,
                                    const double *values, int n)
{
    memset(dense, 0, (size_t)n * (size_t)n * sizeof(double));
    for (int col = 0; col < n; ++col) {
        for (int p = col_ptr[col]; p < col_ptr[col + 1]; ++p) {
            int row = row_ind[p];
            if (row >= 0 && row < n) {
                dense[(size_t)row + (size_t)col * (size_t)n] += values[p];
            }
        }
    }
}

/* Scaled residual max_j ||H x_j - v_j x_j|| / (max(1,|v_j|) max(1,||x_j||)):
 * IPT_C_GPU/test_temp/runtests.cu:191-229. */
ORACLE_API double oracle_max_relative_residual(const double *matrix, const double *vectors,
                                               const double *values, int n, int k)
{
    double *mx = (double *)calloc((size_t)n * (size_t)k, sizeof(double));
    double max_residual = 0.0;
    if (mx == NULL) {
        return INFINITY;
    }
    oracle_dense_matmul(mx, matrix, vectors, n, k);
    for (int col = 0; col < k; ++col) {
        double rs = 0.0, vs = 0.0;
        for (int row = 0; row < n; ++row) {
            size_t idx = (size_t)row + (size_t)col * (size_t)n;
            double r = mx[idx] - vectors[idx] * values[col];
            rs += r * r;
            vs += vectors[idx] * vectors[idx];
        }
        {
            double denom = fmax(1.0, fabs(values[col])) * fmax(1.0, sqrt(vs));
            double rel = sqrt(rs) / denom;
            if (rel > max_residual) {
                max_residual = rel;
            }
        }
    }
    free(mx);
    return max_residual;
}

/* CSC validation: IPT_C_GPU/src/ipt_preparation.cu:148-169. */
ORACLE_API int oracle_validate_csc(const int *col_ptr, const int *row_ind, int n, int nnz)
{
    if (col_ptr == NULL || (nnz > 0 && row_ind == NULL) || n <= 0 || nnz < 0 ||
        col_ptr[0] != 0 || col_ptr[n] != nnz) {
        return 0;
    }
    for (int col = 0; col < n; ++col) {
        if (col_ptr[col] > col_ptr[col + 1]) {
            return 0;
        }
    }
    for (int p = 0; p < nnz; ++p) {
        if (row_ind[p] < 0 || row_ind[p] >= n) {
            return 0;
        }
    }
    return 1;
}

/* Diagonal of a CSC matrix, first matching entry per column:
 * IPT_C_GPU/src/ipt_preparation.cu:171-188. */
ORACLE_API void oracle_csc_diagonal(const int *col_ptr, const int *row_ind, const double *values,
                                    int n, double *diag)
{
    for (int col = 0; col < n; ++col) {
        diag[col] = 0.0;
        for (int p = col_ptr[col]; p < col_ptr[col + 1]; ++p) {
            if (row_ind[p] == col) {
                diag[col] = values[p];
                break;
            }
        }
    }
}

static const double *g_sort_key;
static int oracle_cmp_perm(const void *a, const void *b)
{
    int ia = *(const int *)a, ib = *(const int *)b;
    double da = g_sort_key[ia], db = g_sort_key[ib];
    if (da < db) return -1;
    if (db < da) return 1;
    return (ia > ib) - (ia < ib); /* ties keep the original order (stable) */
}

/* Stable ascending sort of the diagonal: IPT_C_GPU/src/ipt_preparation.cu:190-208.
 * perm[sorted] = original index. */
ORACLE_API void oracle_stable_sort_permutation(const double *diag, int n, int *perm)
{
    for (int i = 0; i < n; ++i) {
        perm[i] = i;
    }
    g_sort_key = diag;
    qsort(perm, (size_t)n, sizeof(int), oracle_cmp_perm);
    g_sort_key = NULL;
}

/* y = H x for H in CSC (any symmetry), x/y column-major n-by-k; scatter over
 * the stored entries in storage order.  This is the product the reference
 * asks cuSPARSE for (CSC passed as CSR with OP_T,
 * IPT_C_GPU/src/ipt_cuda.cu:1535-1559). */
ORACLE_API void oracle_csc_matmul(const int *col_ptr, const int *row_ind, const double *values,
                                  int n, const double *x, int k, double *y)
{
#pragma omp parallel for schedule(static)
    for (int j = 0; j < k; ++j) {
        double *yj = y + (size_t)j * (size_t)n;
        const double *xj = x + (size_t)j * (size_t)n;
        for (int r = 0; r < n; ++r) {
            yj[r] = 0.0;
        }
        for (int col = 0; col < n; ++col) {
            double xv = xj[col];
            for (int p = col_ptr[col]; p < col_ptr[col + 1]; ++p) {
                yj[row_ind[p]] += values[p] * xv;
            }
        }
    }
}

/* y = H x for H in CSR, each row summed in stored order (the gather the CUDA
 * SpMM performs); x/y column-major n-by-k.  Rows are split between threads. */
ORACLE_API void oracle_csr_matmul(const int *row_ptr, const int *col_ind, const double *values,
                                  int n, const double *x, int k, double *y)
{
#pragma omp parallel for schedule(dynamic, 256)
    for (int r = 0; r < n; ++r) {
        for (int j = 0; j < k; ++j) {
            const double *xj = x + (size_t)j * (size_t)n;
            double s = 0.0;
            for (int p = row_ptr[r]; p < row_ptr[r + 1]; ++p) {
                s += values[p] * xj[col_ind[p]];
            }
            y[(size_t)r + (size_t)j * (size_t)n] = s;
        }
    }
}

/* Plain IPT on a CSR matrix (rows summed in stored order), same map and stop
 * rule as oracle_ipt_dense; diag must hold the matrix diagonal. */
ORACLE_API int oracle_ipt_csr(const int *row_ptr, const int *col_ind, const double *values,
                              const double *diag, int n, int k, int maxiter, double tol,
                              int use_tol, const double *x0, double *vectors_out,
                              double *values_out, int *iterations_out,
                              double *fixed_point_residual_out)
{
    size_t elems = (size_t)n * (size_t)k;
    double *x = (double *)calloc(elems, sizeof(double));
    double *y = (double *)calloc(elems, sizeof(double));
    double *cdiag = (double *)calloc((size_t)k, sizeof(double));
    int done = 0;
    int status = 0;
    double fpres = NAN;

    if (x == NULL || y == NULL || cdiag == NULL) {
        free(x); free(y); free(cdiag);
        return -1;
    }
    if (x0 != NULL) {
        memcpy(x, x0, elems * sizeof(double));
    } else {
        for (int col = 0; col < k; ++col) {
            x[(size_t)col + (size_t)col * (size_t)n] = 1.0;
        }
    }
    for (int iter = 0; iter < maxiter; ++iter) {
        oracle_csr_matmul(row_ptr, col_ind, values, n, x, k, y);
        for (int col = 0; col < k; ++col) {
            size_t di = (size_t)col + (size_t)col * (size_t)n;
            cdiag[col] = y[di] - diag[col] * x[di];
        }
#pragma omp parallel for schedule(static)
        for (int col = 0; col < k; ++col) {
            for (int row = 0; row < n; ++row) {
                size_t idx = (size_t)row + (size_t)col * (size_t)n;
                if (row == col) {
                    y[idx] = 1.0;
                } else {
                    double g = 1.0 / (diag[col] - diag[row]);
                    y[idx] = (y[idx] - diag[row] * x[idx] - x[idx] * cdiag[col]) * g;
                }
            }
        }
        done = iter + 1;
        if (use_tol) {
            double dsum = 0.0;
            double xsum = oracle_sum_squares(x, elems);
            for (size_t i = 0; i < elems; ++i) {
                double d = y[i] - x[i];
                dsum += d * d;
            }
            if (!(xsum > 0.0) || !isfinite(xsum)) {
                status = -2;
                break;
            }
            fpres = sqrt(dsum) / sqrt(xsum);
            {
                double *t = x; x = y; y = t;
            }
            if (fpres <= tol) {
                break;
            }
        } else {
            double *t = x; x = y; y = t;
        }
    }
    if (status == 0) {
        oracle_csr_matmul(row_ptr, col_ind, values, n, x, k, y);
        for (int col = 0; col < k; ++col) {
            values_out[col] = y[(size_t)col + (size_t)col * (size_t)n];
        }
        memcpy(vectors_out, x, elems * sizeof(double));
        if (iterations_out != NULL) {
            *iterations_out = done;
        }
        if (fixed_point_residual_out != NULL) {
            *fixed_point_residual_out = fpres;
        }
    }
    free(x); free(y); free(cdiag);
    return status;
}

ORACLE_API int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Thread count of the following oracle calls (a timed single-core sample). */
ORACLE_API void oracle_set_num_threads(int threads)
{
#ifdef _OPENMP
    omp_set_num_threads(threads > 0 ? threads : 1);
#else
    (void)threads;
#endif
}

/* Plain IPT with the eigen-residual read off every step: for the block X
 * entering a step, r_j = H x_j - lambda_j x_j with lambda_j = (H X)_jj equals
 * (d_j - d_i)(F(X) - X)_ij entrywise (zero on the target row).  Returns the
 * number of block products needed until the block entering a step satisfies
 * max_j ||r_j|| / (max(1, hnorm) max(1, ||x_j||)) <= res_tol (that step
 * included: it yields lambda), or -1 if maxiter products do not reach it.
 * Same map and arithmetic as oracle_ipt_dense. */
ORACLE_API int oracle_ipt_dense_products_to_residual(const double *matrix, int n, int k,
                                                     int maxiter, double hnorm, double res_tol,
                                                     double *final_scaled_residual)
{
    size_t elems = (size_t)n * (size_t)k;
    double *x = (double *)calloc(elems, sizeof(double));
    double *y = (double *)calloc(elems, sizeof(double));
    double *diag = (double *)calloc((size_t)n, sizeof(double));
    double *cdiag = (double *)calloc((size_t)k, sizeof(double));
    int found = -1;
    if (x == NULL || y == NULL || diag == NULL || cdiag == NULL) {
        free(x); free(y); free(diag); free(cdiag);
        return -2;
    }
    for (int col = 0; col < k; ++col) {
        x[(size_t)col + (size_t)col * (size_t)n] = 1.0;
    }
    for (int row = 0; row < n; ++row) {
        diag[row] = matrix[(size_t)row + (size_t)row * (size_t)n];
    }
    for (int iter = 0; iter < maxiter; ++iter) {
        double worst = 0.0;
        oracle_dense_matmul(y, matrix, x, n, k);
        for (int col = 0; col < k; ++col) {
            size_t di = (size_t)col + (size_t)col * (size_t)n;
            cdiag[col] = y[di] - diag[col] * x[di];
        }
        for (int col = 0; col < k; ++col) {
            double rs = 0.0, xs = 0.0;
            for (int row = 0; row < n; ++row) {
                size_t idx = (size_t)row + (size_t)col * (size_t)n;
                double xo = x[idx];
                xs += xo * xo;
                if (row == col) {
                    y[idx] = 1.0;
                } else {
                    double g = 1.0 / (diag[col] - diag[row]);
                    y[idx] = (y[idx] - diag[row] * xo - xo * cdiag[col]) * g;
                    double r = (diag[col] - diag[row]) * (y[idx] - xo);
                    rs += r * r;
                }
            }
            {
                double sc = sqrt(rs) / (fmax(1.0, hnorm) * fmax(1.0, sqrt(xs)));
                if (!(sc <= worst)) {
                    worst = sc;
                }
            }
        }
        if (final_scaled_residual != NULL) {
            *final_scaled_residual = worst;
        }
        if (worst <= res_tol) {
            found = iter + 1;
            break;
        }
        {
            double *t = x; x = y; y = t;
        }
    }
    free(x); free(y); free(diag); free(cdiag);
    return found;
}

/* ---- block-cluster path ----------------------------------------------------
 * One block-cluster update of the cluster [first, first + m): the GPU kernel
 * ipt_block_cluster_update_kernel (IPT_C_GPU/src/ipt_cuda.cu:2280-2384) row
 * by row.  basis and y (= H basis) are n x m, column-major; rows inside the
 * cluster get the identity, every other row i solves
 *   (d_i I - h^T) x = d_i basis[i, :] - y[i, :],  h[u + e m] = y[first + u, e]
 * by Gauss-Jordan elimination with partial pivoting: the pivot is the first
 * row with the largest |entry| (the reference's scan, strict comparison),
 * singular when that entry is NaN on the diagonal, not finite, or not above
 * 64 DBL_EPSILON.  The arithmetic is the library's CUDA kernel's, operation
 * for operation, so that both give the same bits: the off-diagonal entries
 * -h, the diagonal d_i - h, the right side fma(d_i, x, -y); per step one
 * reciprocal r = 1 / pivot, the pivot row's later columns times r, the
 * elimination a[e][j] = fma(-a[e][p], a[p][j], a[e][j]) for j > p (column p
 * is never read again); the damping fma(damping, v, (1 - damping) x).  The
 * reference divides by the pivot instead (one rounding apart).  Returns 1 if
 * a row system is singular or a value is not finite, 0 otherwise. */
ORACLE_API int oracle_cluster_update(const double *basis, const double *y, const double *diag,
                                     int n, int first, int m, double damping, double *next)
{
    const int ld = m + 1;
    double *aug = (double *)malloc((size_t)m * (size_t)ld * sizeof(double));
    int singular_any = 0;
    for (int row = 0; row < n; ++row) {
        if (row >= first && row < first + m) {
            for (int e = 0; e < m; ++e) {
                next[(size_t)row + (size_t)e * n] = row == first + e ? 1.0 : 0.0;
            }
            continue;
        }
        const double dr = diag[row];
        for (int e = 0; e < m; ++e) {
            double *a = aug + (size_t)e * ld;
            for (int u = 0; u < m; ++u) {
                const double hv = y[(size_t)(first + u) + (size_t)e * n];
                a[u] = u == e ? dr - hv : -hv;
            }
            a[m] = fma(dr, basis[(size_t)row + (size_t)e * n], -y[(size_t)row + (size_t)e * n]);
        }
        int singular = 0;
        for (int p = 0; p < m; ++p) {
            int piv = p;
            double pa = fabs(aug[(size_t)p * ld + p]);
            for (int c = p + 1; c < m; ++c) {
                const double ca = fabs(aug[(size_t)c * ld + p]);
                if (ca > pa) {
                    pa = ca;
                    piv = c;
                }
            }
            if (!isfinite(pa) || pa <= 64.0 * 2.220446049250313e-16) {
                singular = 1;
                break;
            }
            double *ap = aug + (size_t)p * ld;
            if (piv != p) {
                double *aq = aug + (size_t)piv * ld;
                for (int j = p; j <= m; ++j) {
                    const double t = ap[j];
                    ap[j] = aq[j];
                    aq[j] = t;
                }
            }
            const double r = 1.0 / ap[p];
            for (int j = p + 1; j <= m; ++j) ap[j] = ap[j] * r;
            for (int e = 0; e < m; ++e) {
                if (e == p) continue;
                double *a = aug + (size_t)e * ld;
                const double f = a[p];
                for (int j = p + 1; j <= m; ++j) a[j] = fma(-f, ap[j], a[j]);
            }
        }
        if (!singular) {
            for (int e = 0; e < m; ++e) {
                double v = aug[(size_t)e * ld + m];
                if (damping < 1.0) {
                    v = fma(damping, v, (1.0 - damping) * basis[(size_t)row + (size_t)e * n]);
                }
                if (!isfinite(v)) {
                    singular = 1;
                    v = 0.0;
                }
                next[(size_t)row + (size_t)e * n] = v;
            }
        }
        singular_any |= singular;
    }
    free(aug);
    return singular_any;
}

/* The block-cluster basis of each cluster in turn, as
 * ipt_block_cluster_solve_basis_gpu (IPT_C_GPU/src/ipt_cuda.cu:2871-3037):
 * identity start, Y = H X (CSR rows summed in stored order), one update,
 * residual ||X' - X||_F / max(1, ||X||_F), stop at tol (tol <= 0: 1e-12) or
 * maxiter; damping outside (0, 1] counts as 1.  ranges: nclusters inclusive
 * (first, last) pairs; basis: n x sum of widths.  Returns 0, or 1 + the
 * index of the first cluster whose row system was singular or whose iterate
 * or norms were not finite. */
ORACLE_API int oracle_cluster_basis(const int *row_ptr, const int *col_ind, const double *values,
                                    const double *diag, int n, const int *ranges, int nclusters,
                                    int maxiter, double tol, double damping, double *basis,
                                    int *iterations, double *residuals)
{
    const double eff_tol = tol > 0.0 ? tol : 1.0e-12;
    if (!(damping > 0.0 && damping <= 1.0)) damping = 1.0;
    size_t off = 0;
    for (int c = 0; c < nclusters; ++c) {
        const int first = ranges[2 * c], m = ranges[2 * c + 1] - ranges[2 * c] + 1;
        const size_t cnt = (size_t)n * (size_t)m;
        double *x = basis + off * (size_t)n;
        double *y = (double *)malloc(cnt * sizeof(double));
        double *nx = (double *)malloc(cnt * sizeof(double));
        for (size_t i = 0; i < cnt; ++i) {
            const int j = (int)(i / (size_t)n), r = (int)(i % (size_t)n);
            x[i] = r == first + j ? 1.0 : 0.0;
        }
        iterations[c] = 0;
        residuals[c] = NAN;
        for (int it = 0; it < maxiter; ++it) {
            oracle_csr_matmul(row_ptr, col_ind, values, n, x, m, y);
            int bad = oracle_cluster_update(x, y, diag, n, first, m, damping, nx);
            double dd = 0.0, bb = 0.0;
            for (size_t i = 0; i < cnt; ++i) {
                const double dx = nx[i] - x[i];
                dd += dx * dx;
                bb += x[i] * x[i];
            }
            const double dn = sqrt(dd), bn = sqrt(bb);
            if (bad || !isfinite(dn) || !isfinite(bn) || bn <= 0.0) {
                free(y);
                free(nx);
                return 1 + c;
            }
            memcpy(x, nx, cnt * sizeof(double));
            iterations[c] = it + 1;
            residuals[c] = dn / fmax(1.0, bn);
            if (residuals[c] <= eff_tol) break;
        }
        free(y);
        free(nx);
        off += (size_t)m;
    }
    return 0;
}

/* ---- ACX extrapolation (dense FP64) -------------------------------------------
 * IPT_C_GPU/src/ACX/acx_cuda.cu:390-620: from the identity columns, each step
 * evaluates f1 = F(X) (residuals ||HX_j - X_j (HX)_jj|| and the map with the
 * denominator guard |d_j - d_i| <= DBL_EPSILON, :109-172), stops once
 * ||f1 - X||_F / ||X||_F < min(tol, 1e-12), else extrapolates with order 2
 * (odd steps, :190-240) or order 3 (even steps, :242-296).  Products sum the
 * inner index in ascending order; the map and the extrapolation place their
 * FMAs as the library's CUDA kernels do.  Returns 0, 1 (invalid argument or
 * a zero norm) or 5 (zero denominator); info = {iterations, f_calls,
 * converged}, res = {max_residual, fixed_point_residual}; vectors_out gets
 * the last F(X), values_out diag(H F(X)). */
static int oracle_acx_map(const double *H, const double *d, int n, int k, const double *x,
                          double *y, double *resid)
{
    int bad = 0;
    oracle_dense_matmul(y, H, x, n, k);
    for (int c = 0; c < k; ++c) {
        double *yc = y + (size_t)c * n;
        const double *xc = x + (size_t)c * n;
        const double m = yc[c];
        const double u = fma(-d[c], xc[c], m);
        double rr = 0.0;
        for (int i = 0; i < n; ++i) {
            const double yi = yc[i], xi = xc[i];
            const double r = fma(-xi, m, yi);
            rr = fma(r, r, rr);
            double v = 1.0;
            if (i != c) {
                const double den = d[c] - d[i];
                if (fabs(den) <= 2.220446049250313e-16) {
                    bad = 1;
                    v = 0.0;
                } else {
                    v = fma(-xi, u, fma(-d[i], xi, yi)) / den;
                }
            }
            yc[i] = v;
        }
        resid[c] = sqrt(rr);
    }
    return bad;
}

static int oracle_acx_run(const double *H, int n, int k, double tol, int maxiter,
                          const double *initial, double *vectors_out, double *values_out,
                          int *info, double *res);

ORACLE_API int oracle_acx_dense(const double *H, int n, int k, double tol, int maxiter,
                                double *vectors_out, double *values_out, int *info, double *res)
{
    if (H == NULL || n <= 0 || k <= 0 || k > n || !(tol > 0.0) || maxiter <= 0) return 1;
    return oracle_acx_run(H, n, k, tol, maxiter, NULL, vectors_out, values_out, info, res);
}

/* The FP64 loop from the identity (initial == NULL: the result is the last
 * F(X)) or from a start block (the mixed ACX's second stage,
 * acx_mixed_precision_cuda.cu:575-809: F(X) when the stop was met, else the
 * extrapolated X). */
static int oracle_acx_run(const double *H, int n, int k, double tol, int maxiter,
                          const double *initial, double *vectors_out, double *values_out,
                          int *info, double *res)
{
    const size_t e = (size_t)n * (size_t)k;
    const double stop_tol = tol < 1.0e-12 ? tol : 1.0e-12;
    double *d = (double *)malloc((size_t)n * sizeof(double));
    double *x = (double *)calloc(e, sizeof(double));
    double *f1 = (double *)malloc(e * sizeof(double));
    double *f2 = (double *)malloc(e * sizeof(double));
    double *f3 = (double *)malloc(e * sizeof(double));
    double *resid = (double *)malloc((size_t)k * sizeof(double));
    int status = 0;
    info[0] = info[1] = info[2] = 0;
    res[0] = res[1] = NAN;
    int final_is_x = initial != NULL;
    for (int i = 0; i < n; ++i) d[i] = H[(size_t)i + (size_t)i * n];
    if (initial != NULL) {
        memcpy(x, initial, e * sizeof(double));
    } else {
        for (int c = 0; c < k; ++c) x[(size_t)c + (size_t)c * n] = 1.0;
    }
    for (int iter = 1; iter <= maxiter; ++iter) {
        const int order = (iter % 2 == 1) ? 2 : 3;
        info[0] = iter;
        if (oracle_acx_map(H, d, n, k, x, f1, resid)) {
            status = 5;
            break;
        }
        info[1] += 1;
        double mx = 0.0, dd = 0.0, bb = 0.0;
        for (int c = 0; c < k; ++c) mx = resid[c] > mx ? resid[c] : mx;
        res[0] = mx;
        for (size_t i = 0; i < e; ++i) {
            const double t = f1[i] - x[i];
            dd = fma(t, t, dd);
            bb = fma(x[i], x[i], bb);
        }
        if (!(bb > 0.0) || !isfinite(bb)) {
            status = 1;
            break;
        }
        res[1] = sqrt(dd) / sqrt(bb);
        if (res[1] < stop_tol) {
            info[2] = 1;
            final_is_x = 0;
            break;
        }
        oracle_acx_map(H, d, n, k, f1, f2, resid);
        info[1] += 1;
        if (order == 3) {
            oracle_acx_map(H, d, n, k, f2, f3, resid);
            info[1] += 1;
        }
        for (int c = 0; c < k; ++c) {
            const size_t b = (size_t)c * n;
            double num = 0.0, den = 0.0;
            for (int i = 0; i < n; ++i) {
                const double d2 = fma(-2.0, f1[b + i], f2[b + i]) + x[b + i];
                if (order == 2) {
                    const double d1 = f1[b + i] - x[b + i];
                    num = fma(d2, d1, num);
                    den = fma(d2, d2, den);
                } else {
                    const double d3 = fma(3.0, f1[b + i], fma(-3.0, f2[b + i], f3[b + i])) - x[b + i];
                    num = fma(d3, d2, num);
                    den = fma(d3, d3, den);
                }
            }
            const double g = den > 0.0 ? fabs(num / den) : 0.0, g2 = g * g, g3 = g2 * g;
            for (int i = 0; i < n; ++i) {
                const double xi = x[b + i];
                const double d1 = f1[b + i] - xi;
                const double d2 = fma(-2.0, f1[b + i], f2[b + i]) + xi;
                if (order == 2) {
                    x[b + i] = xi + fma(2.0 * g, d1, g2 * d2);
                } else {
                    const double d3 = fma(3.0, f1[b + i], fma(-3.0, f2[b + i], f3[b + i])) - xi;
                    x[b + i] = xi + fma(3.0 * g, d1, fma(3.0 * g2, d2, g3 * d3));
                }
            }
        }
    }
    if (status == 0) {
        if (final_is_x) memcpy(f1, x, e * sizeof(double));
        memcpy(vectors_out, f1, e * sizeof(double));
        oracle_dense_matmul(f2, H, f1, n, k);
        for (int c = 0; c < k; ++c) values_out[c] = f2[(size_t)c + (size_t)c * n];
    }
    free(d);
    free(x);
    free(f1);
    free(f2);
    free(f3);
    free(resid);
    return status;
}

/* Mixed ACX, IPT_C_GPU/src/ACX/acx_mixed_precision_cuda.cu:360-573 then
 * :575-809: the extrapolation on the map with Delta (zero diagonal) and the
 * diagonal in FP32 (products summed in FP32, inner index ascending; the map
 * (y - x u) / (d_c - d_r) with the FLT_EPSILON guard; FP32 extrapolation,
 * step length from FP64 sums of its FP32 inner products) until the residual
 * is <= tf32_tol, the block (F(X) if the stop was met, else X) widened to
 * FP64, then oracle_acx_run from it.  The reference's TF32 GEMM is an FP32
 * product here, as in the library.  info = {tf32 iterations, tf32 f_calls,
 * tf32 converged, fp64 iterations, fp64 f_calls, fp64 converged}; res =
 * {tf32 fixed-point residual, fp64 max residual, fp64 fixed-point residual}. */
ORACLE_API int oracle_acx_mixed(const double *H, int n, int k, double tf32_tol, int tf32_maxiter,
                                double fp64_tol, int fp64_maxiter, double *vectors_out,
                                double *values_out, int *info, double *res)
{
    if (H == NULL || n <= 0 || k <= 0 || k > n || !(tf32_tol > 0.0) || !(fp64_tol > 0.0) ||
        tf32_maxiter <= 0 || fp64_maxiter <= 0) {
        return 1;
    }
    const size_t e = (size_t)n * (size_t)k;
    float *D = (float *)malloc((size_t)n * (size_t)n * sizeof(float));
    float *d = (float *)malloc((size_t)n * sizeof(float));
    float *x = (float *)calloc(e, sizeof(float));
    float *f[3];
    for (int i = 0; i < 3; ++i) f[i] = (float *)malloc(e * sizeof(float));
    double *initial = (double *)malloc(e * sizeof(double));
    int status = 0;
    for (int i = 0; i < 6; ++i) info[i] = 0;
    res[0] = res[1] = res[2] = NAN;
    for (size_t i = 0; i < (size_t)n * (size_t)n; ++i) {
        const int r = (int)(i % (size_t)n), c = (int)(i / (size_t)n);
        D[i] = r == c ? 0.0f : (float)H[i];
        if (r == c) d[r] = (float)H[i];
    }
    for (int c = 0; c < k; ++c) x[(size_t)c + (size_t)c * n] = 1.0f;
    const float *final_block = x;
    for (int iter = 1; iter <= tf32_maxiter && status == 0; ++iter) {
        const int order = (iter % 2 == 1) ? 2 : 3;
        info[0] = iter;
        const float *src = x;
        for (int step = 0; step < (order == 2 ? 2 : 3); ++step) {
            float *y = f[step];
            for (int c = 0; c < k; ++c) {
                const float *xc = src + (size_t)c * n;
                float *yc = y + (size_t)c * n;
                for (int r = 0; r < n; ++r) {
                    float acc = 0.0f;
                    for (int l = 0; l < n; ++l) acc += D[(size_t)r + (size_t)l * n] * xc[l];
                    yc[r] = acc;
                }
                const float u = yc[c];
                for (int i = 0; i < n; ++i) {
                    float v = 1.0f;
                    if (i != c) {
                        const float den = d[c] - d[i];
                        if (fabsf(den) <= 1.1920928955078125e-07f) {
                            status = 5;
                            v = 0.0f;
                        } else {
                            v = fmaf(-xc[i], u, yc[i]) / den;
                        }
                    }
                    yc[i] = v;
                }
            }
            info[1] += 1;
            if (status != 0) break;
            if (step == 0) {
                double dd = 0.0, bb = 0.0;
                for (size_t i = 0; i < e; ++i) {
                    const double b = (double)x[i], t = (double)f[0][i] - b;
                    dd = fma(t, t, dd);
                    bb = fma(b, b, bb);
                }
                if (!(bb > 0.0) || !isfinite(bb)) {
                    status = 1;
                    break;
                }
                res[0] = sqrt(dd) / sqrt(bb);
                if (res[0] <= tf32_tol) {
                    info[2] = 1;
                    final_block = f[0];
                    break;
                }
            }
            src = y;
        }
        if (status != 0 || info[2]) break;
        for (int c = 0; c < k; ++c) {
            const size_t b = (size_t)c * n;
            const float *f1 = f[0] + b, *f2 = f[1] + b, *f3 = f[2] + b;
            float *xc = x + b;
            float num = 0.0f, den = 0.0f;
            for (int i = 0; i < n; ++i) {
                const float d2 = fmaf(-2.0f, f1[i], f2[i]) + xc[i];
                if (order == 2) {
                    const float d1 = f1[i] - xc[i];
                    num = fmaf(d2, d1, num);
                    den = fmaf(d2, d2, den);
                } else {
                    const float d3 = fmaf(3.0f, f1[i], fmaf(-3.0f, f2[i], f3[i])) - xc[i];
                    num = fmaf(d3, d2, num);
                    den = fmaf(d3, d3, den);
                }
            }
            const double sd = (double)den > 0.0 ? fabs((double)num / (double)den) : 0.0;
            const float g = (float)sd, g2 = g * g, g3 = g2 * g;
            for (int i = 0; i < n; ++i) {
                const float xi = xc[i];
                const float d1 = f1[i] - xi;
                const float d2 = fmaf(-2.0f, f1[i], f2[i]) + xi;
                if (order == 2) {
                    xc[i] = xi + fmaf(2.0f * g, d1, g2 * d2);
                } else {
                    const float d3 = fmaf(3.0f, f1[i], fmaf(-3.0f, f2[i], f3[i])) - xi;
                    xc[i] = xi + fmaf(3.0f * g, d1, fmaf(3.0f * g2, d2, g3 * d3));
                }
            }
        }
        final_block = x;
    }
    if (status == 0) {
        int info64[3];
        double res64[2];
        for (size_t i = 0; i < e; ++i) initial[i] = (double)final_block[i];
        status = oracle_acx_run(H, n, k, fp64_tol, fp64_maxiter, initial, vectors_out, values_out,
                                info64, res64);
        info[3] = info64[0];
        info[4] = info64[1];
        info[5] = info64[2];
        res[1] = res64[0];
        res[2] = res64[1];
    }
    free(D);
    free(d);
    free(x);
    for (int i = 0; i < 3; ++i) free(f[i]);
    free(initial);
    return status;
}
