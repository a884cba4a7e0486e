/*
 * ipt_block.h - block IPT + Rayleigh-Ritz + Davidson solver of libipt_gb300.so.
 *
 * These entry points extend the reference ABI of ipt_cuda.h.  They compute the
 * k lowest eigenpairs of a symmetric H = D + Delta to a scaled residual
 *      ||H x_j - theta_j x_j|| <= residual_tol * max(1, ||H||_inf),  ||x_j|| = 1,
 * the stopping scale of the reference's block path
 * (IPT_C_GPU/src/ipt_cuda.cu:2684-2697), with the steps of its block-cluster
 * + Davidson driver (IPT_C_GPU/src/ipt_cuda.cu:4712-5016): an IPT stage on
 * the lowest diagonal positions, Rayleigh-Ritz on the IPT block, then
 * Davidson corrections with thick restart until every pair converges.
 *
 * The IPT stage runs in the precision chosen by `ipt_precision`; FP16/BF16/
 * TF32 stages multiply on the tensor cores and the FP64 stages that follow
 * (CholQR Gram matrices, projected matrix, eigensolve, residuals and the
 * Davidson sweep) win the accuracy back.  The result is always FP64.
 *
 * Conventions: dense H is column-major with leading dimension n; CSR input
 * is 0-based int32 row_ptr[n+1] / col_ind[nnz] with double values (for a
 * symmetric H these are also its CSC arrays).  Device entry points take
 * device pointers and run on `stream` (NULL = legacy default stream); host
 * entry points copy in and out around the same solve.  Return values are the
 * IPT_CUDA_* status codes of ipt_cuda.h.
 */
#ifndef IPT_GB300_IPT_BLOCK_H
#define IPT_GB300_IPT_BLOCK_H

#include "ipt_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Precision of the IPT stage's block product Delta X. */
enum {
    IPT_BLOCK_FP64 = 0, /* FP64 SIMT product (the plain path) */
    IPT_BLOCK_FP16 = 1, /* FP16 tensor cores (tcgen05), FP32 accumulation */
    IPT_BLOCK_BF16 = 2, /* BF16 tensor cores (tcgen05), FP32 accumulation */
    IPT_BLOCK_TF32 = 3, /* TF32 tensor cores (tcgen05), FP32 accumulation */
    IPT_BLOCK_FP32 = 4, /* FP32 SIMT sweeps, then FP64 (batched solver only) */
    IPT_BLOCK_DF64 = 5  /* FP64-accurate double-float arithmetic on the FP32 pipe
                           (batched solver's certifying sweeps only) */
};

/* Solver strategy.  REFINE (default): IPT fixed point refined to the FP64
 * eigen-residual (low-precision correction solves against FP64 defects),
 * then one Rayleigh-Ritz; falls back to DAVIDSON when the IPT map does not
 * contract.  DAVIDSON: IPT stage, Rayleigh-Ritz, residual-driven Davidson. */
enum {
    IPT_BLOCK_STRATEGY_REFINE = 0,
    IPT_BLOCK_STRATEGY_DAVIDSON = 1
};

/* Davidson preconditioner. */
enum {
    IPT_BLOCK_PRECOND_DIAGONAL = 0, /* t_i = r_i / (d_i - theta), clipped */
    IPT_BLOCK_PRECOND_MLP = 1       /* learned per-row correction, diagonal fallback */
};

typedef struct {
    int ipt_precision;      /* IPT_BLOCK_FP64 / _FP16 / _BF16 / _TF32 */
    int oversample;         /* extra IPT columns carried into Rayleigh-Ritz (>= 0) */
    int ipt_maxiter;        /* IPT iterations before Rayleigh-Ritz */
    double ipt_tol;         /* stop the IPT stage once ||F(X)-X||_F/||X||_F <= ipt_tol */
    int ipt_check_every;    /* fixed-point residual read back every this many iterations
                               (default 8) */
    double residual_tol;    /* scaled residual target (default 1e-8) */
    int davidson_maxsteps;  /* Davidson steps after the first Rayleigh-Ritz */
    int max_basis;          /* restart size; 0 = automatic */
    int preconditioner;     /* IPT_BLOCK_PRECOND_* */
    const float *mlp_params;/* device parameters of the learned preconditioner */
    void *stream;           /* cudaStream_t, NULL = legacy default stream */
    int strategy;           /* IPT_BLOCK_STRATEGY_* */
    int refine_maxiter;     /* FP64 defect products of the refinement (plain FP64: IPT steps) */
    int inner_maxiter;      /* low-precision correction iterations per refinement step */
    double inner_tol;       /* stop the correction solve at this relative change */
} IPTBlockOptions;

typedef struct {
    int n;
    int k;
    int converged;              /* 1 if every pair met residual_tol */
    int ipt_iterations;
    int davidson_steps;
    int restarts;
    int basis_cols;             /* final Rayleigh-Ritz basis size */
    long long fp64_matvecs;     /* FP64 block-product columns */
    long long lowp_matvecs;     /* low-precision block-product columns */
    double ipt_fixed_point_residual;
    double max_scaled_residual;
    double matrix_norm_inf;
    double ipt_ms;              /* device time of the IPT stage */
    double rayleigh_ritz_ms;    /* first CholQR + Rayleigh-Ritz */
    double davidson_ms;
    double total_ms;
    int mlp_steps_accepted;
    int mlp_steps_rejected;
    long long precond_matvecs;  /* block-product columns of the learned correction itself */
} IPTBlockReport;

void ipt_block_default_options(IPTBlockOptions *options);

/* Dense symmetric H on the device; d_vectors (n*k) and d_values (k) are
 * caller-allocated device buffers. */
int ipt_block_solve_dense_device(const double *d_matrix_col_major, int n, int k,
                                 const IPTBlockOptions *options, double *d_vectors,
                                 double *d_values, IPTBlockReport *report);

/* Dense symmetric H in host memory; vectors (n*k) and values (k) are host
 * buffers.  Copies H in, solves, copies the pairs out.  When H is in
 * page-locked memory (8-byte aligned) and the solve is a mixed one
 * (n <= 16384), only its
 * upper triangle (diagonal included) is read, as LAPACK's dsyevd with
 * UPLO = 'U' does: n (n + 1) / 2 entries cross the host link in column
 * chunks while the setup pass of the chunks already on the device runs;
 * otherwise all of H is copied. */
int ipt_block_solve_dense(const double *matrix_col_major, int n, int k,
                          const IPTBlockOptions *options, double *vectors, double *values,
                          IPTBlockReport *report);

/* Symmetric CSR H on the device. */
int ipt_block_solve_csr_device(const int *d_row_ptr, const int *d_col_ind, const double *d_values_csr,
                               int n, int nnz, int k, const IPTBlockOptions *options,
                               double *d_vectors, double *d_values, IPTBlockReport *report);

/* Symmetric CSR H in host memory (sorted by diagonal inside the call; the
 * returned vectors are in the caller's row order). */
int ipt_block_solve_csr(const int *row_ptr, const int *col_ind, const double *values_csr, int n,
                        int nnz, int k, const IPTBlockOptions *options, double *vectors,
                        double *values, IPTBlockReport *report);

/* Eigenpairs of a small symmetric matrix (m <= 112, column-major, device):
 * the solver of the projected Rayleigh-Ritz matrices, replacing the
 * reference's cusolverDnDsyevd call (IPT_C_GPU/src/ipt_cuda.cu:3143-3218):
 * FP32 tridiagonal stage, FP64 iterative refinement, FP64 polish of
 * near-degenerate clusters.  Writes ascending d_w (m) and orthonormal
 * eigenvectors d_Z (m*m, column-major); synchronises `stream`. */
int ipt_block_symmetric_eig(const double *d_T, int m, double *d_w, double *d_Z, void *stream);

/* ---- block-cluster path (the reference's IPT_BLOCK_CLUSTER) --------------
 *
 * Host only.  Cluster ranges of a symmetric CSC matrix whose diagonal is
 * ascending (the prepared, diagonal-sorted matrix; its columns are first
 * sorted by row with duplicates summed and zeros dropped, as the reference's
 * block-cluster preparation does, ipt_cuda.cu:4568-4575): the targets 0..k-1 are
 * joined with the rows whose diagonal gap is numerically zero or small
 * against their coupling, as the reference's degenerate-subspace detection
 * (IPT_C_GPU/src/ipt_preparation.cu:502-644, environment knobs
 * IPT_EPS_MULTIPLIER, IPT_REL_GAP_TOL, IPT_COUPLING_GAP_RATIO_TOL,
 * IPT_COUPLING_ETA, IPT_MAX_LIFT_BLOCK_SIZE); targets left alone become
 * singleton clusters (IPT_C_GPU/src/ipt_cuda.cu:4114-4132); with `adaptive`
 * the cluster of target requested_k-1 grows by its most strongly coupled
 * outside rows while |H_ij|/gap > coupling_tau (ipt_cuda.cu:4134-4272).
 * ranges receives `*count` inclusive (first, last) pairs in ascending order.
 * IPT_CUDA_INVALID_ARGUMENT for invalid input, a cluster wider than the
 * limit (ipt_cuda.cu:4619-4632) or capacity < *count. */
int ipt_block_cluster_ranges(const int *col_ptr, const int *row_ind, const double *vals, int n,
                             int nnz, int k, int requested_k, double degeneracy_threshold,
                             int adaptive, double coupling_tau, int *ranges, int capacity,
                             int *count, int *limit_hit);

/* The same ranges from a device CSR (rows sorted by column without
 * duplicates, symmetric, ascending diagonal: the prepared matrix of the
 * block-cluster path), with the scans over the nonzeros on the GPU and the
 * detection rules (IPT_C_GPU/src/ipt_preparation.cu:502-644,
 * IPT_C_GPU/src/ipt_cuda.cu:4114-4272) on the host, which reads only the
 * target rows and the rows the adaptive expansion visits.  Runs on `stream`
 * and synchronises it. */
int ipt_block_cluster_ranges_device(const int *d_row_ptr, const int *d_col_ind,
                                    const double *d_vals, int n, int nnz, int k, int requested_k,
                                    double degeneracy_threshold, int adaptive, double coupling_tau,
                                    int *ranges, int capacity, int *count, int *limit_hit,
                                    void *stream);

/* Host only.  The plain sparse path's preparation, for checking (replaces
 * the static ipt_prepare_sparse_csc, IPT_C_GPU/src/ipt_preparation.cu:1375-1648):
 * validation, stable diagonal sort and symmetric permutation, then (lift != 0)
 * the degeneracy lifting of the k targets: groups of numerically close indices
 * rotated into the eigenbasis of their diagonal blocks (classical Jacobi), up
 * to IPT_MAX_LIFT_ROUNDS rounds.  Outputs the prepared matrix as CSC
 * (out_col_ptr n+1, out_row_ind / out_vals `capacity`, *out_nnz), its
 * diagonal (n), basis_to_original (n), and *rot_count rotations: block r
 * covers [rot_first[r], rot_first[r] + rot_size[r]) and its rotation matrix
 * (column-major) follows the previous ones in rot_values.
 * IPT_CUDA_INVALID_ARGUMENT for invalid input, capacities too small, a group
 * wider than IPT_MAX_LIFT_BLOCK_SIZE, gaps still unresolved after the
 * rounds, or a group of a non-symmetric matrix (which the reference lifts only
 * when LAPACK dgeev is linked in; with IPT_GB300_GENERAL_LIFT=1 it is lifted
 * here by a general similarity, eigenvectors from this library's real
 * eigensolver, unless an eigenvalue is complex or the eigenvector matrix
 * singular). */
int ipt_block_prepare_csc(const int *col_ptr, const int *row_ind, const double *vals, int n,
                          int k, int nnz, int lift, double degeneracy_threshold, int *out_col_ptr,
                          int *out_row_ind, double *out_vals, int capacity, int *out_nnz,
                          double *out_diag, int *out_perm, int *rot_first, int *rot_size,
                          int rot_capacity, double *rot_values, int rot_values_capacity,
                          int *rot_count);

/* ---- the reference's binary CSC matrix cache (host only) -----------------
 *
 * The file its molecule benchmarks write for a generated FCI Hamiltonian
 * (write_ch4_matrix_cache / read_ch4_matrix_cache,
 * IPT_C_GPU/test/sparse/CH4/benchmark_ch4_sto6g_fci_15876_ipt.cu:1015-1121):
 * a 56-byte little-endian header (magic "IPT" + tag + "C1", version 1, n,
 * nnz, ||H||_inf, orbital and electron counts), then int32 col_ptr[n+1],
 * int32 row_ind[nnz], double values[nnz], double diagonal[n]. */
typedef struct {
    char magic[9];          /* e.g. "IPTCH4C1", NUL-terminated */
    int version;            /* 1 */
    int n;
    int nnz;
    double matrix_inf_norm;
    int norb;
    int nelec;
    int neleca;
    int nelecb;
    int na;
    int nb;
} IPTCscCacheInfo;

/* The header of a cache file; IPT_CUDA_INVALID_ARGUMENT if it is not one. */
int ipt_block_csc_cache_info(const char *path, IPTCscCacheInfo *info);

/* The whole file into caller arrays (n_capacity >= n, nnz_capacity >= nnz,
 * from ipt_block_csc_cache_info).  IPT_CUDA_INVALID_ARGUMENT for a short or
 * foreign file, arrays that are not a valid CSC, or a norm that is negative
 * or not finite (the reference's checks). */
int ipt_block_csc_cache_read(const char *path, int *col_ptr, int *row_ind, double *values,
                             double *diagonal, int n_capacity, int nnz_capacity,
                             IPTCscCacheInfo *info);

/* Write a cache file (info->magic and the counts from the caller; version
 * 1); the data go to path.tmp, renamed over path when complete. */
int ipt_block_csc_cache_write(const char *path, const IPTCscCacheInfo *info, const int *col_ptr,
                              const int *row_ind, const double *values, const double *diagonal);

/* Block-cluster basis (replaces ipt_block_cluster_solve_basis_gpu, one call
 * per cluster, IPT_C_GPU/src/ipt_cuda.cu:2871-3037): for each of the
 * `nclusters` host ranges (inclusive, ascending, disjoint, width <= 64) the
 * fixed point X'[i,:] = (d_i I - h^T)^{-1} (d_i X[i,:] - Y[i,:]) with
 * Y = H X, h = Y[first..last, :] and identity rows inside the cluster, from
 * the identity columns, until ||X'-X||_F / max(1, ||X||_F) <= tol (tol <= 0:
 * 1e-12) or maxiter; damping outside (0, 1] counts as 1.  H is device CSR
 * (0-based) with ascending diagonal d_diag; d_basis (n x sum of widths,
 * column-major) gets the clusters' columns one after the other; iterations
 * and residuals (host, nclusters) the per-cluster iteration counts and last
 * fixed-point residuals.  From 16384 rows the products H X are formed in
 * double-float arithmetic (about 48 bits, the Davidson products' policy,
 * tuning knob IPT_GB300_DF_DAVIDSON).  IPT_CUDA_INVALID_ARGUMENT for a
 * singular row system or a non-finite iterate.  Synchronises `stream`. */
int ipt_block_cluster_basis(const int *d_row_ptr, const int *d_col_ind, const double *d_vals,
                            int n, int nnz, const double *d_diag, const int *ranges,
                            int nclusters, int maxiter, double tol, double damping,
                            double *d_basis, int *iterations, double *residuals, void *stream);

/* One block-cluster update of a single cluster [first, first+m) (replaces
 * ipt_block_cluster_update_kernel, IPT_C_GPU/src/ipt_cuda.cu:2280-2384):
 * d_next from d_basis and d_y = H d_basis (both n x m, device), with the
 * kernel's damping rule (value = (1-damping) x + damping value when
 * damping < 1).  *singular = 1 when a row system is singular (pivot not above
 * 64 DBL_EPSILON or not finite) or a value is not finite.  Synchronises
 * `stream`. */
int ipt_block_cluster_update(const double *d_basis, const double *d_y, const double *d_diag,
                             int n, int first, int m, double damping, double *d_next,
                             int *singular, void *stream);

/* Cholesky factor inverse of a small SPD Gram matrix (m <= 112, column-major,
 * device): G = R^T R, d_Rinv = R^{-1} (upper triangular, column-major), the
 * step of CholQR that replaces the reference's cusolverDnDpotrf + cublasDtrsm
 * pair (IPT_C_GPU/mixed/ipt_rayleigh_mixed_mpqr_cuda.cu:335-360).  A matrix
 * that is not numerically positive definite is factored as G + shift*I with
 * the shift grown from 1e-14 trace(G) by 100x per retry; *shifts gets the
 * number of retries (0 = plain).  Returns IPT_CUDA_INVALID_ARGUMENT with
 * *shifts = -1 when 12 retries do not suffice.  precision 0: FP64; 1:
 * double-float (hi + lo FP32 pairs, about 48 bits) for m <= 32 and no shift,
 * FP64 otherwise.  Synchronises `stream`. */
int ipt_block_cholesky_inverse(const double *d_G, int m, double *d_Rinv, int *shifts,
                               int precision, void *stream);

/* ---- allocation-free FP64 dense solve ------------------------------------ */

/* No counterpart in the reference.  The tolerance-stopped FP64 dense IPT of
 * ipt_cuda_device_tol for callers that cannot let the library allocate
 * device memory (an application-owned memory pool, no allocation after
 * start-up, or pipelines that cudaFree's device-wide synchronisation would
 * stall).  The caller passes H and the outputs d_vectors (n*k) and d_values
 * (k); all scratch lives in one 16 MiB static device array that each GPU
 * loading the library keeps until exit, so n*k is limited to about 1.0e6
 * (2*n*k + n + n*k/128 doubles); larger sizes return
 * IPT_CUDA_INVALID_ARGUMENT with a message on stderr.  Runs on `stream`
 * (cudaStream_t, NULL = legacy default stream).  Every iteration reads two
 * norms back and synchronises the stream, so the entry must never be called
 * inside a stream capture.  Calls share the scratch: calls that overlap on
 * the GPU race and must be serialised by the caller. */
int ipt_cuda_device_tol_noalloc(const double *d_matrix_col_major, int n, int k, double tol,
                                int maxiter, void *stream, double *d_vectors, double *d_values,
                                int *iterations_done_out, double *fixed_point_residual_out);

/* ---- learned Davidson preconditioner -------------------------------------- */

/* No counterpart in the reference, whose Davidson step uses the diagonal
 * correction t_i = r_i / (d_i - theta) (IPT_C_GPU/src/ipt_cuda.cu:2449-2465).
 * The learned correction is t1 + o o u: t1 the plain diagonal correction,
 * u = -(D - theta)^-1 (H - D) t1 the second term of the Neumann series of
 * (H - theta)^-1 r (one block product per step, counted in
 * IPTBlockReport.precond_matvecs), and o a per-row weight from an MLP
 * (IPT_BLOCK_MLP_FEATURES -> 64 -> 64 -> 1, ReLU, FP32 parameters on the
 * device; clamped to [-1, 3]; o = 0 is the plain preconditioner) fed with
 * six row features of the selected Ritz pair.  IPTBlockOptions.preconditioner
 * = IPT_BLOCK_PRECOND_MLP with mlp_params = the trained parameters enables it.
 * Every learned step is checked against the FP64 residual: unless the largest
 * scaled residual drops at least as much as a plain step is expected to (the
 * geometric mean drop of the solve's plain steps, 0.5 before the first, and
 * never less than a 25 % cut) the step is redone with the diagonal
 * correction; two rejections in a row switch the learned correction off
 * (IPTBlockReport counts accepted and rejected learned steps).
 *
 * Training rows are 8 floats: the 6 features, the target weight and its row
 * weight; the loss is the mean of weight * (MLP(features) - target)^2. */
#define IPT_BLOCK_MLP_FEATURES 6
#define IPT_BLOCK_MLP_ROW 8

/* Number of FP32 parameters (4673). */
int ipt_block_mlp_param_count(void);
/* Seeded initialisation (uniform, fan-in scaled; output bias 1, i.e. the
 * plain correction). */
int ipt_block_mlp_init(float *d_params, unsigned long long seed, void *stream);
/* d_out[r] = MLP(d_rows[r*row_stride .. +6]) for r < rows. */
int ipt_block_mlp_forward(const float *d_params, const float *d_rows, long long rows,
                          int row_stride, float *d_out, void *stream);
/* Gradient of the weighted squared error over all `rows` training rows:
 * d_grad[0..param_count) = dL/dparams, d_grad[param_count] = L. */
int ipt_block_mlp_loss_grad(const float *d_params, const float *d_rows, long long rows,
                            float *d_grad, void *stream);
/* `steps` Adam steps (lr, betas 0.9/0.999, eps 1e-8) on batches of `batch`
 * rows drawn by a seeded hash; d_loss_history (steps floats, may be NULL)
 * receives each batch's loss before its update. */
int ipt_block_mlp_train(float *d_params, const float *d_rows, long long rows, int steps,
                        int batch, float lr, unsigned long long seed, float *d_loss_history,
                        void *stream);
/* Training data from the plain solver: runs the diagonal-preconditioned
 * Davidson solver on a CSR matrix (diagonal ascending) and, at every
 * correction, appends per row the features and the exact-correction target
 * computed against the caller's converged eigenvectors d_exact_vectors
 * (n x exact_cols, column-major).  At most `capacity` rows are written;
 * *rows_written reports how many.  With options->preconditioner =
 * IPT_BLOCK_PRECOND_MLP the solver follows the learned corrections of
 * options->mlp_params instead (rows along the learned trajectory). */
int ipt_block_mlp_collect_csr(const int *d_row_ptr, const int *d_col_ind,
                              const double *d_values_csr, int n, int nnz, int k,
                              const IPTBlockOptions *options, const double *d_exact_vectors,
                              int exact_cols, float *d_rows, long long capacity,
                              long long *rows_written, IPTBlockReport *report);

/* ---- batched dense solver ----------------------------------------------- */

/* No counterpart in the reference, which solves one matrix per call.  Many
 * independent dense symmetric instances (column-major FP64 on the device,
 * n >= 1, 1 <= k <= min(16, n)) are solved by one persistent kernel with the
 * reference's plain IPT map (targets = the first k diagonal positions,
 * X_jj = 1, IPT_C_GPU/src/ipt_cuda.cu:1644-1703), stopping each instance at
 * the scaled eigen-residual residual_tol (residuals r_j = H x_j - (HX)_jj x_j,
 * the IPT map's own) and returning the certified block and its Rayleigh
 * quotients x_j^T H x_j / x_j^T x_j.  precision IPT_BLOCK_FP32 runs FP32
 * sweeps to lowp_tol first, then the FP64-accurate sweeps; those run on the
 * FP64 pipe (certify_precision IPT_BLOCK_FP64) or in double-float arithmetic
 * on the FP32 pipe (IPT_BLOCK_DF64, about 2^-48 relative per term; the
 * default after FP32 sweeps).  The plan owns all
 * scratch and a captured CUDA graph of the whole batch; run() launches the
 * graph, autotune() times the launch shapes on the real batch and
 * re-captures the fastest.  Instance pointers must stay valid for the
 * plan's lifetime. */
typedef struct {
    const double *H;  /* n x n, column-major, device */
    int n;
    int k;
    double *vectors;  /* n x k, column-major, device (output) */
    double *values;   /* k, device (output) */
} IPTBatchInstance;

typedef struct {
    int precision;        /* IPT_BLOCK_FP64 or IPT_BLOCK_FP32 */
    double residual_tol;  /* scaled eigen-residual target (1e-8) */
    int maxiter;          /* FP64 sweeps per instance */
    int lowp_maxiter;     /* FP32 sweeps per instance */
    double lowp_tol;      /* FP32 fixed-point residual at which to switch */
    int threads;          /* 0 = default (256) or 128 / 256 / 512 */
    int chunk;            /* 0 = default (128) or 64 / 128 rows of H per stage */
    int certify_precision; /* -1 = default (IPT_BLOCK_DF64 after FP32 sweeps,
                              IPT_BLOCK_FP64 otherwise), IPT_BLOCK_FP64 or
                              IPT_BLOCK_DF64 */
} IPTBatchOptions;

typedef struct {
    int converged;
    int status;               /* 0, or 1 for a non-finite sweep */
    int iterations;           /* all sweeps */
    int fp64_iterations;
    double max_scaled_residual;
    double latency_ms;        /* device time from the instance's start to its end */
    double completion_ms;     /* from the first instance's start to this one's end */
} IPTBatchReport;

void ipt_block_batch_default_options(IPTBatchOptions *options);
int ipt_block_batch_plan_create(const IPTBatchInstance *instances, int count,
                                const IPTBatchOptions *options, void **plan);
int ipt_block_batch_plan_run(void *plan, void *stream);
int ipt_block_batch_plan_autotune(void *plan, void *stream, int *threads, int *chunk,
                                  double *best_ms);
int ipt_block_batch_plan_reports(void *plan, IPTBatchReport *reports);
/* The launch shape in use: threads per CTA, rows of H per stage, cluster size
 * of the launch (1: no clusters), the number of CTAs, and how many of the
 * most expensive instances a whole cluster solves together. */
int ipt_block_batch_plan_shape(void *plan, int *threads, int *chunk, int *cluster, int *ctas,
                               int *team_instances);
int ipt_block_batch_plan_destroy(void *plan);

/* ---- matrix-free FCI-like Hamiltonians ------------------------------------ */

/* No counterpart in the reference (its FCI matrices are assembled into CSC
 * from PySCF integrals, IPT_C_GPU/test/sparse/H2O/
 * benchmark_h2o_631g_cas10e10o_primme_vs_ipt.cu:390-766).  H over all
 * (alpha, beta) occupation-string pairs of norb orbitals, never stored:
 * eps_p = 0.5 p + 0.05 g(31, p), H_II = E(I) + 0.01 g(32, I),
 * H_IJ = offdiag_sigma g(33, min(I,J), max(I,J)) exp(-|E(J) - E(I)|) for
 * single and double excitations (E = summed occupied eps; g a seeded
 * Box-Muller normal evaluated in FP32 by the library's own deterministic
 * log/cos/exp).  Determinant I = ia * (number of beta strings) + ib. */
typedef struct {
    int norb;
    int nalpha;
    int nbeta;
    unsigned long long seed;
    double offdiag_sigma;   /* 0.05 for the FCI-like workloads */
} IPTFciSpec;

int ipt_fci_dimension(const IPTFciSpec *spec, long long *n);
int ipt_fci_diagonal(const IPTFciSpec *spec, double *d_diag, void *stream);
/* d_Y (n x k, column-major) = H d_X; precision IPT_BLOCK_FP64 (FP64
 * accumulation), IPT_BLOCK_FP32 or IPT_BLOCK_BF16 (X rounded to that type,
 * FP32 accumulation). */
int ipt_fci_sigma(const IPTFciSpec *spec, const double *d_X, int k, double *d_Y, int precision,
                  void *stream);
/* k lowest eigenpairs by Davidson on the matrix-free sigma, starting from the
 * unit vectors of the lowest diagonal entries.  ipt_precision IPT_BLOCK_BF16
 * or IPT_BLOCK_FP32 runs a low-precision-sigma phase first (to a scaled
 * residual of 1e-2 / 1e-5) and finishes with FP64 sigma to residual_tol;
 * IPT_BLOCK_FP64 uses FP64 sigma throughout. */
int ipt_block_solve_fci(const IPTFciSpec *spec, int k, const IPTBlockOptions *options,
                        double *d_vectors, double *d_values, IPTBlockReport *report);

/* ---- double-FP32 operands ------------------------------------------------- */

/* hi = RN_float(a), lo = RN_float(a - hi) elementwise (a = hi + lo to about
 * 2^-48 relative): the operands of the FP64-accurate products that run on the
 * FP32 pipe.  The device version converts on the integer pipe (GB300's FP64
 * pipe, which also executes double<->float conversions, is too slow for a
 * pass over a large matrix); results are bit-identical to the FP64
 * conversions.  The host version runs the same conversion on the CPU. */
int ipt_block_split_double(const double *d_in, long long count, float *d_hi, float *d_lo,
                           void *stream);
int ipt_block_split_double_host(const double *in, long long count, float *hi, float *lo);

/* ---- FP64-accurate product on the tensor cores ------------------------------ */

/* Y = H X for a column-major n x n H and n x c X (device buffers, ld n),
 * the FP64-accurate block product that replaces the reference's FP64
 * cublasDgemm (IPT_C_GPU/src/mixed_precision/ipt_mixed_precision_cuda.cu:
 * 917,958) in this library's mixed solve.  The diagonal of H is applied in
 * FP64; H minus its diagonal runs on the FP16 tensor cores by an error-free
 * split of both operands into six 8-bit digit slices with one power-of-two
 * scale per row of H and per column of X (Ozaki, Ogita, Oishi and Rump,
 * Numer. Algorithms 59 (2012); the fixed-point form of Mukunoki et al., ISC
 * 2020).  The error of an entry is below about 2^-46 times
 * max_l |H_il| max_l |X_lc| times the number of terms, plus the rounding of
 * |H_ii X_ic|.  The solver splits H once per solve; this entry splits it on
 * every call (for checking and one-off products).  Runs on `stream`
 * (cudaStream_t, NULL = legacy default stream) and synchronises it. */
int ipt_block_accurate_product(const double *d_H, int n, const double *d_X, int c,
                               double *d_Y, void *stream);

/* The split of the product above on the host, for checking: the exponent e
 * with max_abs < 2^e (*exponent_out; 0 when max_abs is 0, INT_MAX for a
 * non-finite max_abs) and the six digits of round(v 2^(48 - e)) in balanced
 * base 256 (digits_out[6 i + s], s = 0 most significant) of every value. */
int ipt_block_accurate_split_host(const double *values, long long count, double max_abs,
                                  int *exponent_out, int *digits_out);

/* ---- Householder column signs -------------------------------------------- */

/* Part of the orthonormalisation step of ipt_rayleigh_mixed_tf32_cuda_device_tol,
 * which replaces the reference's Householder QR (cusolverDnDgeqrf/Dorgqr,
 * IPT_C_GPU/src/mixed_precision/ipt_rayleigh_mixed_cuda.cu:141-254) by
 * CholQR.  Given the top k x k block (column-major) of an orthonormal
 * n x k factor Q_c whose R has a positive diagonal, signs[j] is the sign of
 * the j-th diagonal entry of R in a LAPACK Householder QR of the same
 * block, so that Q_c diag(signs) is the Householder factor.  Host-only. */
int ipt_block_householder_signs(const double *top, int k, int n, double *signs);

/* ---- instrumentation ---------------------------------------------------- */

/* Number of kernels this library has launched in the calling process. */
long long ipt_block_launch_count(void);

/* Per-kernel CUDA-event timing of the main kernels (off by default).  When
 * enabled, every launch of an instrumented kernel is bracketed by events on
 * its own stream.  Kernel ids: 0 low-precision product (tcgen05 / FP32 SIMT),
 * 1 low-precision update, 2 FP64 dense product, 3 FP64 update / partial sum,
 * 4 FP64 CSR product, 5 small eigensolver, 6 Gram products, 7 tall-by-small
 * products, 8 learned-preconditioner kernels, 9 block-cluster update. */
void ipt_block_profile_enable(int on);
void ipt_block_profile_reset(void);
int ipt_block_profile_read(int kernel, const char **name, double *total_ms, long long *launches);

/* Phase marks of the solvers (off by default).  Enabling clears the list.
 * While enabled, each mark point of a solve (setup passes, IPT checks,
 * refinement steps, Rayleigh-Ritz, end) launches a one-thread kernel that
 * stores the GPU global timer (ns) in stream order, and keeps the host's
 * steady clock (ns) at the call: gpu - host offsets that grow between two
 * marks show the GPU waiting for the host.  read copies the first count
 * marks (labels are static strings); at most 4096 marks are kept. */
int ipt_block_trace_enable(int on);
int ipt_block_trace_count(void);
int ipt_block_trace_read(int count, const char **labels, long long *host_ns, long long *gpu_ns);

/* FP64 FMA throughput of the current device in TFLOP/s (a short DFMA
 * throughput kernel); the FP64 roofline denominator. */
int ipt_block_measure_fp64_peak(double *tflops);
/* FP32 FMA throughput in TFLOP/s; the denominator of the double-FP32
 * (FP64-accurate) products. */
int ipt_block_measure_fp32_peak(double *tflops);

#ifdef __cplusplus
}
#endif

#endif /* IPT_GB300_IPT_BLOCK_H */
