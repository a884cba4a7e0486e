/*
 * ipt_cuda.h - the block-IPT solver C ABI, binary compatible with the
 * FJennie/BLOCK_IPT reference declarations (IPT_C_GPU/src/ipt_cuda.cu:75-312,
 * IPT_C_GPU/src/mixed_precision/ipt_mixed_precision_cuda.cu:12-84).
 *
 * A caller that was built against the reference declarations links against
 * libipt_gb300.so instead of compiling ipt_cuda.cu into its own unit.  Every
 * entry point keeps the reference's name, argument order, argument meaning,
 * status codes and ownership rules:
 *
 *  - host entry points (ipt_cuda*, ipt_cuda_sparse_csc*) copy the inputs to the
 *    device, return host vectors/values malloc'd inside IPTCudaResult; the
 *    caller releases them with ipt_cuda_free_result();
 *  - device entry points (*_device*) take device pointers and a cuBLAS handle;
 *    the solver runs on the stream attached to that handle and returns
 *    cudaMalloc'd buffers released with ipt_cuda_free_device_result();
 *  - on error every output pointer is NULL and the result is reset.
 *
 * Dense matrices are column-major doubles with leading dimension n.  Sparse
 * matrices are 0-based int32 CSC (col_ptr[n+1], row_ind[nnz], values[nnz]).
 *
 * The struct layouts below are part of the binary interface and follow the
 * reference field-for-field (IPT_C_GPU/src/ipt_cuda.cu:92-260,
 * IPT_C_GPU/src/mixed_precision/ipt_mixed_precision_cuda.cu:19-59).
 */
#ifndef IPT_GB300_IPT_CUDA_H
#define IPT_GB300_IPT_CUDA_H

#ifdef __cplusplus
extern "C" {
#endif

/* Opaque cuBLAS handle; identical to the typedef in cublas_api.h, so this
 * header can be included with or without the cuBLAS headers. */
typedef struct cublasContext *cublasHandle_t;

/* Status codes: IPT_C_GPU/src/ipt_cuda.cu:82-90. */
enum {
    IPT_CUDA_SUCCESS = 0,
    IPT_CUDA_INVALID_ARGUMENT = 1,
    IPT_CUDA_ALLOCATION_FAILED = 2,
    IPT_CUDA_CUDA_ERROR = 3,
    IPT_CUDA_CUBLAS_ERROR = 4,
    IPT_CUDA_CUSPARSE_ERROR = 5,
    IPT_CUDA_CUSOLVER_ERROR = 6
};

/* One Davidson history record (IPT_C_GPU/src/ipt_cuda.cu:92-133). */
typedef struct {
    int davidson_step;
    int active_pair_index;
    double residual_before;
    double residual_after;
    int accepted;
    int basis_cols;
    double max_relative_eigen_residual;
    int max_relative_eigen_residual_index;
    double pair_28_residual;
    double pair_29_residual;
    double orthogonality_max_abs_error;
    int restarted;
    int best_so_far_updated;
    int best_so_far_step;
    double best_so_far_max_residual;
    double pair28_best_residual;
    double pair29_best_residual;
    int accept_global_ok;
    int accept_active_ok;
    int accept_locked_safe;
    char accept_reason[64];
    int accepted_steps;
    int rejected_steps;
    int early_jump_to_continuation;
    double gap28_29;
    double relative_gap28_29;
    double cluster_residual_fro_before;
    double cluster_residual_fro_after;
    double cluster_residual_max_before;
    double cluster_residual_max_after;
    double ritz_overlap_28_28;
    double ritz_overlap_28_29;
    double ritz_overlap_29_28;
    double ritz_overlap_29_29;
    int ritz_overlap_swap_detected;
    char pair28_lock_state[16];
    char pair29_lock_state[16];
    int cluster_hard_locked;
    int cluster_soft_locked_count;
} IPTDavidsonHistoryEntry;

/* Per-candidate Davidson selection record (IPT_C_GPU/src/ipt_cuda.cu:135-147). */
typedef struct {
    int davidson_step;
    int pair_index;
    double residual;
    int selected_by_residual;
    int selected_forced;
    int selected_auto_cluster;
    int skipped_converged_in_cluster;
    int skipped_linear_dependent;
    int skipped_locked_old_logic_should_not_happen;
    double correction_norm_before_ortho;
    double correction_norm_after_ortho;
} IPTDavidsonSelectionEntry;

/* Per-step block record (IPT_C_GPU/src/ipt_cuda.cu:149-194). */
typedef struct {
    int davidson_step;
    char active_pairs[64];
    int accepted_corrections;
    int rejected_corrections;
    char correction_norm_before_ortho[256];
    char correction_norm_after_ortho[256];
    double residual_before_global;
    double residual_after_global;
    double pair_28_before;
    double pair_28_after;
    double pair_29_before;
    double pair_29_after;
    int accepted;
    char reject_reason[64];
    int basis_cols_before;
    int basis_cols_after;
    double orthogonality_error_before;
    double orthogonality_error_after;
    int best_so_far_updated;
    int best_so_far_step;
    double best_so_far_max_residual;
    double pair28_best_residual;
    double pair29_best_residual;
    int accept_global_ok;
    int accept_active_ok;
    int accept_locked_safe;
    char accept_reason[64];
    int accepted_steps;
    int rejected_steps;
    int early_jump_to_continuation;
    double gap28_29;
    double relative_gap28_29;
    double cluster_residual_fro_before;
    double cluster_residual_fro_after;
    double cluster_residual_max_before;
    double cluster_residual_max_after;
    double ritz_overlap_28_28;
    double ritz_overlap_28_29;
    double ritz_overlap_29_28;
    double ritz_overlap_29_29;
    int ritz_overlap_swap_detected;
    char pair28_lock_state[16];
    char pair29_lock_state[16];
    int cluster_hard_locked;
    int cluster_soft_locked_count;
} IPTDavidsonBlockHistoryEntry;

/* Host result (IPT_C_GPU/src/ipt_cuda.cu:196-260). */
typedef struct {
    int n;
    int k;
    int iterations;
    double *vectors; /* column-major n-by-k eigenvector estimate */
    double *values;  /* length k */
    int basis_cols;
    long long matvecs;
    double preparation_time_sec;
    double transfer_setup_time_sec;
    double iteration_time_sec;
    double rayleigh_ritz_time_sec;
    double davidson_time_sec;
    double solve_time_sec;
    double fixed_point_residual;
    int oversample;
    int rayleigh_ritz_used_qr;
    double basis_orthogonality_frobenius_error;
    double basis_orthogonality_max_abs_error;
    double ritz_vectors_orthogonality_frobenius_error;
    double ritz_vectors_orthogonality_max_abs_error;
    int basis_has_nan_or_inf;
    int ritz_vectors_has_nan_or_inf;
    int davidson_attempted;
    int davidson_accepted;
    int davidson_target_index;
    double davidson_residual_before;
    double davidson_residual_after;
    double davidson_denom_clip;
    int adaptive_block_enabled;
    double adaptive_coupling_tau;
    int adaptive_limit_hit;
    int adaptive_target_block_start;
    int adaptive_target_block_end;
    char adaptive_added_indices[256];
    int davidson_history_count;
    IPTDavidsonHistoryEntry *davidson_history;
    int davidson_restart_count;
    int davidson_selection_history_count;
    IPTDavidsonSelectionEntry *davidson_selection_history;
    int davidson_block_history_count;
    IPTDavidsonBlockHistoryEntry *davidson_block_history;
    int best_so_far_enabled;
    int best_so_far_updated;
    int best_so_far_update_count;
    int best_so_far_step;
    char best_so_far_source[32];
    int best_so_far_basis_cols;
    double best_so_far_max_residual;
    int best_so_far_max_residual_index;
    int final_returned_from_best_so_far;
    double pair28_best_residual;
    double pair29_best_residual;
    int accepted_steps;
    int rejected_steps;
    int early_jump_to_continuation;
    double gap28_29;
    double relative_gap28_29;
    double cluster_residual_fro;
    double cluster_residual_max;
    char pair28_lock_state[16];
    char pair29_lock_state[16];
    int cluster_hard_locked;
    int cluster_soft_locked_count;
} IPTCudaResult;

/* Mixed-precision device results
 * (IPT_C_GPU/src/mixed_precision/ipt_mixed_precision_cuda.cu:19-59). */
typedef struct {
    int n;
    int k;
    int fp16_iterations;
    int fp64_iterations;
    double fp16_time_sec;
    double fp64_time_sec;
    double total_time_sec;
    double fp16_fixed_point_residual;
    double fp64_fixed_point_residual;
    double *d_vectors;
    double *d_values;
} IPTMixedCudaDeviceResult;

typedef struct {
    int n;
    int k;
    int fp32_iterations;
    int fp64_iterations;
    double fp32_time_sec;
    double fp64_time_sec;
    double total_time_sec;
    double fp32_fixed_point_residual;
    double fp64_fixed_point_residual;
    double *d_vectors;
    double *d_values;
} IPTMixedFP32CudaDeviceResult;

typedef struct {
    int n;
    int k;
    int tf32_iterations;
    int fp64_iterations;
    double tf32_time_sec;
    double fp64_time_sec;
    double total_time_sec;
    double tf32_fixed_point_residual;
    double fp64_fixed_point_residual;
    double *d_vectors;
    double *d_values;
} IPTMixedTF32CudaDeviceResult;

/* Rayleigh-mixed device result
 * (IPT_C_GPU/src/mixed_precision/ipt_rayleigh_mixed_cuda.cu:19-34; the same
 * struct in IPT_C_GPU/mixed/ipt_rayleigh_mixed_mpqr_cuda.cu:19-34). */
typedef struct {
    int n;
    int k;
    int tf32_iterations;
    int fp64_iterations;
    double tf32_time_sec;
    double orthogonalize_time_sec;
    double rayleigh_transform_time_sec;
    double fp64_time_sec;
    double backtransform_time_sec;
    double total_time_sec;
    double tf32_fixed_point_residual;
    double fp64_fixed_point_residual;
    double *d_vectors;
    double *d_values;
} IPTRayleighMixedCudaDeviceResult;

/* --- utilities: IPT_C_GPU/src/ipt_cuda.cu:262-264 ------------------------ */
const char *ipt_cuda_status_string(int status);
void ipt_cuda_free_result(IPTCudaResult *result);
void ipt_cuda_free_device_result(double *d_vectors, double *d_values);

/* --- dense, host buffers: IPT_C_GPU/src/ipt_cuda.cu:265-275 -------------- */
int ipt_cuda(const double *matrix_col_major, int n, int k, int iterations,
             IPTCudaResult *result);
int ipt_cuda_tol(const double *matrix_col_major, int n, int k, double tol,
                 int maxiter, IPTCudaResult *result);
int ipt_cuda_with_initial(const double *matrix_col_major,
                          const double *initial_vectors_col_major, int n,
                          int k, int iterations, IPTCudaResult *result);
int ipt_cuda_with_initial_tol(const double *matrix_col_major,
                              const double *initial_vectors_col_major, int n,
                              int k, double tol, int maxiter,
                              IPTCudaResult *result);

/* --- dense, device buffers: IPT_C_GPU/src/ipt_cuda.cu:276-283 ------------ */
int ipt_cuda_device(const double *d_matrix_col_major, int n, int k,
                    int iterations, cublasHandle_t handle,
                    double **d_vectors_out, double **d_values_out);
int ipt_cuda_device_tol(const double *d_matrix_col_major, int n, int k,
                        double tol, int maxiter, cublasHandle_t handle,
                        double **d_vectors_out, double **d_values_out,
                        int *iterations_done_out,
                        double *fixed_point_residual_out);

/* --- sparse CSC, host buffers: IPT_C_GPU/src/ipt_cuda.cu:284-298 --------- */
int ipt_cuda_sparse_csc(const int *col_ptr, const int *row_ind,
                        const double *matrix_values, int n, int k, int nnz,
                        int iterations, IPTCudaResult *result);
int ipt_cuda_sparse_csc_tol(const int *col_ptr, const int *row_ind,
                            const double *matrix_values, int n, int k,
                            int nnz, double tol, int maxiter,
                            IPTCudaResult *result);
int ipt_cuda_sparse_csc_with_initial(
    const int *col_ptr, const int *row_ind, const double *matrix_values,
    const double *initial_vectors_col_major, int n, int k, int nnz,
    int iterations, IPTCudaResult *result);
int ipt_cuda_sparse_csc_with_initial_tol(
    const int *col_ptr, const int *row_ind, const double *matrix_values,
    const double *initial_vectors_col_major, int n, int k, int nnz,
    double tol, int maxiter, IPTCudaResult *result);

/* --- sparse CSC, device buffers: IPT_C_GPU/src/ipt_cuda.cu:299-308 ------- */
int ipt_cuda_sparse_csc_device(
    const int *d_col_ptr, const int *d_row_ind,
    const double *d_matrix_values, int n, int k, int nnz, int iterations,
    cublasHandle_t handle, double **d_vectors_out, double **d_values_out);
int ipt_cuda_sparse_csc_device_tol(
    const int *d_col_ptr, const int *d_row_ind,
    const double *d_matrix_values, int n, int k, int nnz, double tol,
    int maxiter, cublasHandle_t handle, double **d_vectors_out,
    double **d_values_out, int *iterations_done_out,
    double *fixed_point_residual_out);

/* --- mixed precision, device buffers:
 *     IPT_C_GPU/src/mixed_precision/ipt_mixed_precision_cuda.cu:61-78 ------ */
void ipt_mixed_precision_cuda_free_device_result(
    IPTMixedCudaDeviceResult *result);
int ipt_mixed_precision_cuda_device_tol(
    const double *d_matrix_col_major, int n, int k, double fp16_tol,
    int fp16_maxiter, double fp64_tol, int fp64_maxiter,
    cublasHandle_t handle, IPTMixedCudaDeviceResult *result);
void ipt_mixed_precision_fp32_cuda_free_device_result(
    IPTMixedFP32CudaDeviceResult *result);
int ipt_mixed_precision_fp32_cuda_device_tol(
    const double *d_matrix_col_major, int n, int k, double fp32_tol,
    int fp32_maxiter, double fp64_tol, int fp64_maxiter,
    cublasHandle_t handle, IPTMixedFP32CudaDeviceResult *result);
void ipt_mixed_precision_tf32_cuda_free_device_result(
    IPTMixedTF32CudaDeviceResult *result);
int ipt_mixed_precision_tf32_cuda_device_tol(
    const double *d_matrix_col_major, int n, int k, double tf32_tol,
    int tf32_maxiter, double fp64_tol, int fp64_maxiter,
    cublasHandle_t handle, IPTMixedTF32CudaDeviceResult *result);

/* --- Rayleigh-mixed, device buffers:
 *     IPT_C_GPU/src/mixed_precision/ipt_rayleigh_mixed_cuda.cu:36-41 (driver
 *     :274-400; mixed-CholQR twin IPT_C_GPU/mixed/ipt_rayleigh_mixed_mpqr_cuda.cu:406-538).
 * TF32 IPT of the k lowest diagonal positions to tf32_tol (tensor cores),
 * orthonormal basis Q of that block with the column signs of a Householder
 * QR, B = sym(Q^T H Q), FP64 IPT on the k x k matrix B to fp64_tol, and the
 * vectors Q Z (n x k, column-major, Z with Z_jj = 1) and values (B Z)_jj in
 * cudaMalloc'd buffers that ipt_rayleigh_mixed_cuda_free_device_result
 * releases.  Runs on the handle's stream. ------------------------------- */
void ipt_rayleigh_mixed_cuda_free_device_result(
    IPTRayleighMixedCudaDeviceResult *result);
int ipt_rayleigh_mixed_tf32_cuda_device_tol(
    const double *d_matrix_col_major, int n, int k, double tf32_tol,
    int tf32_maxiter, double fp64_tol, int fp64_maxiter,
    cublasHandle_t handle, IPTRayleighMixedCudaDeviceResult *result);

#ifdef __cplusplus
}
#endif

#endif /* IPT_GB300_IPT_CUDA_H */
