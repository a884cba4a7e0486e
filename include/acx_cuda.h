/*
 * acx_cuda.h - ACX extrapolation over the IPT map (dense FP64), libipt_gb300.so.
 *
 * Drop-in for the reference's IPT_C_GPU/src/ACX/acx_cuda.cu:12-33 (status
 * codes, ACXCudaResult) and its entry points acx_cuda_status_string,
 * acx_cuda_reset_result, acx_cuda_free_result (:44-80) and
 * acx_cuda_device_tol (:390-620): from the identity columns, alternate
 * order-2 and order-3 cyclic extrapolation steps over the IPT map
 *     F(X) = E + G o (HX - X diag(HX)),  G_ij = 1/(d_j - d_i),  F(X)_jj = 1,
 * with a per-column step length sigma from the differences of F(X), F(F(X))
 * (and F^3(X)), until ||F(X) - X||_F / ||X||_F < min(tol, 1e-12).  The
 * product HX runs on this library's split-K FP64 kernels (no cuBLAS call);
 * the cuBLAS handle only names the stream (NULL: the legacy default stream).
 * Result vectors (F(X) of the last step, not normalised) and values
 * (diag(H F(X))) are device buffers freed by acx_cuda_free_result.
 */
#ifndef IPT_GB300_ACX_CUDA_H
#define IPT_GB300_ACX_CUDA_H

#include "ipt_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ACX_CUDA_SUCCESS 0
#define ACX_CUDA_INVALID_ARGUMENT 1
#define ACX_CUDA_ALLOCATION_FAILED 2
#define ACX_CUDA_CUDA_ERROR 3
#define ACX_CUDA_CUBLAS_ERROR 4
#define ACX_CUDA_ZERO_DENOMINATOR 5

typedef struct {
    int n;
    int k;
    int iterations;
    int f_calls;
    int converged;
    double time_sec;
    double iteration_time_sec;
    double finalization_time_sec;
    double max_residual;          /* max_j ||(HX)_j - X_j (HX)_jj|| at the last step's X */
    double fixed_point_residual;  /* ||F(X) - X||_F / ||X||_F at the last step */
    double *d_vectors;
    double *d_values;
} ACXCudaResult;

/* Mixed ACX (replaces IPT_C_GPU/src/ACX/acx_mixed_precision_cuda.cu:19-48,
 * 811-905): the extrapolation first on the map with Delta and the diagonal in
 * FP32 until ||F(X) - X|| / ||X|| <= tf32_tol (or tf32_maxiter steps), then
 * the FP64 extrapolation from that block to min(fp64_tol, 1e-12).  The FP32
 * stage multiplies with this library's FP32 split-K kernel where the
 * reference uses a TF32 GEMM (no operand rounded to 10 bits).  The vectors
 * are the FP64 stage's F(X) when it converged, else its last extrapolated X.
 * A NULL handle is an invalid argument, as in the reference. */
typedef struct {
    int n;
    int k;
    int tf32_iterations;
    int fp64_iterations;
    int tf32_f_calls;
    int fp64_f_calls;
    int tf32_converged;
    int fp64_converged;
    double tf32_time_sec;
    double fp64_time_sec;
    double total_time_sec;
    double finalization_time_sec;
    double tf32_fixed_point_residual;
    double fp64_fixed_point_residual;
    double fp64_max_residual;
    double *d_vectors;
    double *d_values;
} ACXMixedTF32CudaResult;

/* Rayleigh ACX result (IPT_C_GPU/src/ACX/acx_rayleigh_mixed_precision_cuda.cu:19-42). */
typedef struct {
    int n;
    int k;
    int tf32_iterations;
    int fp64_iterations;
    int tf32_f_calls;
    int fp64_f_calls;
    int tf32_converged;
    int fp64_converged;
    double tf32_time_sec;
    double orthogonalize_time_sec;
    double rayleigh_transform_time_sec;
    double fp64_time_sec;
    double finalization_time_sec;
    double backtransform_time_sec;
    double total_time_sec;
    double tf32_fixed_point_residual;
    double fp64_fixed_point_residual;
    double fp64_max_residual;
    double *d_vectors;
    double *d_values;
} ACXRayleighMixedTF32CudaResult;

/* IPT_C_GPU/src/ACX/acx_rayleigh_mixed_precision_cuda.cu:44-51 (driver
 * :289-434): ACX of the low-precision map to tf32_tol (the FP32 stage of
 * acx_mixed_precision_tf32_cuda_device_tol), an orthonormal basis Q of that
 * block with the column signs of a Householder QR, B = sym(Q^T H Q), FP64 ACX
 * on the k x k matrix B to fp64_tol, and the vectors Q Z.  k <= 112. */
void acx_rayleigh_mixed_tf32_cuda_reset_result(ACXRayleighMixedTF32CudaResult *result);
void acx_rayleigh_mixed_tf32_cuda_free_result(ACXRayleighMixedTF32CudaResult *result);
int acx_rayleigh_mixed_tf32_cuda_device_tol(const double *d_matrix_col_major, int n, int k,
                                            double tf32_tol, int tf32_maxiter, double fp64_tol,
                                            int fp64_maxiter, cublasHandle_t handle,
                                            ACXRayleighMixedTF32CudaResult *result);

void acx_mixed_precision_tf32_cuda_reset_result(ACXMixedTF32CudaResult *result);
void acx_mixed_precision_tf32_cuda_free_result(ACXMixedTF32CudaResult *result);
int acx_mixed_precision_tf32_cuda_device_tol(const double *d_matrix_col_major, int n, int k,
                                             double tf32_tol, int tf32_maxiter, double fp64_tol,
                                             int fp64_maxiter, cublasHandle_t handle,
                                             ACXMixedTF32CudaResult *result);

const char *acx_cuda_status_string(int status);
void acx_cuda_reset_result(ACXCudaResult *result);
void acx_cuda_free_result(ACXCudaResult *result);
int acx_cuda_device_tol(const double *d_matrix_col_major, int n, int k, double tol, int maxiter,
                        cublasHandle_t handle, ACXCudaResult *result);

#ifdef __cplusplus
}
#endif

#endif
