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

const char *acx_cuda_status_string(int status);
void acx_cuda_reset_result(ACXCudaResult *result);
void acx_cuda_free_result(ACXCudaResult *result);
int acx_cuda_device_tol(const double *d_matrix_col_major, int n, int k, double tol, int maxiter,
                        cublasHandle_t handle, ACXCudaResult *result);

#ifdef __cplusplus
}
#endif

#endif
