// kernels.cuh - launchers of the library's CUDA kernels (internal).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace iptgb {

// Scratch for the deterministic grid-wide norm reductions.
struct NormScratch {
    double2 *partials = nullptr;  // one slot per block of the reducing grid
    int capacity = 0;             // number of slots
    unsigned int *counter = nullptr;  // ticket counter, zero between launches
    double *norms = nullptr;      // [0] = ||delta||_F, [1] = ||X||_F
    // Optional per-step history with a device-side stop (tensor-core
    // operator): step t adds its (||delta||^2, ||X||^2) into hist[2t..2t+1]
    // with atomics; once a step meets ||delta|| <= stop_tol ||X||, the later
    // steps' kernels pass the block through unchanged (and copy the
    // history entry forward), so the host reads the history only now and then.
    double *hist = nullptr;
    int hist_cap = 0;    // steps the history holds
    int step = 0;        // index of the next step
    double stop_tol = 0.0;
};

// Did the history entry before `step` meet the stop tolerance?
__device__ __forceinline__ bool hist_stopped(const double *hist, int step, double tol)
{
    if (hist == nullptr || step <= 0) return false;
    const double d2 = __ldcg(hist + 2 * (step - 1));
    const double x2 = __ldcg(hist + 2 * (step - 1) + 1);
    return x2 > 0.0 && d2 <= tol * tol * x2;  // NaN never stops
}

// ---- FP64 dense (k_dense64.cu) -------------------------------------------
int dense64_split_for(int n, int k, int sms);
int launch_dense64_partial(const double *H, int n, long long ldh, const double *X,
                           long long ldx, int k, double *P, int S, cudaStream_t stream);
int launch_dense32_partial(const float *H, int n, long long ldh, const float *X, long long ldx,
                           int k, float *P, int S, cudaStream_t stream);
int launch_sum_partials(const double *P, int S, size_t elems, double *Y, cudaStream_t stream);
// Double-FP32 (hi + lo) FP64-accurate products (k_df64.cu).
int launch_df_split(const double *A, size_t count, float *hi, float *lo, cudaStream_t stream);
// Y = H X for CSR H with double-float values (vh, vl) (k_csr64.cu)
int launch_csr_df_spmm(const int *row_ptr, const int *col_ind, const float *vh, const float *vl,
                       int n, const double *X, int k, double *Y, cudaStream_t stream);
// K slices of the double-FP32 product for an n x k block
int df64_split_for(int n, int k, int sms);
// Y = the sum of launch_df64_partial's S slices (which hold double-float
// pairs in the FP64 partial buffer P)
int launch_df_sum_partials(const double *P, int S, size_t elems, double *Y, cudaStream_t stream);
int launch_df64_partial(const float *Hh, const float *Hl, int n, long long ldh, const float *Xh,
                        const float *Xl, long long ldx, int k, double *P, int S,
                        cudaStream_t stream);
int launch_dense64_update(const double *P, int S, int n, int k, const double *X,
                          const double *d, double *Xn, int want_norms, NormScratch *ns,
                          cudaStream_t stream);
int launch_set_identity(double *x, int n, int k, cudaStream_t stream);
int launch_extract_diagonal(const double *H, long long ldh, int n, double *d,
                            cudaStream_t stream);
int launch_dense64_diag_values(const double *H, long long ldh, int n, const double *X, int k,
                               double *values, cudaStream_t stream);

// ---- FP64 CSR (k_csr64.cu) ------------------------------------------------
// Y = H X with H in CSR (rows sorted, 0-based), X/Y column-major n-by-k.
int launch_csr64_spmm(const int *row_ptr, const int *col_ind, const double *vals, int n,
                      const double *X, int k, double *Y, cudaStream_t stream);
// IPT update from a full Y = H X block (Y may alias nothing); same map as
// launch_dense64_update with S = 1 partial.
int launch_ipt_update_from_y(const double *Y, int n, int k, const double *X, const double *d,
                             double *Xn, int want_norms, NormScratch *ns, cudaStream_t stream);
int launch_csr64_diagonal(const int *row_ptr, const int *col_ind, const double *vals, int n,
                          double *d, cudaStream_t stream);
int launch_csr64_diag_values(const int *row_ptr, const int *col_ind, const double *vals,
                             int n, const double *X, int k, double *values,
                             cudaStream_t stream);

}  // namespace iptgb
