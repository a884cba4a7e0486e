// abi.cu - the reference-compatible C ABI (include/ipt_cuda.h).
//
// Each entry point keeps the reference's validation order, status codes,
// output ownership and error behaviour; the work behind it is the GB300
// kernels of this library.
#include <cublas_v2.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <climits>
#include <vector>

#include "common.cuh"
#include "ipt_plain.h"
#include "prep.h"

using namespace iptgb;

#define IPT_API extern "C" __attribute__((visibility("default")))

namespace {

double seconds_since(const std::chrono::steady_clock::time_point &t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// The stream a cuBLAS handle is bound to (the reference runs everything on
// the handle's stream, IPT_C_GPU/src/ipt_cuda.cu:276-283).
int handle_stream(cublasHandle_t handle, cudaStream_t *stream)
{
    if (cublasGetStream(handle, stream) != CUBLAS_STATUS_SUCCESS) {
        return IPT_CUDA_CUBLAS_ERROR;
    }
    return IPT_CUDA_SUCCESS;
}

struct OwnedStream {
    cudaStream_t s = nullptr;
    ~OwnedStream()
    {
        if (s != nullptr) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
    int create()
    {
        IPTGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        return IPT_CUDA_SUCCESS;
    }
};

// Shared FP64 dense loop on device buffers.  X_out / values_out are
// caller-provided device buffers (n*k and k doubles).
int dense_plain_device(const double *dH, int n, int k, const double *dX0, int maxiter,
                       double tol, int use_tol, double *X_out, double *values_out,
                       int *iterations_done, double *fixed_point_residual, cudaStream_t stream)
{
    const size_t elems = (size_t)n * (size_t)k;
    DeviceBuffer<double> xa, xb, d, P;
    IPTGB_CHECK(xa.alloc(elems, stream));
    IPTGB_CHECK(xb.alloc(elems, stream));
    IPTGB_CHECK(d.alloc((size_t)n, stream));
    DenseFp64Operator op;
    op.H = dH;
    op.ldh = n;
    op.n = n;
    op.k = k;
    op.S = dense64_split_for(n, k, device_sm_count());
    op.stream = stream;
    IPTGB_CHECK(P.alloc((size_t)op.S * elems, stream));
    op.P = P.ptr;
    SolveScratch scratch;
    int status = scratch.init(elems, stream);
    if (status == IPT_CUDA_SUCCESS) {
        if (dX0 != nullptr) {
            status = cudaMemcpyAsync(xa.ptr, dX0, elems * sizeof(double),
                                     cudaMemcpyDeviceToDevice, stream) == cudaSuccess
                         ? IPT_CUDA_SUCCESS
                         : IPT_CUDA_CUDA_ERROR;
        } else {
            status = launch_set_identity(xa.ptr, n, k, stream);
        }
    }
    if (status == IPT_CUDA_SUCCESS) {
        status = launch_extract_diagonal(dH, n, n, d.ptr, stream);
    }
    double *xfinal = nullptr;
    if (status == IPT_CUDA_SUCCESS) {
        status = run_plain_ipt(op, n, k, d.ptr, maxiter, tol, use_tol, xa.ptr, xb.ptr, &xfinal,
                               iterations_done, fixed_point_residual, &scratch, stream);
    }
    if (status == IPT_CUDA_SUCCESS) {
        status = op.diag_values(xfinal, values_out);
    }
    if (status == IPT_CUDA_SUCCESS &&
        cudaMemcpyAsync(X_out, xfinal, elems * sizeof(double), cudaMemcpyDeviceToDevice,
                        stream) != cudaSuccess) {
        status = IPT_CUDA_CUDA_ERROR;
    }
    scratch.release(stream);
    return status;
}

// Shared FP64 CSR loop on device buffers.
int csr_plain_device(const int *row_ptr, const int *col_ind, const double *vals, const double *dd,
                     int n, int k, const double *dX0, int maxiter, double tol, int use_tol,
                     double *X_out, double *values_out, int *iterations_done,
                     double *fixed_point_residual, cudaStream_t stream)
{
    const size_t elems = (size_t)n * (size_t)k;
    DeviceBuffer<double> xa, xb, Y;
    IPTGB_CHECK(xa.alloc(elems, stream));
    IPTGB_CHECK(xb.alloc(elems, stream));
    IPTGB_CHECK(Y.alloc(elems, stream));
    CsrFp64Operator op;
    op.row_ptr = row_ptr;
    op.col_ind = col_ind;
    op.vals = vals;
    op.n = n;
    op.k = k;
    op.Y = Y.ptr;
    op.stream = stream;
    SolveScratch scratch;
    int status = scratch.init(elems, stream);
    if (status == IPT_CUDA_SUCCESS) {
        if (dX0 != nullptr) {
            status = cudaMemcpyAsync(xa.ptr, dX0, elems * sizeof(double),
                                     cudaMemcpyDeviceToDevice, stream) == cudaSuccess
                         ? IPT_CUDA_SUCCESS
                         : IPT_CUDA_CUDA_ERROR;
        } else {
            status = launch_set_identity(xa.ptr, n, k, stream);
        }
    }
    double *xfinal = nullptr;
    if (status == IPT_CUDA_SUCCESS) {
        status = run_plain_ipt(op, n, k, dd, maxiter, tol, use_tol, xa.ptr, xb.ptr, &xfinal,
                               iterations_done, fixed_point_residual, &scratch, stream);
    }
    if (status == IPT_CUDA_SUCCESS) {
        status = op.diag_values(xfinal, values_out);
    }
    if (status == IPT_CUDA_SUCCESS &&
        cudaMemcpyAsync(X_out, xfinal, elems * sizeof(double), cudaMemcpyDeviceToDevice,
                        stream) != cudaSuccess) {
        status = IPT_CUDA_CUDA_ERROR;
    }
    scratch.release(stream);
    return status;
}

void reset_result_head(IPTCudaResult *result)
{
    result->n = 0;
    result->k = 0;
    result->iterations = 0;
    result->vectors = nullptr;
    result->values = nullptr;
    result->basis_cols = 0;
    result->fixed_point_residual = NAN;
}

}  // namespace

namespace iptgb {
// FP64 dense IPT loop on device buffers (shared with the mixed entry points).
int dense_plain_device_entry(const double *dH, int n, int k, const double *dX0, int maxiter,
                             double tol, int use_tol, double *X_out, double *values_out,
                             int *iterations_done, double *fixed_point_residual,
                             cudaStream_t stream)
{
    return dense_plain_device(dH, n, k, dX0, maxiter, tol, use_tol, X_out, values_out,
                              iterations_done, fixed_point_residual, stream);
}
}  // namespace iptgb

// ---------------------------------------------------------------------------
// Utilities (IPT_C_GPU/src/ipt_cuda.cu:375-483)
// ---------------------------------------------------------------------------
IPT_API const char *ipt_cuda_status_string(int status)
{
    switch (status) {
    case IPT_CUDA_SUCCESS:
        return "success";
    case IPT_CUDA_INVALID_ARGUMENT:
        return "invalid argument";
    case IPT_CUDA_ALLOCATION_FAILED:
        return "allocation failed";
    case IPT_CUDA_CUDA_ERROR:
        return "CUDA runtime error";
    case IPT_CUDA_CUBLAS_ERROR:
        return "cuBLAS error";
    case IPT_CUDA_CUSPARSE_ERROR:
        return "cuSPARSE error";
    case IPT_CUDA_CUSOLVER_ERROR:
        return "cuSOLVER error";
    default:
        return "unknown error";
    }
}

IPT_API void ipt_cuda_free_result(IPTCudaResult *result)
{
    if (result == nullptr) {
        return;
    }
    free(result->vectors);
    free(result->values);
    free(result->davidson_history);
    free(result->davidson_selection_history);
    free(result->davidson_block_history);
    // Every field back to its "no result" value (ipt_cuda.cu:398-475).
    memset(result, 0, sizeof(*result));
    result->fixed_point_residual = NAN;
    result->basis_orthogonality_frobenius_error = NAN;
    result->basis_orthogonality_max_abs_error = NAN;
    result->ritz_vectors_orthogonality_frobenius_error = NAN;
    result->ritz_vectors_orthogonality_max_abs_error = NAN;
    result->davidson_target_index = -1;
    result->davidson_residual_before = NAN;
    result->davidson_residual_after = NAN;
    result->davidson_denom_clip = NAN;
    result->adaptive_coupling_tau = NAN;
    result->adaptive_target_block_start = -1;
    result->adaptive_target_block_end = -1;
    result->best_so_far_step = -1;
    result->best_so_far_max_residual = NAN;
    result->best_so_far_max_residual_index = -1;
    result->pair28_best_residual = NAN;
    result->pair29_best_residual = NAN;
    result->gap28_29 = NAN;
    result->relative_gap28_29 = NAN;
    result->cluster_residual_fro = NAN;
    result->cluster_residual_max = NAN;
    strcpy(result->pair28_lock_state, "unknown");
    strcpy(result->pair29_lock_state, "unknown");
}

IPT_API void ipt_cuda_free_device_result(double *d_vectors, double *d_values)
{
    cudaFree(d_vectors);
    cudaFree(d_values);
}

// ---------------------------------------------------------------------------
// Dense, device buffers (IPT_C_GPU/src/ipt_cuda.cu:1562-1770)
// ---------------------------------------------------------------------------
static int ipt_dense_device_entry(const double *dH, int n, int k, int maxiter, double tol,
                                  int use_tol, cublasHandle_t handle, double **d_vectors_out,
                                  double **d_values_out, int *iterations_done_out,
                                  double *fixed_point_residual_out)
{
    if (d_vectors_out != nullptr) *d_vectors_out = nullptr;
    if (d_values_out != nullptr) *d_values_out = nullptr;
    if (iterations_done_out != nullptr) *iterations_done_out = 0;
    if (fixed_point_residual_out != nullptr) *fixed_point_residual_out = NAN;
    if (dH == nullptr || handle == nullptr || d_vectors_out == nullptr ||
        d_values_out == nullptr || n <= 0 || k <= 0 || k > n || maxiter < 0 ||
        (use_tol && (tol <= 0.0 || maxiter <= 0))) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    const size_t elems = (size_t)n * (size_t)k;
    if (elems > (size_t)INT_MAX) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t stream = nullptr;
    IPTGB_CHECK(handle_stream(handle, &stream));
    double *vec = nullptr, *val = nullptr;
    IPTGB_CUDA(cudaMalloc((void **)&vec, elems * sizeof(double)));
    if (cudaMalloc((void **)&val, (size_t)k * sizeof(double)) != cudaSuccess) {
        cudaFree(vec);
        return IPT_CUDA_CUDA_ERROR;
    }
    int iters = 0;
    double fpres = NAN;
    int status = dense_plain_device(dH, n, k, nullptr, maxiter, tol, use_tol, vec, val, &iters,
                                    &fpres, stream);
    if (status != IPT_CUDA_SUCCESS) {
        cudaStreamSynchronize(stream);
        cudaFree(vec);
        cudaFree(val);
        return status;
    }
    *d_vectors_out = vec;
    *d_values_out = val;
    if (iterations_done_out != nullptr) *iterations_done_out = iters;
    if (fixed_point_residual_out != nullptr) *fixed_point_residual_out = fpres;
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_cuda_device(const double *d_matrix_col_major, int n, int k, int iterations,
                            cublasHandle_t handle, double **d_vectors_out, double **d_values_out)
{
    return ipt_dense_device_entry(d_matrix_col_major, n, k, iterations, 0.0, 0, handle,
                                  d_vectors_out, d_values_out, nullptr, nullptr);
}

IPT_API int ipt_cuda_device_tol(const double *d_matrix_col_major, int n, int k, double tol,
                                int maxiter, cublasHandle_t handle, double **d_vectors_out,
                                double **d_values_out, int *iterations_done_out,
                                double *fixed_point_residual_out)
{
    return ipt_dense_device_entry(d_matrix_col_major, n, k, maxiter, tol, 1, handle,
                                  d_vectors_out, d_values_out, iterations_done_out,
                                  fixed_point_residual_out);
}

// ---------------------------------------------------------------------------
// Dense, host buffers (IPT_C_GPU/src/ipt_cuda.cu:1779-1991)
// ---------------------------------------------------------------------------
static int ipt_dense_host_entry(const double *H, const double *X0, int n, int k, int maxiter,
                                double tol, int use_tol, IPTCudaResult *result)
{
    if (result != nullptr) {
        reset_result_head(result);
    }
    if (H == nullptr || result == nullptr || n <= 0 || k <= 0 || k > n || maxiter < 0 ||
        (use_tol && (tol <= 0.0 || maxiter <= 0))) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    const size_t mat = (size_t)n * (size_t)n;
    const size_t elems = (size_t)n * (size_t)k;
    if (mat > (size_t)INT_MAX || elems > (size_t)INT_MAX) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    auto t0 = std::chrono::steady_clock::now();
    result->vectors = (double *)calloc(elems, sizeof(double));
    result->values = (double *)calloc((size_t)k, sizeof(double));
    if (result->vectors == nullptr || result->values == nullptr) {
        ipt_cuda_free_result(result);
        return IPT_CUDA_ALLOCATION_FAILED;
    }
    int status = IPT_CUDA_SUCCESS;
    {
        OwnedStream os;
        status = os.create();
        DeviceBuffer<double> dH, dX0, dX, dv;
        if (status == IPT_CUDA_SUCCESS) status = dH.alloc(mat, os.s);
        if (status == IPT_CUDA_SUCCESS && X0 != nullptr) status = dX0.alloc(elems, os.s);
        if (status == IPT_CUDA_SUCCESS) status = dX.alloc(elems, os.s);
        if (status == IPT_CUDA_SUCCESS) status = dv.alloc((size_t)k, os.s);
        if (status == IPT_CUDA_SUCCESS &&
            cudaMemcpyAsync(dH.ptr, H, mat * sizeof(double), cudaMemcpyHostToDevice, os.s) !=
                cudaSuccess) {
            status = IPT_CUDA_CUDA_ERROR;
        }
        if (status == IPT_CUDA_SUCCESS && X0 != nullptr &&
            cudaMemcpyAsync(dX0.ptr, X0, elems * sizeof(double), cudaMemcpyHostToDevice,
                            os.s) != cudaSuccess) {
            status = IPT_CUDA_CUDA_ERROR;
        }
        int iters = 0;
        double fpres = NAN;
        const double transfer = seconds_since(t0);
        auto t1 = std::chrono::steady_clock::now();
        if (status == IPT_CUDA_SUCCESS) {
            status = dense_plain_device(dH.ptr, n, k, dX0.ptr, maxiter, tol, use_tol, dX.ptr,
                                        dv.ptr, &iters, &fpres, os.s);
        }
        if (status == IPT_CUDA_SUCCESS &&
            (cudaMemcpyAsync(result->vectors, dX.ptr, elems * sizeof(double),
                             cudaMemcpyDeviceToHost, os.s) != cudaSuccess ||
             cudaMemcpyAsync(result->values, dv.ptr, (size_t)k * sizeof(double),
                             cudaMemcpyDeviceToHost, os.s) != cudaSuccess ||
             cudaStreamSynchronize(os.s) != cudaSuccess)) {
            status = IPT_CUDA_CUDA_ERROR;
        }
        if (status == IPT_CUDA_SUCCESS) {
            result->n = n;
            result->k = k;
            result->iterations = iters;
            result->basis_cols = k;
            result->fixed_point_residual = fpres;
            result->matvecs = (long long)(iters + 1) * (long long)k;
            result->transfer_setup_time_sec = transfer;
            result->iteration_time_sec = seconds_since(t1);
            result->solve_time_sec = result->iteration_time_sec;
        }
    }
    if (status != IPT_CUDA_SUCCESS) {
        ipt_cuda_free_result(result);
    }
    return status;
}

IPT_API int ipt_cuda_with_initial(const double *matrix_col_major,
                                  const double *initial_vectors_col_major, int n, int k,
                                  int iterations, IPTCudaResult *result)
{
    return ipt_dense_host_entry(matrix_col_major, initial_vectors_col_major, n, k, iterations,
                                0.0, 0, result);
}

IPT_API int ipt_cuda_with_initial_tol(const double *matrix_col_major,
                                      const double *initial_vectors_col_major, int n, int k,
                                      double tol, int maxiter, IPTCudaResult *result)
{
    return ipt_dense_host_entry(matrix_col_major, initial_vectors_col_major, n, k, maxiter, tol,
                                1, result);
}

IPT_API int ipt_cuda(const double *matrix_col_major, int n, int k, int iterations,
                     IPTCudaResult *result)
{
    return ipt_cuda_with_initial(matrix_col_major, nullptr, n, k, iterations, result);
}

IPT_API int ipt_cuda_tol(const double *matrix_col_major, int n, int k, double tol, int maxiter,
                         IPTCudaResult *result)
{
    return ipt_cuda_with_initial_tol(matrix_col_major, nullptr, n, k, tol, maxiter, result);
}

// ---------------------------------------------------------------------------
// Sparse CSC, device buffers (IPT_C_GPU/src/ipt_cuda.cu:1994-2232).  The
// reference feeds the CSC arrays to cuSPARSE as CSR with OP_T, i.e. it
// multiplies by the CSC matrix without sorting.  Here the arrays are read
// back once, transposed to CSR on the host, and the CSR gather kernel runs
// on the handle's stream; the diagonal is the first stored entry of each
// column, as extract_csc_diagonal_kernel (ipt_cuda.cu:1469-1489).
// ---------------------------------------------------------------------------
static int ipt_sparse_device_entry(const int *d_col_ptr, const int *d_row_ind,
                                   const double *d_vals, int n, int k, int nnz, int maxiter,
                                   double tol, int use_tol, cublasHandle_t handle,
                                   double **d_vectors_out, double **d_values_out,
                                   int *iterations_done_out, double *fixed_point_residual_out)
{
    if (d_vectors_out != nullptr) *d_vectors_out = nullptr;
    if (d_values_out != nullptr) *d_values_out = nullptr;
    if (iterations_done_out != nullptr) *iterations_done_out = 0;
    if (fixed_point_residual_out != nullptr) *fixed_point_residual_out = NAN;
    if (d_col_ptr == nullptr || d_row_ind == nullptr || d_vals == nullptr || handle == nullptr ||
        d_vectors_out == nullptr || d_values_out == nullptr || n <= 0 || k <= 0 || k > n ||
        nnz < 0 || maxiter < 0 || (use_tol && (tol <= 0.0 || maxiter <= 0))) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    const size_t elems = (size_t)n * (size_t)k;
    if (elems > (size_t)INT_MAX) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t stream = nullptr;
    IPTGB_CHECK(handle_stream(handle, &stream));
    std::vector<int> cp((size_t)n + 1U), ri((size_t)nnz);
    std::vector<double> va((size_t)nnz);
    IPTGB_CUDA(cudaMemcpyAsync(cp.data(), d_col_ptr, cp.size() * sizeof(int),
                               cudaMemcpyDeviceToHost, stream));
    if (nnz > 0) {
        IPTGB_CUDA(cudaMemcpyAsync(ri.data(), d_row_ind, ri.size() * sizeof(int),
                                   cudaMemcpyDeviceToHost, stream));
        IPTGB_CUDA(cudaMemcpyAsync(va.data(), d_vals, va.size() * sizeof(double),
                                   cudaMemcpyDeviceToHost, stream));
    }
    IPTGB_CUDA(cudaStreamSynchronize(stream));
    if (!validate_csc(cp.data(), ri.data(), n, nnz)) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    std::vector<double> diag;
    csc_diagonal(cp.data(), ri.data(), va.data(), n, &diag);
    std::vector<int> rp, ci;
    std::vector<double> cv;
    csc_to_csr(cp.data(), ri.data(), va.data(), n, nnz, &rp, &ci, &cv);

    DeviceBuffer<int> drp, dci;
    DeviceBuffer<double> dcv, dd;
    IPTGB_CHECK(drp.alloc(rp.size(), stream));
    IPTGB_CHECK(dci.alloc(ci.size(), stream));
    IPTGB_CHECK(dcv.alloc(cv.size(), stream));
    IPTGB_CHECK(dd.alloc((size_t)n, stream));
    IPTGB_CUDA(cudaMemcpyAsync(drp.ptr, rp.data(), rp.size() * sizeof(int),
                               cudaMemcpyHostToDevice, stream));
    if (nnz > 0) {
        IPTGB_CUDA(cudaMemcpyAsync(dci.ptr, ci.data(), ci.size() * sizeof(int),
                                   cudaMemcpyHostToDevice, stream));
        IPTGB_CUDA(cudaMemcpyAsync(dcv.ptr, cv.data(), cv.size() * sizeof(double),
                                   cudaMemcpyHostToDevice, stream));
    }
    IPTGB_CUDA(cudaMemcpyAsync(dd.ptr, diag.data(), (size_t)n * sizeof(double),
                               cudaMemcpyHostToDevice, stream));
    double *vec = nullptr, *val = nullptr;
    IPTGB_CUDA(cudaMalloc((void **)&vec, elems * sizeof(double)));
    if (cudaMalloc((void **)&val, (size_t)k * sizeof(double)) != cudaSuccess) {
        cudaFree(vec);
        return IPT_CUDA_CUDA_ERROR;
    }
    int iters = 0;
    double fpres = NAN;
    int status = csr_plain_device(drp.ptr, dci.ptr, dcv.ptr, dd.ptr, n, k, nullptr, maxiter, tol,
                                  use_tol, vec, val, &iters, &fpres, stream);
    // host vectors above must outlive the async copies
    cudaStreamSynchronize(stream);
    if (status != IPT_CUDA_SUCCESS) {
        cudaFree(vec);
        cudaFree(val);
        return status;
    }
    *d_vectors_out = vec;
    *d_values_out = val;
    if (iterations_done_out != nullptr) *iterations_done_out = iters;
    if (fixed_point_residual_out != nullptr) *fixed_point_residual_out = fpres;
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_cuda_sparse_csc_device(const int *d_col_ptr, const int *d_row_ind,
                                       const double *d_matrix_values, int n, int k, int nnz,
                                       int iterations, cublasHandle_t handle,
                                       double **d_vectors_out, double **d_values_out)
{
    return ipt_sparse_device_entry(d_col_ptr, d_row_ind, d_matrix_values, n, k, nnz, iterations,
                                   0.0, 0, handle, d_vectors_out, d_values_out, nullptr,
                                   nullptr);
}

IPT_API int ipt_cuda_sparse_csc_device_tol(const int *d_col_ptr, const int *d_row_ind,
                                           const double *d_matrix_values, int n, int k, int nnz,
                                           double tol, int maxiter, cublasHandle_t handle,
                                           double **d_vectors_out, double **d_values_out,
                                           int *iterations_done_out,
                                           double *fixed_point_residual_out)
{
    return ipt_sparse_device_entry(d_col_ptr, d_row_ind, d_matrix_values, n, k, nnz, maxiter,
                                   tol, 1, handle, d_vectors_out, d_values_out,
                                   iterations_done_out, fixed_point_residual_out);
}

// ---------------------------------------------------------------------------
// Sparse CSC, host buffers (IPT_C_GPU/src/ipt_cuda.cu:5018-5316, plain path):
// host preparation (validate, stable diagonal sort, permutation), the CSR
// IPT loop on the device, then the output rows are scattered back to the
// original order.
// ---------------------------------------------------------------------------
int ipt_block_sparse_host_entry(const int *col_ptr, const int *row_ind, const double *vals,
                                int n, int k, int nnz, int maxiter, double tol, int use_tol,
                                IPTCudaResult *result);

static int ipt_sparse_host_entry(const int *col_ptr, const int *row_ind, const double *vals,
                                 const double *X0, int n, int k, int nnz, int maxiter, double tol,
                                 int use_tol, IPTCudaResult *result)
{
    if (result != nullptr) {
        reset_result_head(result);
    }
    if (col_ptr == nullptr || row_ind == nullptr || vals == nullptr || result == nullptr ||
        n <= 0 || k <= 0 || k > n || nnz < 0 || maxiter < 0 ||
        (use_tol && (tol <= 0.0 || maxiter <= 0))) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    if (X0 == nullptr && env_flag("IPT_BLOCK_CLUSTER", 0)) {
        return ipt_block_sparse_host_entry(col_ptr, row_ind, vals, n, k, nnz, maxiter, tol,
                                           use_tol, result);
    }
    auto t0 = std::chrono::steady_clock::now();
    PreparedCsr prep;
    // the reference's plain sparse path lifts degeneracies (ipt_cuda.cu:5077-5090)
    int status = prepare_csc(col_ptr, row_ind, vals, n, nnz, true, &prep, k,
                             env_double("IPT_DEGENERACY_THRESHOLD", 0.0));
    if (status != IPT_CUDA_SUCCESS) {
        ipt_cuda_free_result(result);
        return status;
    }
    const size_t elems = (size_t)n * (size_t)k;
    if (elems > (size_t)INT_MAX) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    result->vectors = (double *)calloc(elems, sizeof(double));
    result->values = (double *)calloc((size_t)k, sizeof(double));
    if (result->vectors == nullptr || result->values == nullptr) {
        ipt_cuda_free_result(result);
        return IPT_CUDA_ALLOCATION_FAILED;
    }
    const double prep_time = seconds_since(t0);
    {
        OwnedStream os;
        status = os.create();
        DeviceBuffer<int> drp, dci;
        DeviceBuffer<double> dcv, dd, dX0, dX, dv;
        if (status == IPT_CUDA_SUCCESS) status = drp.alloc(prep.row_ptr.size(), os.s);
        if (status == IPT_CUDA_SUCCESS) status = dci.alloc(prep.col_ind.size(), os.s);
        if (status == IPT_CUDA_SUCCESS) status = dcv.alloc(prep.vals.size(), os.s);
        if (status == IPT_CUDA_SUCCESS) status = dd.alloc((size_t)n, os.s);
        if (status == IPT_CUDA_SUCCESS && X0 != nullptr) status = dX0.alloc(elems, os.s);
        if (status == IPT_CUDA_SUCCESS) status = dX.alloc(elems, os.s);
        if (status == IPT_CUDA_SUCCESS) status = dv.alloc((size_t)k, os.s);
        auto cpy = [&](void *dst, const void *src, size_t bytes) {
            if (status == IPT_CUDA_SUCCESS && bytes > 0 &&
                cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, os.s) != cudaSuccess) {
                status = IPT_CUDA_CUDA_ERROR;
            }
        };
        cpy(drp.ptr, prep.row_ptr.data(), prep.row_ptr.size() * sizeof(int));
        cpy(dci.ptr, prep.col_ind.data(), prep.col_ind.size() * sizeof(int));
        cpy(dcv.ptr, prep.vals.data(), prep.vals.size() * sizeof(double));
        cpy(dd.ptr, prep.diag.data(), (size_t)n * sizeof(double));
        if (X0 != nullptr) {
            // The initial block is taken as given, in the prepared basis
            // (the reference copies it unchanged, ipt_cuda.cu:5133-5139).
            cpy(dX0.ptr, X0, elems * sizeof(double));
        }
        const double transfer = seconds_since(t0) - prep_time;
        auto t1 = std::chrono::steady_clock::now();
        int iters = 0;
        double fpres = NAN;
        if (status == IPT_CUDA_SUCCESS) {
            status = csr_plain_device(drp.ptr, dci.ptr, dcv.ptr, dd.ptr, n, k, dX0.ptr, maxiter,
                                      tol, use_tol, dX.ptr, dv.ptr, &iters, &fpres, os.s);
        }
        if (status == IPT_CUDA_SUCCESS &&
            (cudaMemcpyAsync(result->vectors, dX.ptr, elems * sizeof(double),
                             cudaMemcpyDeviceToHost, os.s) != cudaSuccess ||
             cudaMemcpyAsync(result->values, dv.ptr, (size_t)k * sizeof(double),
                             cudaMemcpyDeviceToHost, os.s) != cudaSuccess ||
             cudaStreamSynchronize(os.s) != cudaSuccess)) {
            status = IPT_CUDA_CUDA_ERROR;
        }
        if (status == IPT_CUDA_SUCCESS) {
            unpermute_vectors(prep, result->vectors, k);
            result->n = n;
            result->k = k;
            result->iterations = iters;
            result->basis_cols = k;
            result->fixed_point_residual = fpres;
            result->matvecs = (long long)(iters + 1) * (long long)k;
            result->preparation_time_sec = prep_time;
            result->transfer_setup_time_sec = transfer;
            result->iteration_time_sec = seconds_since(t1);
            result->solve_time_sec = result->iteration_time_sec;
        }
    }
    if (status != IPT_CUDA_SUCCESS) {
        ipt_cuda_free_result(result);
    }
    return status;
}

IPT_API int ipt_cuda_sparse_csc_with_initial(const int *col_ptr, const int *row_ind,
                                             const double *matrix_values,
                                             const double *initial_vectors_col_major, int n,
                                             int k, int nnz, int iterations,
                                             IPTCudaResult *result)
{
    return ipt_sparse_host_entry(col_ptr, row_ind, matrix_values, initial_vectors_col_major, n, k,
                                 nnz, iterations, 0.0, 0, result);
}

IPT_API int ipt_cuda_sparse_csc_with_initial_tol(const int *col_ptr, const int *row_ind,
                                                 const double *matrix_values,
                                                 const double *initial_vectors_col_major, int n,
                                                 int k, int nnz, double tol, int maxiter,
                                                 IPTCudaResult *result)
{
    return ipt_sparse_host_entry(col_ptr, row_ind, matrix_values, initial_vectors_col_major, n, k,
                                 nnz, maxiter, tol, 1, result);
}

IPT_API int ipt_cuda_sparse_csc(const int *col_ptr, const int *row_ind,
                                const double *matrix_values, int n, int k, int nnz,
                                int iterations, IPTCudaResult *result)
{
    return ipt_cuda_sparse_csc_with_initial(col_ptr, row_ind, matrix_values, nullptr, n, k, nnz,
                                            iterations, result);
}

IPT_API int ipt_cuda_sparse_csc_tol(const int *col_ptr, const int *row_ind,
                                    const double *matrix_values, int n, int k, int nnz,
                                    double tol, int maxiter, IPTCudaResult *result)
{
    return ipt_cuda_sparse_csc_with_initial_tol(col_ptr, row_ind, matrix_values, nullptr, n, k,
                                                nnz, tol, maxiter, result);
}
