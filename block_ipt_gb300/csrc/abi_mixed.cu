// abi_mixed.cu - the reference's mixed-precision entry points
// (IPT_C_GPU/src/mixed_precision/ipt_mixed_precision_cuda.cu:61-78,1005-1225).
//
// Stage 1 iterates the IPT map with a low-precision block product until the
// fixed-point residual reaches the low-precision tolerance: FP16 and TF32 on
// the tensor cores (tcgen05), FP32 on the SIMT FP32 pipe.  Stage 2 refines the
// converted block with the FP64 IPT loop to the FP64 tolerance and returns
// (H X)_jj as the values.  Residual-check time is excluded from the stage-1
// time, as in the reference (:1186-1190).
#include <cublas_v2.h>
#include <math.h>

#include <climits>
#include <memory>

#include "common.cuh"
#include "ipt_plain.h"
#include "lowp.h"

#define IPT_API extern "C" __attribute__((visibility("default")))

using namespace iptgb;

namespace iptgb {
int dense_plain_device_entry(const double *dH, int n, int k, const double *dX0, int maxiter,
                             double tol, int use_tol, double *X_out, double *values_out,
                             int *iterations_done, double *fixed_point_residual,
                             cudaStream_t stream);
}

namespace {

template <typename R>
void reset_mixed(R *r)
{
    if (r == nullptr) return;
    r->n = 0;
    r->k = 0;
    r->d_vectors = nullptr;
    r->d_values = nullptr;
}

struct MixedOut {
    int lowp_iterations = 0;
    int fp64_iterations = 0;
    double lowp_time = NAN;
    double fp64_time = NAN;
    double total_time = NAN;
    double lowp_fpres = NAN;
    double fp64_fpres = NAN;
    double *vec = nullptr;
    double *val = nullptr;
};

float event_ms(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

int mixed_run(const double *dH, int n, int k, int kind, double lp_tol, int lp_maxiter,
              double fp64_tol, int fp64_maxiter, cublasHandle_t handle, MixedOut *out)
{
    if (dH == nullptr || handle == nullptr || n <= 0 || k <= 0 || k > n || !(lp_tol > 0.0) ||
        !(fp64_tol > 0.0) || lp_maxiter <= 0 || fp64_maxiter <= 0) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    if ((size_t)n * (size_t)k > (size_t)INT_MAX) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = nullptr;
    if (cublasGetStream(handle, &s) != CUBLAS_STATUS_SUCCESS) {
        return IPT_CUDA_CUBLAS_ERROR;
    }
    cudaEvent_t ev[4] = {};
    for (auto &e : ev) {
        IPTGB_CUDA(cudaEventCreate(&e));
    }
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard()
        {
            for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]);
        }
    } guard{ev};
    const size_t elems = (size_t)n * k;
    DeviceBuffer<double> d, X0;
    IPTGB_CHECK(d.alloc((size_t)n, s));
    IPTGB_CHECK(X0.alloc(elems, s));
    IPTGB_CUDA(cudaEventRecord(ev[0], s));
    IPTGB_CHECK(launch_extract_diagonal(dH, n, n, d.ptr, s));
    int st = IPT_CUDA_SUCCESS;
    std::unique_ptr<LowpDenseOperator> op(make_lowp_dense_operator(dH, n, kind, s, &st));
    if (!op) {
        return st != IPT_CUDA_SUCCESS ? st : IPT_CUDA_CUDA_ERROR;
    }
    IPTGB_CHECK(op->set_width(k));
    IPTGB_CHECK(op->reset_identity(d.ptr));
    long long mv = 0;
    IPTGB_CHECK(run_lowp_ipt(*op, n, k, lp_maxiter, lp_tol, 1, X0.ptr, &out->lowp_iterations,
                             &out->lowp_fpres, &mv, s, false));
    IPTGB_CUDA(cudaEventRecord(ev[1], s));
    op.reset();
    double *vec = nullptr, *val = nullptr;
    IPTGB_CUDA(cudaMalloc((void **)&vec, elems * sizeof(double)));
    if (cudaMalloc((void **)&val, (size_t)k * sizeof(double)) != cudaSuccess) {
        cudaFree(vec);
        return IPT_CUDA_CUDA_ERROR;
    }
    IPTGB_CUDA(cudaEventRecord(ev[2], s));
    st = dense_plain_device_entry(dH, n, k, X0.ptr, fp64_maxiter, fp64_tol, 1, vec, val,
                                  &out->fp64_iterations, &out->fp64_fpres, s);
    cudaEventRecord(ev[3], s);
    cudaStreamSynchronize(s);
    if (st != IPT_CUDA_SUCCESS) {
        cudaFree(vec);
        cudaFree(val);
        return st;
    }
    out->lowp_time = 1e-3 * event_ms(ev[0], ev[1]);
    out->fp64_time = 1e-3 * event_ms(ev[2], ev[3]);
    out->total_time = out->lowp_time + out->fp64_time;
    out->vec = vec;
    out->val = val;
    return IPT_CUDA_SUCCESS;
}

template <typename R>
void store(R *r, int n, int k, const MixedOut &o, int *lp_it, double *lp_time, double *lp_fp)
{
    r->n = n;
    r->k = k;
    *lp_it = o.lowp_iterations;
    r->fp64_iterations = o.fp64_iterations;
    *lp_time = o.lowp_time;
    r->fp64_time_sec = o.fp64_time;
    r->total_time_sec = o.total_time;
    *lp_fp = o.lowp_fpres;
    r->fp64_fixed_point_residual = o.fp64_fpres;
    r->d_vectors = o.vec;
    r->d_values = o.val;
}

}  // namespace

IPT_API void ipt_mixed_precision_cuda_free_device_result(IPTMixedCudaDeviceResult *result)
{
    if (result == nullptr) return;
    cudaFree(result->d_vectors);
    cudaFree(result->d_values);
    reset_mixed(result);
    result->fp16_iterations = 0;
    result->fp64_iterations = 0;
    result->fp16_time_sec = NAN;
    result->fp64_time_sec = NAN;
    result->total_time_sec = NAN;
    result->fp16_fixed_point_residual = NAN;
    result->fp64_fixed_point_residual = NAN;
}

IPT_API void ipt_mixed_precision_fp32_cuda_free_device_result(IPTMixedFP32CudaDeviceResult *result)
{
    if (result == nullptr) return;
    cudaFree(result->d_vectors);
    cudaFree(result->d_values);
    reset_mixed(result);
    result->fp32_iterations = 0;
    result->fp64_iterations = 0;
    result->fp32_time_sec = NAN;
    result->fp64_time_sec = NAN;
    result->total_time_sec = NAN;
    result->fp32_fixed_point_residual = NAN;
    result->fp64_fixed_point_residual = NAN;
}

IPT_API void ipt_mixed_precision_tf32_cuda_free_device_result(IPTMixedTF32CudaDeviceResult *result)
{
    if (result == nullptr) return;
    cudaFree(result->d_vectors);
    cudaFree(result->d_values);
    reset_mixed(result);
    result->tf32_iterations = 0;
    result->fp64_iterations = 0;
    result->tf32_time_sec = NAN;
    result->fp64_time_sec = NAN;
    result->total_time_sec = NAN;
    result->tf32_fixed_point_residual = NAN;
    result->fp64_fixed_point_residual = NAN;
}

IPT_API int ipt_mixed_precision_cuda_device_tol(const double *d_matrix_col_major, int n, int k,
                                                double fp16_tol, int fp16_maxiter,
                                                double fp64_tol, int fp64_maxiter,
                                                cublasHandle_t handle,
                                                IPTMixedCudaDeviceResult *result)
{
    if (result == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    result->d_vectors = nullptr;
    result->d_values = nullptr;
    ipt_mixed_precision_cuda_free_device_result(result);
    MixedOut o;
    const int st = mixed_run(d_matrix_col_major, n, k, kLowpF16, fp16_tol, fp16_maxiter, fp64_tol,
                             fp64_maxiter, handle, &o);
    if (st != IPT_CUDA_SUCCESS) return st;
    store(result, n, k, o, &result->fp16_iterations, &result->fp16_time_sec,
          &result->fp16_fixed_point_residual);
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_mixed_precision_fp32_cuda_device_tol(const double *d_matrix_col_major, int n,
                                                     int k, double fp32_tol, int fp32_maxiter,
                                                     double fp64_tol, int fp64_maxiter,
                                                     cublasHandle_t handle,
                                                     IPTMixedFP32CudaDeviceResult *result)
{
    if (result == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    result->d_vectors = nullptr;
    result->d_values = nullptr;
    ipt_mixed_precision_fp32_cuda_free_device_result(result);
    MixedOut o;
    const int st = mixed_run(d_matrix_col_major, n, k, kLowpF32, fp32_tol, fp32_maxiter, fp64_tol,
                             fp64_maxiter, handle, &o);
    if (st != IPT_CUDA_SUCCESS) return st;
    store(result, n, k, o, &result->fp32_iterations, &result->fp32_time_sec,
          &result->fp32_fixed_point_residual);
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_mixed_precision_tf32_cuda_device_tol(const double *d_matrix_col_major, int n,
                                                     int k, double tf32_tol, int tf32_maxiter,
                                                     double fp64_tol, int fp64_maxiter,
                                                     cublasHandle_t handle,
                                                     IPTMixedTF32CudaDeviceResult *result)
{
    if (result == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    result->d_vectors = nullptr;
    result->d_values = nullptr;
    ipt_mixed_precision_tf32_cuda_free_device_result(result);
    MixedOut o;
    const int st = mixed_run(d_matrix_col_major, n, k, kLowpTF32, tf32_tol, tf32_maxiter, fp64_tol,
                             fp64_maxiter, handle, &o);
    if (st != IPT_CUDA_SUCCESS) return st;
    store(result, n, k, o, &result->tf32_iterations, &result->tf32_time_sec,
          &result->tf32_fixed_point_residual);
    return IPT_CUDA_SUCCESS;
}
