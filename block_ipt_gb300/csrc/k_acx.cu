// k_acx.cu - ACX extrapolation over the dense FP64 IPT map.
//
// The reference (IPT_C_GPU/src/ACX/acx_cuda.cu:390-620) accelerates the IPT
// fixed point X <- F(X) with alternating order-2 / order-3 cyclic
// extrapolation (a SQUAREM-like scheme): with d1 = F(X) - X,
// d2 = F^2(X) - 2F(X) + X, d3 = F^3(X) - 3F^2(X) + 3F(X) - X and per column
//     order 2: s = |<d2, d1> / <d2, d2>|,  X += 2 s d1 + s^2 d2
//     order 3: s = |<d3, d2> / <d3, d3>|,  X += 3 s d1 + 3 s^2 d2 + s^3 d3,
// stopping once ||F(X) - X||_F / ||X||_F < min(tol, 1e-12).  It forms HX
// with cublasDgemm and reads a flag, k residuals and two cuBLAS norms back
// per map evaluation.
//
// Here HX is the split-K FP64 product of the plain path (k_dense64.cu); F is
// one CTA per column that reads (HX)_cc, evaluates the column's residual
// norm and the map in one pass, in place; the two Frobenius norms are one
// deterministic grid reduction; an extrapolation step is one CTA per column
// (the two inner products, then the update).  The host reads k + 3 values
// per step.  The map's denominator test only depends on the diagonal, so the
// first evaluation decides it for the whole run.
#include <cublas_v2.h>
#include <float.h>
#include <math.h>
#include <string.h>

#include <chrono>
#include <vector>

#include "../../include/acx_cuda.h"
#include "common.cuh"
#include "ipt_plain.h"
#include "kernels.cuh"
#include "reduce.cuh"

namespace iptgb {

constexpr int kAcxThreads = 256;
constexpr int kAcxNormBlocks = 256;

// Y = F(X) in place on Y = H X, one CTA per column c:
//   m = Y[c,c], u = m - d[c] X[c,c], r_c = ||Y[:,c] - X[:,c] m||,
//   Y[c,c] = 1, Y[i,c] = (Y[i,c] - d[i] X[i,c] - X[i,c] u) / (d[c] - d[i])
// and a flag where |d[c] - d[i]| <= DBL_EPSILON (acx_cuda.cu:109-172).
__global__ void __launch_bounds__(kAcxThreads)
acx_map_kernel(double *__restrict__ Y, const double *__restrict__ X, const double *__restrict__ d,
               int n, double *__restrict__ resid, int *__restrict__ flag)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const int c = blockIdx.x;
    double *y = Y + (size_t)c * n;
    const double *x = X + (size_t)c * n;
    __shared__ double mu[2];
    if (threadIdx.x == 0) {
        const double m = y[c];
        mu[0] = m;
        mu[1] = fma(-d[c], x[c], m);
    }
    __syncthreads();
    const double m = mu[0], u = mu[1], dc = d[c];
    double rr = 0.0;
    bool bad = false;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double yi = y[i], xi = x[i];
        const double r = fma(-xi, m, yi);
        rr = fma(r, r, rr);
        double v = 1.0;
        if (i != c) {
            const double den = dc - d[i];
            if (fabs(den) <= DBL_EPSILON) {
                bad = true;
                v = 0.0;
            } else {
                v = fma(-xi, u, fma(-d[i], xi, yi)) / den;
            }
        }
        y[i] = v;
    }
    const double2 s = block_sum2(rr, 0.0);
    if (threadIdx.x == 0) resid[c] = sqrt(s.x);
    if (bad) atomicOr(flag, 1);
}

// out = (||A - B||_F, ||B||_F), deterministic.
__global__ void __launch_bounds__(kAcxThreads)
acx_norms_kernel(const double *__restrict__ A, const double *__restrict__ B, size_t count,
                 double2 *__restrict__ partials, unsigned int *__restrict__ counter,
                 double *__restrict__ out)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    double dd = 0.0, bb = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (size_t)gridDim.x * blockDim.x) {
        const double b = B[i];
        const double t = A[i] - b;
        dd = fma(t, t, dd);
        bb = fma(b, b, bb);
    }
    grid_finish_norms2(block_sum2(dd, bb), partials, counter, out);
}

// One extrapolation step, one CTA per column (acx_cuda.cu:190-296); F3 is
// null for an order-2 step.
__global__ void __launch_bounds__(kAcxThreads)
acx_extrapolate_kernel(double *__restrict__ X, const double *__restrict__ F1,
                       const double *__restrict__ F2, const double *__restrict__ F3, int n)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const size_t base = (size_t)blockIdx.x * n;
    double *x = X + base;
    const double *f1 = F1 + base;
    const double *f2 = F2 + base;
    const double *f3 = F3 != nullptr ? F3 + base : nullptr;
    double num = 0.0, den = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double d2 = fma(-2.0, f1[i], f2[i]) + x[i];
        if (f3 == nullptr) {
            const double d1 = f1[i] - x[i];
            num = fma(d2, d1, num);
            den = fma(d2, d2, den);
        } else {
            const double d3 = fma(3.0, f1[i], fma(-3.0, f2[i], f3[i])) - x[i];
            num = fma(d3, d2, num);
            den = fma(d3, d3, den);
        }
    }
    const double2 s = block_sum2(num, den);
    __shared__ double sig;
    if (threadIdx.x == 0) sig = s.y > 0.0 ? fabs(s.x / s.y) : 0.0;
    __syncthreads();
    const double g = sig, g2 = g * g, g3 = g2 * g;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double xi = x[i];
        const double d1 = f1[i] - xi;
        const double d2 = fma(-2.0, f1[i], f2[i]) + xi;
        if (f3 == nullptr) {
            x[i] = xi + fma(2.0 * g, d1, g2 * d2);
        } else {
            const double d3 = fma(3.0, f1[i], fma(-3.0, f2[i], f3[i])) - xi;
            x[i] = xi + fma(3.0 * g, d1, fma(3.0 * g2, d2, g3 * d3));
        }
    }
}

namespace {

struct AcxDense {
    const double *H = nullptr;
    int n = 0, k = 0, S = 1;
    cudaStream_t s = nullptr;
    const double *d = nullptr;
    double *P = nullptr, *resid = nullptr;
    int *flag = nullptr;
    // Y = F(X)
    int apply(const double *X, double *Y)
    {
        if (S > 1) {
            IPTGB_CHECK(launch_dense64_partial(H, n, n, X, n, k, P, S, s));
            IPTGB_CHECK(launch_sum_partials(P, S, (size_t)n * k, Y, s));
        } else {
            IPTGB_CHECK(launch_dense64_partial(H, n, n, X, n, k, Y, 1, s));
        }
        return launch_pdl(acx_map_kernel, dim3(k), dim3(kAcxThreads), 0, s, Y, X, d, n, resid,
                          flag);
    }
};

double seconds_since(std::chrono::steady_clock::time_point t)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
}

}  // namespace

}  // namespace iptgb

#define IPT_API extern "C" __attribute__((visibility("default")))

using namespace iptgb;

IPT_API const char *acx_cuda_status_string(int status)
{
    switch (status) {
    case ACX_CUDA_SUCCESS: return "success";
    case ACX_CUDA_INVALID_ARGUMENT: return "invalid argument";
    case ACX_CUDA_ALLOCATION_FAILED: return "allocation failed";
    case ACX_CUDA_CUDA_ERROR: return "cuda error";
    case ACX_CUDA_CUBLAS_ERROR: return "cublas error";
    case ACX_CUDA_ZERO_DENOMINATOR: return "zero diagonal denominator";
    default: return "unknown error";
    }
}

IPT_API void acx_cuda_reset_result(ACXCudaResult *result)
{
    if (result == nullptr) return;
    memset(result, 0, sizeof(*result));
    result->max_residual = NAN;
    result->fixed_point_residual = NAN;
}

IPT_API void acx_cuda_free_result(ACXCudaResult *result)
{
    if (result == nullptr) return;
    cudaFree(result->d_vectors);
    cudaFree(result->d_values);
    acx_cuda_reset_result(result);
}

IPT_API int acx_cuda_device_tol(const double *d_matrix_col_major, int n, int k, double tol,
                                int maxiter, cublasHandle_t handle, ACXCudaResult *result)
{
    if (result == nullptr) return ACX_CUDA_INVALID_ARGUMENT;
    acx_cuda_reset_result(result);
    const auto t0 = std::chrono::steady_clock::now();
    if (d_matrix_col_major == nullptr || n <= 0 || k <= 0 || k > n || !(tol > 0.0) ||
        maxiter <= 0) {
        return ACX_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = nullptr;
    if (handle != nullptr && cublasGetStream(handle, &s) != CUBLAS_STATUS_SUCCESS) {
        return ACX_CUDA_CUBLAS_ERROR;
    }
    const size_t elems = (size_t)n * (size_t)k;
    const double stop_tol = tol < 1.0e-12 ? tol : 1.0e-12;  // ACX_FIXED_POINT_RTOL
    double *f1 = nullptr, *values = nullptr;
    if (cudaMalloc((void **)&f1, elems * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void **)&values, (size_t)k * sizeof(double)) != cudaSuccess) {
        cudaFree(f1);
        return ACX_CUDA_ALLOCATION_FAILED;
    }
    int status = ACX_CUDA_SUCCESS;
    {
        AcxDense F;
        F.H = d_matrix_col_major;
        F.n = n;
        F.k = k;
        F.s = s;
        F.S = dense64_split_for(n, k, device_sm_count());
        DeviceBuffer<double> X, F2, F3, P, small;
        DeviceBuffer<double2> part;
        DeviceBuffer<int> flags;
        // small: d (n) | resid (k) | norms (2)
        bool ok = X.alloc(elems, s) == IPT_CUDA_SUCCESS && F2.alloc(elems, s) == IPT_CUDA_SUCCESS &&
                  F3.alloc(elems, s) == IPT_CUDA_SUCCESS &&
                  (F.S <= 1 || P.alloc(elems * (size_t)F.S, s) == IPT_CUDA_SUCCESS) &&
                  small.alloc((size_t)n + (size_t)k + 2, s) == IPT_CUDA_SUCCESS &&
                  part.alloc(kAcxNormBlocks, s) == IPT_CUDA_SUCCESS &&
                  flags.alloc(2, s) == IPT_CUDA_SUCCESS;
        if (!ok) status = ACX_CUDA_ALLOCATION_FAILED;
        double *d = small.ptr, *resid = small.ptr + n, *norms = small.ptr + n + k;
        int *flag = flags.ptr;
        unsigned int *counter = reinterpret_cast<unsigned int *>(flags.ptr + 1);
        F.d = d;
        F.P = P.ptr;
        F.resid = resid;
        F.flag = flag;
        auto cuda_ok = [&](cudaError_t e) {
            if (e != cudaSuccess && status == ACX_CUDA_SUCCESS) status = ACX_CUDA_CUDA_ERROR;
            return status == ACX_CUDA_SUCCESS;
        };
        auto lib_ok = [&](int st) {
            if (st != IPT_CUDA_SUCCESS && status == ACX_CUDA_SUCCESS) status = ACX_CUDA_CUDA_ERROR;
            return status == ACX_CUDA_SUCCESS;
        };
        if (status == ACX_CUDA_SUCCESS) {
            cuda_ok(cudaMemsetAsync(flags.ptr, 0, 2 * sizeof(int), s));
            lib_ok(launch_extract_diagonal(d_matrix_col_major, n, n, d, s));
            lib_ok(launch_set_identity(X.ptr, n, k, s));
        }
        std::vector<double> host((size_t)k + 2);
        int hflag = 0;
        const auto t_iter = std::chrono::steady_clock::now();
        for (int iter = 1; iter <= maxiter && status == ACX_CUDA_SUCCESS; ++iter) {
            const int order = (iter % 2 == 1) ? 2 : 3;
            result->iterations = iter;
            if (!lib_ok(F.apply(X.ptr, f1))) break;
            result->f_calls += 1;
            if (!lib_ok(launch_pdl(acx_norms_kernel, dim3(kAcxNormBlocks), dim3(kAcxThreads), 0,
                                   s, (const double *)f1, (const double *)X.ptr, elems, part.ptr,
                                   counter, norms))) {
                break;
            }
            if (!cuda_ok(cudaMemcpyAsync(host.data(), resid, ((size_t)k + 2) * sizeof(double),
                                         cudaMemcpyDeviceToHost, s)) ||
                !cuda_ok(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, s)) ||
                !cuda_ok(cudaStreamSynchronize(s))) {
                break;
            }
            if (hflag != 0) {
                status = ACX_CUDA_ZERO_DENOMINATOR;
                break;
            }
            double mx = 0.0;
            for (int c = 0; c < k; ++c) mx = host[(size_t)c] > mx ? host[(size_t)c] : mx;
            result->max_residual = mx;
            const double dn = host[(size_t)k], xn = host[(size_t)k + 1];
            if (!(xn > 0.0) || !isfinite(xn)) {
                status = ACX_CUDA_INVALID_ARGUMENT;
                break;
            }
            result->fixed_point_residual = dn / xn;
            if (result->fixed_point_residual < stop_tol) {
                result->converged = 1;
                break;
            }
            if (!lib_ok(F.apply(f1, F2.ptr))) break;
            result->f_calls += 1;
            if (order == 3) {
                if (!lib_ok(F.apply(F2.ptr, F3.ptr))) break;
                result->f_calls += 1;
            }
            lib_ok(launch_pdl(acx_extrapolate_kernel, dim3(k), dim3(kAcxThreads), 0, s, X.ptr,
                              (const double *)f1, (const double *)F2.ptr,
                              order == 3 ? (const double *)F3.ptr : (const double *)nullptr, n));
        }
        result->iteration_time_sec = seconds_since(t_iter);
        const auto t_fin = std::chrono::steady_clock::now();
        if (status == ACX_CUDA_SUCCESS) {
            lib_ok(launch_dense64_diag_values(d_matrix_col_major, n, n, f1, k, values, s));
            cuda_ok(cudaStreamSynchronize(s));
        }
        result->finalization_time_sec = seconds_since(t_fin);
    }
    if (status != ACX_CUDA_SUCCESS) {
        cudaFree(f1);
        cudaFree(values);
        acx_cuda_reset_result(result);
        return status;
    }
    result->n = n;
    result->k = k;
    result->d_vectors = f1;
    result->d_values = values;
    result->time_sec = seconds_since(t0);
    return ACX_CUDA_SUCCESS;
}
