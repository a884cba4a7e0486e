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
#include "rayleigh.h"
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

// out = (||A - B||_F, ||B||_F), deterministic (sums in FP64 for either type).
template <typename T>
__global__ void __launch_bounds__(kAcxThreads)
acx_norms_kernel(const T *__restrict__ A, const T *__restrict__ B, size_t count,
                 double2 *__restrict__ partials, unsigned int *__restrict__ counter,
                 double *__restrict__ out)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    double dd = 0.0, bb = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (size_t)gridDim.x * blockDim.x) {
        const double b = (double)B[i];
        const double t = (double)A[i] - b;
        dd = fma(t, t, dd);
        bb = fma(b, b, bb);
    }
    grid_finish_norms2(block_sum2(dd, bb), partials, counter, out);
}

// One extrapolation step, one CTA per column (acx_cuda.cu:190-296, and the
// FP32 pair of acx_mixed_precision_cuda.cu:198-319); F3 is null for an
// order-2 step.  The inner products accumulate in T, the step length is
// formed in FP64 from their block sums.
template <typename T>
__global__ void __launch_bounds__(kAcxThreads)
acx_extrapolate_kernel(T *__restrict__ X, const T *__restrict__ F1, const T *__restrict__ F2,
                       const T *__restrict__ F3, int n)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const size_t base = (size_t)blockIdx.x * n;
    T *x = X + base;
    const T *f1 = F1 + base;
    const T *f2 = F2 + base;
    const T *f3 = F3 != nullptr ? F3 + base : nullptr;
    const T two = T(2), three = T(3);
    T num = T(0), den = T(0);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const T d2 = fma(-two, f1[i], f2[i]) + x[i];
        if (f3 == nullptr) {
            const T d1 = f1[i] - x[i];
            num = fma(d2, d1, num);
            den = fma(d2, d2, den);
        } else {
            const T d3 = fma(three, f1[i], fma(-three, f2[i], f3[i])) - x[i];
            num = fma(d3, d2, num);
            den = fma(d3, d3, den);
        }
    }
    const double2 s = block_sum2((double)num, (double)den);
    __shared__ double sig;
    if (threadIdx.x == 0) sig = s.y > 0.0 ? fabs(s.x / s.y) : 0.0;
    __syncthreads();
    const T g = (T)sig, g2 = g * g, g3 = g2 * g;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const T xi = x[i];
        const T d1 = f1[i] - xi;
        const T d2 = fma(-two, f1[i], f2[i]) + xi;
        if (f3 == nullptr) {
            x[i] = xi + fma(two * g, d1, g2 * d2);
        } else {
            const T d3 = fma(three, f1[i], fma(-three, f2[i], f3[i])) - xi;
            x[i] = xi + fma(three * g, d1, fma(three * g2, d2, g3 * d3));
        }
    }
}

// ---- FP32 stage of the mixed ACX (acx_mixed_precision_cuda.cu:100-360) ----
// Delta in FP32 with a zero diagonal, and the diagonal in FP32.
__global__ void acx_offdiag_f32_kernel(const double *__restrict__ H, int n, float *__restrict__ D,
                                       float *__restrict__ dg)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const size_t total = (size_t)n * n;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(i % (size_t)n), c = (int)(i / (size_t)n);
        const float v = __double2float_rn(H[i]);
        D[i] = r == c ? 0.0f : v;
        if (r == c) dg[r] = v;
    }
}

__global__ void acx_sum_partials_f32_kernel(const float *__restrict__ P, int S, size_t elems,
                                            float *__restrict__ Y)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= elems) return;
    float y = 0.0f;
    for (int s = 0; s < S; ++s) y += P[(size_t)s * elems + idx];
    Y[idx] = y;
}

// Y = F(X) in place on Y = Delta X (FP32), one CTA per column c:
//   u = Y[c,c], Y[c,c] = 1, Y[i,c] = (Y[i,c] - X[i,c] u) / (d[c] - d[i])
// and a flag where |d[c] - d[i]| <= FLT_EPSILON (acx_mixed_precision_cuda.cu:160-196).
__global__ void __launch_bounds__(kAcxThreads)
acx_map_f32_kernel(float *__restrict__ Y, const float *__restrict__ X, const float *__restrict__ d,
                   int n, int *__restrict__ flag)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const int c = blockIdx.x;
    float *y = Y + (size_t)c * n;
    const float *x = X + (size_t)c * n;
    __shared__ float u_sh;
    if (threadIdx.x == 0) u_sh = y[c];
    __syncthreads();
    const float u = u_sh, dc = d[c];
    bool bad = false;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        float v = 1.0f;
        if (i != c) {
            const float den = dc - d[i];
            if (fabsf(den) <= FLT_EPSILON) {
                bad = true;
                v = 0.0f;
            } else {
                v = __fdiv_rn(fmaf(-x[i], u, y[i]), den);
            }
        }
        y[i] = v;
    }
    if (bad) atomicOr(flag, 1);
}

__global__ void acx_f32_to_f64_kernel(const float *__restrict__ in, size_t count,
                                      double *__restrict__ out)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) out[i] = (double)in[i];
}

__global__ void acx_identity_f32_kernel(float *__restrict__ X, int n, int k)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const size_t total = (size_t)n * k;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        X[i] = (int)(i % (size_t)n) == (int)(i / (size_t)n) ? 1.0f : 0.0f;
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

struct AcxDense32 {
    const float *D = nullptr;  // Delta, zero diagonal
    const float *d = nullptr;
    int n = 0, k = 0, S = 1;
    cudaStream_t s = nullptr;
    float *P = nullptr;
    int *flag = nullptr;
    int apply(const float *X, float *Y)
    {
        if (S > 1) {
            IPTGB_CHECK(launch_dense32_partial(D, n, n, X, n, k, P, S, s));
            IPTGB_CHECK(launch_pdl(acx_sum_partials_f32_kernel, dim3(blocks_for((size_t)n * k)),
                                   dim3(kThreads), 0, s, (const float *)P, S, (size_t)n * k, Y));
        } else {
            IPTGB_CHECK(launch_dense32_partial(D, n, n, X, n, k, Y, 1, s));
        }
        return launch_pdl(acx_map_f32_kernel, dim3(k), dim3(kAcxThreads), 0, s, Y, X, d, n, flag);
    }
};

double seconds_since(std::chrono::steady_clock::time_point t)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
}

// grid-stride kernels: at most eight CTAs per SM
int grid_cap(size_t count)
{
    const int b = blocks_for(count);
    const int cap = 8 * device_sm_count();
    return b < cap ? b : cap;
}

// The FP64 ACX loop (acx_cuda.cu:390-620).  From the identity (initial ==
// nullptr) the result vectors are the last F(X); from a given start block
// (the second stage of the mixed ACX, acx_mixed_precision_cuda.cu:575-809)
// they are F(X) when the stop was met and the extrapolated X otherwise.
// Values are diag(H V).  On success result->d_vectors / d_values are
// cudaMalloc buffers owned by the caller.
int acx_fp64_run(const double *H, int n, int k, double tol, int maxiter, const double *initial,
                 cudaStream_t s, ACXCudaResult *result)
{
    const auto t0 = std::chrono::steady_clock::now();
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
        F.H = H;
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
            lib_ok(launch_extract_diagonal(H, n, n, d, s));
            if (initial == nullptr) {
                lib_ok(launch_set_identity(X.ptr, n, k, s));
            } else {
                cuda_ok(cudaMemcpyAsync(X.ptr, initial, elems * sizeof(double),
                                        cudaMemcpyDeviceToDevice, s));
            }
        }
        std::vector<double> host((size_t)k + 2);
        int hflag = 0;
        bool final_is_x = initial != nullptr;
        const auto t_iter = std::chrono::steady_clock::now();
        for (int iter = 1; iter <= maxiter && status == ACX_CUDA_SUCCESS; ++iter) {
            const int order = (iter % 2 == 1) ? 2 : 3;
            result->iterations = iter;
            if (!lib_ok(F.apply(X.ptr, f1))) break;
            result->f_calls += 1;
            if (!lib_ok(launch_pdl(acx_norms_kernel<double>, dim3(kAcxNormBlocks),
                                   dim3(kAcxThreads), 0, s, (const double *)f1,
                                   (const double *)X.ptr, elems, part.ptr, counter, norms))) {
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
                final_is_x = false;
                break;
            }
            if (!lib_ok(F.apply(f1, F2.ptr))) break;
            result->f_calls += 1;
            if (order == 3) {
                if (!lib_ok(F.apply(F2.ptr, F3.ptr))) break;
                result->f_calls += 1;
            }
            lib_ok(launch_pdl(acx_extrapolate_kernel<double>, dim3(k), dim3(kAcxThreads), 0, s,
                              X.ptr, (const double *)f1, (const double *)F2.ptr,
                              order == 3 ? (const double *)F3.ptr : (const double *)nullptr, n));
        }
        result->iteration_time_sec = seconds_since(t_iter);
        const auto t_fin = std::chrono::steady_clock::now();
        if (status == ACX_CUDA_SUCCESS) {
            if (final_is_x) {
                cuda_ok(cudaMemcpyAsync(f1, X.ptr, elems * sizeof(double),
                                        cudaMemcpyDeviceToDevice, s));
            }
            lib_ok(launch_dense64_diag_values(H, n, n, f1, k, values, s));
            cuda_ok(cudaStreamSynchronize(s));
        }
        result->finalization_time_sec = seconds_since(t_fin);
    }
    if (status != ACX_CUDA_SUCCESS) {
        cudaFree(f1);
        cudaFree(values);
        return status;
    }
    result->n = n;
    result->k = k;
    result->d_vectors = f1;
    result->d_values = values;
    result->time_sec = seconds_since(t0);
    return ACX_CUDA_SUCCESS;
}

// The FP32 stage of the mixed ACX (acx_mixed_precision_cuda.cu:360-573):
// the same extrapolation on the map with Delta and the diagonal in FP32,
// stopping at ||F(X) - X|| / ||X|| <= tol; `initial` (n x k, FP64) receives
// F(X) when the stop was met and the extrapolated X otherwise.  The reference
// multiplies with a TF32 GEMM; here the product is the FP32 split-K kernel
// (k_dense64.cu), which rounds no operand.
int acx_fp32_run(const double *H, int n, int k, double tol, int maxiter, cudaStream_t s,
                 double *initial, int *iterations, int *f_calls, int *converged, double *fpres)
{
    const size_t elems = (size_t)n * (size_t)k;
    AcxDense32 F;
    F.n = n;
    F.k = k;
    F.s = s;
    F.S = dense64_split_for(n, k, device_sm_count());
    DeviceBuffer<float> D, dg, X, F1, F2, F3, P;
    DeviceBuffer<double> norms;
    DeviceBuffer<double2> part;
    DeviceBuffer<int> flags;
    if (D.alloc((size_t)n * n, s) != IPT_CUDA_SUCCESS || dg.alloc((size_t)n, s) != IPT_CUDA_SUCCESS ||
        X.alloc(elems, s) != IPT_CUDA_SUCCESS || F1.alloc(elems, s) != IPT_CUDA_SUCCESS ||
        F2.alloc(elems, s) != IPT_CUDA_SUCCESS || F3.alloc(elems, s) != IPT_CUDA_SUCCESS ||
        (F.S > 1 && P.alloc(elems * (size_t)F.S, s) != IPT_CUDA_SUCCESS) ||
        norms.alloc(2, s) != IPT_CUDA_SUCCESS || part.alloc(kAcxNormBlocks, s) != IPT_CUDA_SUCCESS ||
        flags.alloc(2, s) != IPT_CUDA_SUCCESS) {
        return ACX_CUDA_ALLOCATION_FAILED;
    }
    F.D = D.ptr;
    F.d = dg.ptr;
    F.P = P.ptr;
    F.flag = flags.ptr;
    unsigned int *counter = reinterpret_cast<unsigned int *>(flags.ptr + 1);
    if (cudaMemsetAsync(flags.ptr, 0, 2 * sizeof(int), s) != cudaSuccess ||
        launch_pdl(acx_offdiag_f32_kernel, dim3(grid_cap((size_t)n * n)), dim3(kThreads), 0, s, H,
                   n, D.ptr, dg.ptr) != IPT_CUDA_SUCCESS ||
        launch_pdl(acx_identity_f32_kernel, dim3(grid_cap(elems)), dim3(kThreads), 0, s, X.ptr, n,
                   k) != IPT_CUDA_SUCCESS) {
        return ACX_CUDA_CUDA_ERROR;
    }
    const float *final_block = X.ptr;
    double host[2];
    int hflag = 0;
    for (int iter = 1; iter <= maxiter; ++iter) {
        const int order = (iter % 2 == 1) ? 2 : 3;
        *iterations = iter;
        if (F.apply(X.ptr, F1.ptr) != IPT_CUDA_SUCCESS) return ACX_CUDA_CUDA_ERROR;
        *f_calls += 1;
        if (launch_pdl(acx_norms_kernel<float>, dim3(kAcxNormBlocks), dim3(kAcxThreads), 0, s,
                       (const float *)F1.ptr, (const float *)X.ptr, elems, part.ptr, counter,
                       norms.ptr) != IPT_CUDA_SUCCESS ||
            cudaMemcpyAsync(host, norms.ptr, sizeof(host), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(&hflag, flags.ptr, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            return ACX_CUDA_CUDA_ERROR;
        }
        if (hflag != 0) return ACX_CUDA_ZERO_DENOMINATOR;
        if (!(host[1] > 0.0) || !isfinite(host[1])) return ACX_CUDA_INVALID_ARGUMENT;
        *fpres = host[0] / host[1];
        if (*fpres <= tol) {
            *converged = 1;
            final_block = F1.ptr;
            break;
        }
        if (F.apply(F1.ptr, F2.ptr) != IPT_CUDA_SUCCESS) return ACX_CUDA_CUDA_ERROR;
        *f_calls += 1;
        if (order == 3) {
            if (F.apply(F2.ptr, F3.ptr) != IPT_CUDA_SUCCESS) return ACX_CUDA_CUDA_ERROR;
            *f_calls += 1;
        }
        if (launch_pdl(acx_extrapolate_kernel<float>, dim3(k), dim3(kAcxThreads), 0, s, X.ptr,
                       (const float *)F1.ptr, (const float *)F2.ptr,
                       order == 3 ? (const float *)F3.ptr : (const float *)nullptr,
                       n) != IPT_CUDA_SUCCESS) {
            return ACX_CUDA_CUDA_ERROR;
        }
        final_block = X.ptr;
    }
    if (launch_pdl(acx_f32_to_f64_kernel, dim3(blocks_for(elems)), dim3(kThreads), 0, s,
                   final_block, elems, initial) != IPT_CUDA_SUCCESS ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        return ACX_CUDA_CUDA_ERROR;
    }
    return ACX_CUDA_SUCCESS;
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
    if (d_matrix_col_major == nullptr || n <= 0 || k <= 0 || k > n || !(tol > 0.0) ||
        maxiter <= 0) {
        return ACX_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = nullptr;
    if (handle != nullptr && cublasGetStream(handle, &s) != CUBLAS_STATUS_SUCCESS) {
        return ACX_CUDA_CUBLAS_ERROR;
    }
    const int st = acx_fp64_run(d_matrix_col_major, n, k, tol, maxiter, nullptr, s, result);
    if (st != ACX_CUDA_SUCCESS) acx_cuda_reset_result(result);
    return st;
}

IPT_API void acx_mixed_precision_tf32_cuda_reset_result(ACXMixedTF32CudaResult *result)
{
    if (result == nullptr) return;
    memset(result, 0, sizeof(*result));
    result->tf32_time_sec = NAN;
    result->fp64_time_sec = NAN;
    result->total_time_sec = NAN;
    result->finalization_time_sec = NAN;
    result->tf32_fixed_point_residual = NAN;
    result->fp64_fixed_point_residual = NAN;
    result->fp64_max_residual = NAN;
}

IPT_API void acx_mixed_precision_tf32_cuda_free_result(ACXMixedTF32CudaResult *result)
{
    if (result == nullptr) return;
    cudaFree(result->d_vectors);
    cudaFree(result->d_values);
    acx_mixed_precision_tf32_cuda_reset_result(result);
}

IPT_API int acx_mixed_precision_tf32_cuda_device_tol(const double *d_matrix_col_major, int n,
                                                     int k, double tf32_tol, int tf32_maxiter,
                                                     double fp64_tol, int fp64_maxiter,
                                                     cublasHandle_t handle,
                                                     ACXMixedTF32CudaResult *result)
{
    if (result == nullptr) return ACX_CUDA_INVALID_ARGUMENT;
    acx_mixed_precision_tf32_cuda_reset_result(result);
    if (d_matrix_col_major == nullptr || handle == nullptr || n <= 0 || k <= 0 || k > n ||
        !(tf32_tol > 0.0) || !(fp64_tol > 0.0) || tf32_maxiter <= 0 || fp64_maxiter <= 0) {
        return ACX_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = nullptr;
    if (cublasGetStream(handle, &s) != CUBLAS_STATUS_SUCCESS) return ACX_CUDA_CUBLAS_ERROR;
    const auto t0 = std::chrono::steady_clock::now();
    DeviceBuffer<double> initial;
    if (initial.alloc((size_t)n * (size_t)k, s) != IPT_CUDA_SUCCESS) {
        return ACX_CUDA_ALLOCATION_FAILED;
    }
    int st = acx_fp32_run(d_matrix_col_major, n, k, tf32_tol, tf32_maxiter, s, initial.ptr,
                          &result->tf32_iterations, &result->tf32_f_calls,
                          &result->tf32_converged, &result->tf32_fixed_point_residual);
    result->tf32_time_sec = seconds_since(t0);
    ACXCudaResult r64;
    acx_cuda_reset_result(&r64);
    const auto t1 = std::chrono::steady_clock::now();
    if (st == ACX_CUDA_SUCCESS) {
        st = acx_fp64_run(d_matrix_col_major, n, k, fp64_tol, fp64_maxiter, initial.ptr, s, &r64);
    }
    if (st != ACX_CUDA_SUCCESS) {
        acx_mixed_precision_tf32_cuda_reset_result(result);
        return st;
    }
    result->fp64_time_sec = seconds_since(t1);
    result->total_time_sec = seconds_since(t0);
    result->n = n;
    result->k = k;
    result->fp64_iterations = r64.iterations;
    result->fp64_f_calls = r64.f_calls;
    result->fp64_converged = r64.converged;
    result->finalization_time_sec = r64.finalization_time_sec;
    result->fp64_fixed_point_residual = r64.fixed_point_residual;
    result->fp64_max_residual = r64.max_residual;
    result->d_vectors = r64.d_vectors;
    result->d_values = r64.d_values;
    return ACX_CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------
// Rayleigh ACX (IPT_C_GPU/src/ACX/acx_rayleigh_mixed_precision_cuda.cu:289-434)
// ---------------------------------------------------------------------------
IPT_API void acx_rayleigh_mixed_tf32_cuda_reset_result(ACXRayleighMixedTF32CudaResult *result)
{
    if (result == nullptr) return;
    memset(result, 0, sizeof(*result));
    result->tf32_time_sec = NAN;
    result->orthogonalize_time_sec = NAN;
    result->rayleigh_transform_time_sec = NAN;
    result->fp64_time_sec = NAN;
    result->finalization_time_sec = NAN;
    result->backtransform_time_sec = NAN;
    result->total_time_sec = NAN;
    result->tf32_fixed_point_residual = NAN;
    result->fp64_fixed_point_residual = NAN;
    result->fp64_max_residual = NAN;
}

IPT_API void acx_rayleigh_mixed_tf32_cuda_free_result(ACXRayleighMixedTF32CudaResult *result)
{
    if (result == nullptr) return;
    cudaFree(result->d_vectors);
    cudaFree(result->d_values);
    acx_rayleigh_mixed_tf32_cuda_reset_result(result);
}

namespace {

// Largest k of the Rayleigh ACX: the CholQR's Cholesky inverse holds two
// k x k FP64 matrices in one CTA's shared memory.
constexpr int kAcxRayleighMaxK = 112;

int acx_rayleigh_run(const double *dH, int n, int k, double tf32_tol, int tf32_maxiter,
                     double fp64_tol, int fp64_maxiter, cudaStream_t s,
                     ACXRayleighMixedTF32CudaResult *out)
{
    const size_t elems = (size_t)n * (size_t)k;
    DeviceBuffer<double> X0, Q, B;
    IPTGB_CHECK(X0.alloc(elems, s));
    // 1. ACX of the low-precision map (the reference's TF32 ACX stage)
    auto t = std::chrono::steady_clock::now();
    IPTGB_CHECK(acx_fp32_run(dH, n, k, tf32_tol, tf32_maxiter, s, X0.ptr, &out->tf32_iterations,
                             &out->tf32_f_calls, &out->tf32_converged,
                             &out->tf32_fixed_point_residual));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    out->tf32_time_sec = seconds_since(t);
    // 2. orthonormal basis; the reference normalises the columns first, which
    // changes neither the span nor the Householder column signs
    BlockOps ops;
    ops.stream = s;
    ops.sms = device_sm_count();
    struct OpsGuard {
        BlockOps *o;
        ~OpsGuard() { o->release(); }
    } og{&ops};
    t = std::chrono::steady_clock::now();
    IPTGB_CHECK(Q.alloc(elems, s));
    IPTGB_CHECK(householder_basis(ops, X0.ptr, n, k, Q.ptr, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    out->orthogonalize_time_sec = seconds_since(t);
    // 3. B = sym(Q^T H Q)
    t = std::chrono::steady_clock::now();
    IPTGB_CHECK(B.alloc((size_t)k * k, s));
    IPTGB_CHECK(projected_matrix(ops, dH, n, Q.ptr, k, B.ptr, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    out->rayleigh_transform_time_sec = seconds_since(t);
    // 4. FP64 ACX on the k x k matrix
    t = std::chrono::steady_clock::now();
    ACXCudaResult r64;
    acx_cuda_reset_result(&r64);
    int st = acx_fp64_run(B.ptr, k, k, fp64_tol, fp64_maxiter, nullptr, s, &r64);
    if (st != ACX_CUDA_SUCCESS) return st;
    out->fp64_time_sec = seconds_since(t);
    out->fp64_iterations = r64.iterations;
    out->fp64_f_calls = r64.f_calls;
    out->fp64_converged = r64.converged;
    out->finalization_time_sec = r64.finalization_time_sec;
    out->fp64_fixed_point_residual = r64.fixed_point_residual;
    out->fp64_max_residual = r64.max_residual;
    // 5. vectors = Q Z
    t = std::chrono::steady_clock::now();
    double *vecs = nullptr;
    if (cudaMalloc((void **)&vecs, elems * sizeof(double)) != cudaSuccess) {
        acx_cuda_free_result(&r64);
        return ACX_CUDA_ALLOCATION_FAILED;
    }
    st = ops.tall_gemm(Q.ptr, n, r64.d_vectors, k, vecs, n, n, k, k);
    if (st == IPT_CUDA_SUCCESS && cudaStreamSynchronize(s) != cudaSuccess) {
        st = ACX_CUDA_CUDA_ERROR;
    }
    if (st != IPT_CUDA_SUCCESS) {
        cudaFree(vecs);
        acx_cuda_free_result(&r64);
        return st;
    }
    out->backtransform_time_sec = seconds_since(t);
    cudaFree(r64.d_vectors);
    out->d_vectors = vecs;
    out->d_values = r64.d_values;
    out->total_time_sec = out->tf32_time_sec + out->orthogonalize_time_sec +
                          out->rayleigh_transform_time_sec + out->fp64_time_sec +
                          out->backtransform_time_sec;
    out->n = n;
    out->k = k;
    return ACX_CUDA_SUCCESS;
}

}  // namespace

IPT_API int acx_rayleigh_mixed_tf32_cuda_device_tol(const double *d_matrix_col_major, int n,
                                                    int k, double tf32_tol, int tf32_maxiter,
                                                    double fp64_tol, int fp64_maxiter,
                                                    cublasHandle_t handle,
                                                    ACXRayleighMixedTF32CudaResult *result)
{
    if (result == nullptr) return ACX_CUDA_INVALID_ARGUMENT;
    acx_rayleigh_mixed_tf32_cuda_reset_result(result);
    if (d_matrix_col_major == nullptr || handle == nullptr || n <= 0 || k <= 0 || k > n ||
        !(tf32_tol > 0.0) || !(fp64_tol > 0.0) || tf32_maxiter <= 0 || fp64_maxiter <= 0) {
        return ACX_CUDA_INVALID_ARGUMENT;
    }
    if ((size_t)n * (size_t)k > (size_t)INT_MAX || (size_t)k * (size_t)k > (size_t)INT_MAX) {
        return ACX_CUDA_INVALID_ARGUMENT;
    }
    if (k > kAcxRayleighMaxK) {
        fprintf(stderr, "ipt_gb300: acx_rayleigh_mixed_tf32_cuda_device_tol supports k <= %d "
                        "(got %d)\n", kAcxRayleighMaxK, k);
        return ACX_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = nullptr;
    if (cublasGetStream(handle, &s) != CUBLAS_STATUS_SUCCESS) return ACX_CUDA_CUBLAS_ERROR;
    const int st = acx_rayleigh_run(d_matrix_col_major, n, k, tf32_tol, tf32_maxiter, fp64_tol,
                                    fp64_maxiter, s, result);
    if (st != ACX_CUDA_SUCCESS) {
        cudaFree(result->d_vectors);
        cudaFree(result->d_values);
        acx_rayleigh_mixed_tf32_cuda_reset_result(result);
    }
    return st;
}

