// ipt_plain.cu - FP64 plain-IPT driver loop.
#include <math.h>

#include "common.cuh"
#include "ipt_plain.h"

namespace iptgb {

int device_sm_count()
{
    int dev = 0;
    int sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0) {
        return 148;
    }
    return sms;
}

int DenseFp64Operator::step(const double *X, double *Xn, const double *d, int want_norms,
                            NormScratch *ns)
{
    {
        KernelTimerScope timer(kProfFp64Product, stream);
        IPTGB_CHECK(launch_dense64_partial(H, n, ldh, X, n, k, P, S, stream));
    }
    KernelTimerScope timer(kProfFp64Update, stream);
    return launch_dense64_update(P, S, n, k, X, d, Xn, want_norms, ns, stream);
}

int DenseFp64Operator::diag_values(const double *X, double *values)
{
    return launch_dense64_diag_values(H, ldh, n, X, k, values, stream);
}

int CsrFp64Operator::step(const double *X, double *Xn, const double *d, int want_norms,
                          NormScratch *ns)
{
    {
        KernelTimerScope timer(kProfCsrProduct, stream);
        IPTGB_CHECK(launch_csr64_spmm(row_ptr, col_ind, vals, n, X, k, Y, stream));
    }
    KernelTimerScope timer(kProfFp64Update, stream);
    return launch_ipt_update_from_y(Y, n, k, X, d, Xn, want_norms, ns, stream);
}

int CsrFp64Operator::diag_values(const double *X, double *values)
{
    return launch_csr64_diag_values(row_ptr, col_ind, vals, n, X, k, values, stream);
}

int SolveScratch::init(size_t max_elems, cudaStream_t stream)
{
    const int slots = blocks_for(max_elems);
    IPTGB_CUDA(cudaMallocAsync((void **)&ns.partials, (size_t)slots * sizeof(double2), stream));
    // [counter u32 | pad][norms double x2]
    IPTGB_CUDA(cudaMallocAsync((void **)&ns.counter, 32, stream));
    ns.norms = (double *)((char *)ns.counter + 16);
    ns.capacity = slots;
    IPTGB_CUDA(cudaMemsetAsync(ns.counter, 0, 16, stream));
    return IPT_CUDA_SUCCESS;
}

int SolveScratch::arm_history(int steps, double tol, cudaStream_t stream)
{
    if (steps > ns.hist_cap) {
        if (ns.hist != nullptr) cudaFreeAsync(ns.hist, stream);
        ns.hist = nullptr;
        ns.hist_cap = 0;
        IPTGB_CUDA(cudaMallocAsync((void **)&ns.hist, 2 * (size_t)steps * sizeof(double), stream));
        ns.hist_cap = steps;
    }
    IPTGB_CUDA(cudaMemsetAsync(ns.hist, 0, 2 * (size_t)steps * sizeof(double), stream));
    ns.step = 0;
    ns.stop_tol = tol;
    return IPT_CUDA_SUCCESS;
}

int SolveScratch::read_history(int count, int *stopped_at, double *rel, cudaStream_t stream)
{
    host_hist.resize(2 * (size_t)count);
    if (count > 0) {
        IPTGB_CUDA(cudaMemcpyAsync(host_hist.data(), ns.hist, 2 * (size_t)count * sizeof(double),
                                   cudaMemcpyDeviceToHost, stream));
    }
    IPTGB_CUDA(cudaStreamSynchronize(stream));
    *stopped_at = -1;
    *rel = NAN;
    const double t2 = ns.stop_tol * ns.stop_tol;
    for (int i = 0; i < count; ++i) {
        const double d2 = host_hist[2 * (size_t)i], x2 = host_hist[2 * (size_t)i + 1];
        *rel = sqrt(d2) / sqrt(x2);
        if (x2 > 0.0 && d2 <= t2 * x2) {
            *stopped_at = i;
            break;
        }
    }
    return IPT_CUDA_SUCCESS;
}

void SolveScratch::release(cudaStream_t stream)
{
    if (ns.partials != nullptr) {
        cudaFreeAsync(ns.partials, stream);
    }
    if (ns.counter != nullptr) {
        cudaFreeAsync(ns.counter, stream);
    }
    if (ns.hist != nullptr) {
        cudaFreeAsync(ns.hist, stream);
    }
    ns = NormScratch();
}

int run_plain_ipt(Fp64Operator &op, int n, int k, const double *d, int maxiter, double tol,
                  int use_tol, double *X_a, double *X_b, double **X_final,
                  int *iterations_done, double *fixed_point_residual, SolveScratch *scratch,
                  cudaStream_t stream)
{
    double *x = X_a;
    double *y = X_b;
    int done = 0;
    double fpres = NAN;
    (void)n;
    (void)k;
    for (int iter = 0; iter < maxiter; ++iter) {
        IPTGB_CHECK(op.step(x, y, d, use_tol, &scratch->ns));
        done = iter + 1;
        if (use_tol) {
            IPTGB_CUDA(cudaMemcpyAsync(scratch->host_norms, scratch->ns.norms,
                                       2 * sizeof(double), cudaMemcpyDeviceToHost, stream));
            IPTGB_CUDA(cudaStreamSynchronize(stream));
            const double delta_norm = scratch->host_norms[0];
            const double current_norm = scratch->host_norms[1];
            if (current_norm <= 0.0 || !isfinite(current_norm)) {
                return IPT_CUDA_INVALID_ARGUMENT;
            }
            fpres = delta_norm / current_norm;
            double *t = x;
            x = y;
            y = t;
            if (fpres <= tol) {
                break;
            }
        } else {
            double *t = x;
            x = y;
            y = t;
        }
    }
    *X_final = x;
    *iterations_done = done;
    *fixed_point_residual = fpres;
    return IPT_CUDA_SUCCESS;
}

}  // namespace iptgb
