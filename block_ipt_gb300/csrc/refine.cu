// refine.cu - mixed-precision iterative refinement of the IPT fixed point.
//
// The IPT map F(X) = E + G o (Delta X - X diag(Delta X)) has the k lowest
// eigenvectors (normalised X_jj = 1) as its fixed point.  This driver reaches
// it to an FP64 eigen-residual with few FP64 products:
//
//   X  <- low-precision IPT (tensor cores), or the identity start
//   loop:
//     HX <- H X in FP64 (one accurate block product)
//     R0 <- F(X) - X in FP64 (the defect), c_j = (Delta X)_jj, and the exact
//           eigen-residuals r_ij = (d_j - d_i) R0_ij (r_jj = 0) of X with
//           lambda_j = (H X)_jj = d_j + c_j
//     stop when max_j ||r_j|| / (max(1,||H||_inf) max(1,||x_j||)) <= tol
//     plain FP64:  X <- X + R0            (the reference's IPT step)
//     mixed:       X <- X + delta, delta from the correction equation
//                  delta = R0 + G o (Delta delta - X diag(Delta delta)
//                                    - delta diag(c + diag(Delta delta)))
//                  iterated on the tensor cores (lowp.h refine_*)
//   Rayleigh-Ritz on span(X) with the HX of the last product (CholQR2 with
//   FP64 Gram matrices, FP64 projected matrix and eigensolve, FP64
//   residuals): unit-norm Ritz vectors in ascending order.
//
// This is the reference's mixed scheme (low-precision IPT, then FP64 IPT
// refinement: IPT_C_GPU/src/mixed_precision/ipt_mixed_precision_cuda.cu:
// 832-1003, 1153-1225) with the FP64 refinement iterations replaced by
// low-precision correction solves against FP64 defects.  If the fixed point
// stops improving (an IPT map that does not contract, e.g. near-degenerate
// target clusters) the caller falls back to the Davidson driver.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "block_ops.h"
#include "block_solver.h"
#include "common.cuh"
#include "lowp.h"
#include "reduce.cuh"

namespace iptgb {

namespace {

constexpr int kDefectRows = 2048;

// Per (row chunk, column): R0 = F(X) - X and partial sums of ||r||^2,
// ||x||^2 and max |R0| (see file header).  Partials [chunk][col][3].
// lowp_rhs: R0 only feeds the low-precision correction solve (converted to
// FP32 there), so 1/gap is taken in FP32 instead of an FP64 division, which
// GB300 runs as a long sequence on its slow FP64 pipe; the residual norms
// stay exact FP64 (r = gap * R0 needs no division).  The plain FP64 path adds
// R0 to X and keeps the exact quotient.
__global__ void defect_partial_kernel(const double *__restrict__ X, const double *__restrict__ HX,
                                      const double *__restrict__ d, int n, int k,
                                      double *__restrict__ R0, double *__restrict__ c_out,
                                      double *__restrict__ P, int lowp_rhs)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    __shared__ double smax[32];
    const int j = blockIdx.y;
    const size_t dj = (size_t)j + (size_t)j * n;
    const double c = HX[dj] - d[j] * X[dj];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        c_out[j] = c;
    }
    const int r0 = blockIdx.x * kDefectRows;
    const int r1 = min(n, r0 + kDefectRows);
    double rs = 0.0, xs = 0.0, mx = 0.0;
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const size_t idx = (size_t)i + (size_t)j * n;
        const double x = X[idx];
        double rdef = 0.0;
        if (i != j) {
            const double gap = d[j] - d[i];
            const double a = HX[idx] - d[i] * x;
            double r;
            if (lowp_rhs) {
                r = (a - x * c) - gap * x;
                const double g =
                    (isfinite(gap) && gap != 0.0) ? (double)__frcp_rn((float)gap) : NAN;
                rdef = r * g;
            } else {
                const double g = (isfinite(gap) && gap != 0.0) ? 1.0 / gap : NAN;
                rdef = (a - x * c) * g - x;
                r = gap * rdef;
            }
            rs = fma(r, r, rs);
            mx = fmax(mx, fabs(rdef));
        }
        R0[idx] = rdef;
        xs = fma(x, x, xs);
    }
    const double2 t = block_sum2(rs, xs);
    for (int off = 16; off > 0; off >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) mx = fmax(mx, smax[w]);
        double *out = P + ((size_t)blockIdx.x * k + j) * 3;
        out[0] = t.x;
        out[1] = t.y;
        out[2] = mx;
    }
}

// Per column: the scaled residual, the largest |R0_ij| and the power-of-two
// scale sigma_j = 2^floor(log2(1024 / max_i |R0_ij|)) (1 for a zero or
// non-finite column, clamped to [1e-20, 1e20]) that brings the correction's
// right-hand side into the low-precision operand's range.  floor(log2(x)) is
// read from the exponent bits of x, exactly.
__global__ void defect_finish_kernel(const double *__restrict__ P, int chunks, int k, double hnorm,
                                     double *__restrict__ scaled, double *__restrict__ colmax,
                                     float *__restrict__ sigma)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k) return;
    double rs = 0.0, xs = 0.0, mx = 0.0;
    for (int b = 0; b < chunks; ++b) {
        const double *q = P + ((size_t)b * k + j) * 3;
        rs += q[0];
        xs += q[1];
        mx = fmax(mx, q[2]);
    }
    scaled[j] = sqrt(rs) / (fmax(1.0, hnorm) * fmax(1.0, sqrt(xs)));
    colmax[j] = mx;
    float sg = 1.0f;
    if (mx > 0.0 && isfinite(mx)) {
        const double x = 1024.0 / mx;
        const int e = (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7FF) - 1023;
        sg = (float)ldexp(1.0, e);
    }
    sigma[j] = fminf(fmaxf(sg, 1e-20f), 1e20f);
}

// Steps launched past a correction check before the host waits for its
// norms (each step ~25 us at n = 8192; a host round trip ~40 us).
constexpr int kLookahead = 2;

// Largest check interval of a correction solve with Anderson mixing.
constexpr int kMixedCheck = 4;

// Per host thread: a small page-locked buffer the check norms are copied
// into, so that the copy is asynchronous (allocated on the thread's first
// refinement and kept for the life of the process).
double *pinned_check_norms()
{
    static thread_local double *buf = nullptr;
    if (buf == nullptr) {
        void *p = nullptr;
        if (cudaMallocHost(&p, 4 * sizeof(double)) != cudaSuccess) return nullptr;
        buf = static_cast<double *>(p);
    }
    return buf;
}

__global__ void add_kernel(double *__restrict__ X, const double *__restrict__ D, size_t count)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count) X[e] += D[e];
}

float ev_ms(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

}  // namespace

int refine_solve(const RefineInput &in, double *X_out, double *values_out, IPTBlockReport *rep,
                 cudaStream_t s, bool *converged_out, double *X_fallback)
{
    const int n = in.n;
    const int k = in.k;
    const size_t elems = (size_t)n * k;
    const double tol = in.opt.residual_tol > 0.0 ? in.opt.residual_tol : 1e-8;
    *converged_out = false;
    memset(rep, 0, sizeof(*rep));
    rep->n = n;
    rep->k = k;
    rep->matrix_norm_inf = in.hnorm;
    rep->max_scaled_residual = NAN;
    rep->ipt_fixed_point_residual = NAN;

    BlockOps ops;
    ops.stream = s;
    ops.sms = device_sm_count();
    // the Rayleigh-Ritz products of the converged block in double-float
    // (about 48 bits: far below the 1e-8 residual and the 1e-10 ||H||
    // eigenvalue accuracy they serve)
    ops.df_products = true;
    const int chunks = (n + kDefectRows - 1) / kDefectRows;
    DeviceBuffer<double> X, HX, R0, Q, HQ, small;
    IPTGB_CHECK(X.alloc(elems, s));
    IPTGB_CHECK(HX.alloc(elems, s));
    IPTGB_CHECK(R0.alloc(elems, s));
    IPTGB_CHECK(Q.alloc(elems, s));
    IPTGB_CHECK(HQ.alloc(elems, s));
    const size_t kk = (size_t)k * k;
    IPTGB_CHECK(small.alloc(4 * kk + 8 * (size_t)k + (size_t)chunks * k * 3 + 64, s));
    double *G = small.ptr;
    double *Rinv = G + kk;
    double *T = Rinv + kk;
    double *Z = T + kk;
    double *c = Z + kk;
    double *scaled = c + k;
    double *colmax = scaled + k;
    double *theta = colmax + k;
    double *rnorm = theta + k;
    float *sigma = reinterpret_cast<float *>(rnorm + k);  // k floats
    int *st_dev = reinterpret_cast<int *>(rnorm + 2 * k);
    double *P = rnorm + 3 * k;
    std::vector<double> h_scaled((size_t)k);
    int h_status = 0;

    cudaEvent_t ev[4];
    for (auto &e : ev) IPTGB_CUDA(cudaEventCreate(&e));
    struct Guard {
        cudaEvent_t *e;
        ~Guard()
        {
            for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]);
        }
    } guard{ev};
    IPTGB_CUDA(cudaEventRecord(ev[0], s));
    trace_mark("refine:start", s);

    // ---- initial block ---------------------------------------------------------
    if (in.ipt != nullptr) {
        int it = 0;
        double fp = NAN;
        long long mv = 0;
        IPTGB_CHECK(in.ipt->run(k, in.opt.ipt_maxiter, in.opt.ipt_tol,
                                std::max(1, in.opt.ipt_check_every), X.ptr, &it, &fp, &mv));
        rep->ipt_iterations = it;
        rep->ipt_fixed_point_residual = fp;
        rep->lowp_matvecs += mv;
    } else {
        IPTGB_CHECK(launch_set_identity(X.ptr, n, k, s));
    }
    IPTGB_CUDA(cudaEventRecord(ev[1], s));
    trace_mark("refine:ipt_done", s);

    // ---- outer refinement ---------------------------------------------------------
    const int max_outer = std::max(1, in.max_outer);
    double best = INFINITY, prev = INFINITY;
    int stalls = 0;
    int outer = 0;
    bool conv = false;
    SolveScratch scratch;
    IPTGB_CHECK(scratch.init(elems, s));
    double *check_norms = pinned_check_norms();
    if (check_norms == nullptr) return IPT_CUDA_ALLOCATION_FAILED;
    cudaEvent_t check_ev = nullptr;
    IPTGB_CUDA(cudaEventCreateWithFlags(&check_ev, cudaEventDisableTiming));
    struct EventGuard {
        cudaEvent_t e;
        ~EventGuard() { cudaEventDestroy(e); }
    } check_guard{check_ev};
    for (; outer < max_outer; ++outer) {
        trace_mark("refine:defect", s);
        IPTGB_CHECK(in.apply->apply(X.ptr, k, HX.ptr));
        trace_mark("refine:defect_product_done", s);
        rep->fp64_matvecs += k;
        IPTGB_CHECK(launch_pdl(defect_partial_kernel, dim3(chunks, k), dim3(256), 0, s,
                               (const double *)X.ptr, (const double *)HX.ptr, in.d, n, k, R0.ptr,
                               c, P, in.lowp != nullptr ? 1 : 0));
        IPTGB_CHECK(launch_pdl(defect_finish_kernel, dim3(blocks_for(k)), dim3(kThreads), 0, s,
                               (const double *)P, chunks, k, in.hnorm, scaled, colmax, sigma));
        IPTGB_CUDA(cudaMemcpyAsync(h_scaled.data(), scaled, (size_t)k * sizeof(double),
                                   cudaMemcpyDeviceToHost, s));
        IPTGB_CUDA(cudaStreamSynchronize(s));
        double mx = 0.0;
        for (int j = 0; j < k; ++j) {
            const double r = h_scaled[(size_t)j];
            mx = isfinite(r) ? std::max(mx, r) : INFINITY;
        }
        if (!isfinite(mx)) {
            break;  // the iterate blew up: hand over to Davidson
        }
        best = std::min(best, mx);
        if (mx <= tol) {
            conv = true;
            break;
        }
        if (outer + 1 == max_outer) {
            break;
        }
        // stall detection: the map no longer contracts.  A mixed step should
        // gain about the operand precision; a plain IPT step gains the
        // contraction factor of the map, which can be close to one.
        const double gain = in.lowp != nullptr ? 0.5 : 0.999;
        stalls = mx > gain * prev ? stalls + 1 : 0;
        if (mx > 2.0 * prev || mx > 1e3 * best) {
            break;  // diverging: the map does not contract at these targets
        }
        prev = mx;
        if (stalls >= (in.lowp != nullptr ? 2 : 4)) {
            break;
        }
        if (in.lowp != nullptr) {
            // sigma: written by defect_finish_kernel
            trace_mark("refine:correction", s);
            IPTGB_CHECK(in.lowp->refine_begin(R0.ptr, X.ptr, c, sigma));
            // device-side stop at inner_tol; the history is read every `check` steps
            const bool device_stop = lowp_device_stop(*in.lowp);
            if (device_stop) {
                IPTGB_CHECK(scratch.arm_history(std::max(1, in.inner_maxiter), in.inner_tol, s));
            }
            // with Anderson mixing the solve converges in about half the
            // steps, so its checks come at least every kMixedCheck steps
            const int check = in.mixing ? std::max(1, std::min(in.opt.ipt_check_every, kMixedCheck))
                                        : std::max(1, in.opt.ipt_check_every);
            int ran = 0;
            // A check's norms are copied to pinned memory and the next
            // kLookahead steps are launched before the host waits for them,
            // so the GPU keeps iterating through the host's round trip; a
            // correction that met inner_tol at the check takes those steps
            // too (they only refine it further).
            int pending = -1;
            for (int i = 0; i < in.inner_maxiter; ++i) {
                const int want = ((i + 1) % check == 0) || i + 1 == in.inner_maxiter;
                IPTGB_CHECK(in.lowp->refine_step(device_stop ? 0 : want, &scratch.ns));
                ran = i + 1;
                if (want && pending >= 0) {
                    // a check still in flight (check interval <= kLookahead):
                    // judge it before its norms are overwritten
                    IPTGB_CUDA(cudaEventSynchronize(check_ev));
                    pending = -1;
                    const double rel = check_norms[0] / check_norms[1];
                    if (!(rel > in.inner_tol)) break;  // met (or non-finite): stop
                }
                if (want) {
                    trace_mark("refine:correction_check", s);
                    if (device_stop) {
                        int stopped_at = -1;
                        double rel = NAN;
                        IPTGB_CHECK(scratch.read_history(i + 1, &stopped_at, &rel, s));
                        if (stopped_at >= 0) {
                            ran = stopped_at + 1;
                            break;
                        }
                        if (!(rel > in.inner_tol)) break;  // non-finite: stop
                        continue;
                    }
                    IPTGB_CUDA(cudaMemcpyAsync(check_norms, scratch.ns.norms, 2 * sizeof(double),
                                               cudaMemcpyDeviceToHost, s));
                    IPTGB_CUDA(cudaEventRecord(check_ev, s));
                    pending = i;
                }
                if (pending >= 0 && (i - pending >= kLookahead || i + 1 == in.inner_maxiter)) {
                    IPTGB_CUDA(cudaEventSynchronize(check_ev));
                    pending = -1;
                    const double rel = check_norms[0] / check_norms[1];
                    if (!(rel > in.inner_tol)) break;  // met (or non-finite): stop
                }
            }
            rep->lowp_matvecs += (long long)ran * k;
            IPTGB_CHECK(in.lowp->refine_apply(X.ptr));
        } else {
            add_kernel<<<blocks_for(elems), kThreads, 0, s>>>(X.ptr, R0.ptr, elems);
            IPTGB_LAUNCH();
        }
        ++rep->davidson_steps;  // refinement steps
    }
    scratch.release(s);
    rep->restarts = outer;
    IPTGB_CUDA(cudaEventRecord(ev[2], s));
    trace_mark("refine:rayleigh_ritz", s);
    if (!conv) {
        rep->max_scaled_residual = best;
        IPTGB_CUDA(cudaMemcpyAsync(X_fallback, X.ptr, elems * sizeof(double),
                                   cudaMemcpyDeviceToDevice, s));
        IPTGB_CUDA(cudaStreamSynchronize(s));
        ops.release();
        return IPT_CUDA_SUCCESS;
    }

    // ---- Rayleigh-Ritz on span(X) with the FP64 HX of the last product ----------
    // CholQR2 (the reference orthonormalises with an FP32 QR and one
    // Cholesky repair pass, IPT_C_GPU/mixed/ipt_rayleigh_mixed_mpqr_cuda.cu:
    // 319-360).  The second pass only repairs the orthogonality the first
    // leaves, about cond(G) * eps for the column-scaled Gram matrix G: with
    // the bound of that condition number at most kCholQr1Cond the first pass
    // is kept (an IPT block near convergence is close to orthogonal).
    constexpr double kCholQr1Cond = 100.0;
    double *cond_dev = P + (size_t)chunks * k * 3;  // spare tail of `small`
    auto cholqr_pair = [&](double *A, double *HA, double *A2, double *HA2, double *cond_out,
                           double *h_cond) -> int {
        IPTGB_CHECK(ops.gram(A, n, k, A, n, k, n, G, k));
        // double-float factor: the Rayleigh-Ritz basis is well conditioned
        // here (the second pass runs otherwise)
        IPTGB_CHECK(ops.chol_inverse(G, k, Rinv, st_dev, cond_out, true));
        IPTGB_CHECK(ops.tall_gemm(A, n, Rinv, k, A2, n, n, k, k));
        IPTGB_CHECK(ops.tall_gemm(HA, n, Rinv, k, HA2, n, n, k, k));
        IPTGB_CUDA(cudaMemcpyAsync(&h_status, st_dev, sizeof(int), cudaMemcpyDeviceToHost, s));
        if (cond_out != nullptr) {
            IPTGB_CUDA(cudaMemcpyAsync(h_cond, cond_out, sizeof(double), cudaMemcpyDeviceToHost,
                                       s));
        }
        IPTGB_CUDA(cudaStreamSynchronize(s));
        return h_status < 0 ? IPT_CUDA_INVALID_ARGUMENT : IPT_CUDA_SUCCESS;
    };
    double h_cond = INFINITY;
    IPTGB_CHECK(cholqr_pair(X.ptr, HX.ptr, Q.ptr, HQ.ptr, k <= 32 ? cond_dev : nullptr, &h_cond));
    // basis B / HB, output O / HO
    double *B = Q.ptr, *HB = HQ.ptr, *O = X.ptr, *HO = HX.ptr;
    trace_mark("refine:cholqr1_done", s);
    if (!(h_cond <= kCholQr1Cond)) {
        trace_mark("refine:cholqr2", s);
        IPTGB_CHECK(cholqr_pair(Q.ptr, HQ.ptr, X.ptr, HX.ptr, nullptr, nullptr));
        B = X.ptr;
        HB = HX.ptr;
        O = Q.ptr;
        HO = HQ.ptr;
    }
    IPTGB_CHECK(ops.gram(B, n, k, HB, n, k, n, T, k));
    trace_mark("refine:projected_eig", s);
    IPTGB_CHECK(ops.symmetric_eig(T, k, theta, Z, st_dev));
    trace_mark("refine:projected_eig_done", s);
    IPTGB_CHECK(ops.tall_gemm(B, n, Z, k, O, n, n, k, k));
    IPTGB_CHECK(ops.tall_gemm(HB, n, Z, k, HO, n, n, k, k));
    IPTGB_CHECK(ops.residuals(O, HO, theta, n, k, n, in.hnorm, R0.ptr, rnorm, scaled));
    IPTGB_CUDA(cudaMemcpyAsync(h_scaled.data(), scaled, (size_t)k * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaMemcpyAsync(X_out, O, elems * sizeof(double), cudaMemcpyDeviceToDevice, s));
    IPTGB_CUDA(cudaMemcpyAsync(values_out, theta, (size_t)k * sizeof(double),
                               cudaMemcpyDeviceToDevice, s));
    IPTGB_CUDA(cudaEventRecord(ev[3], s));
    trace_mark("refine:end", s);
    IPTGB_CUDA(cudaStreamSynchronize(s));
    double mx = 0.0;
    for (int j = 0; j < k; ++j) {
        const double r = h_scaled[(size_t)j];
        mx = isfinite(r) ? std::max(mx, r) : INFINITY;
    }
    ops.release();
    rep->max_scaled_residual = mx;
    rep->converged = mx <= tol ? 1 : 0;
    rep->basis_cols = k;
    rep->ipt_ms = ev_ms(ev[0], ev[1]);
    rep->davidson_ms = ev_ms(ev[1], ev[2]);
    rep->rayleigh_ritz_ms = ev_ms(ev[2], ev[3]);
    rep->total_ms = ev_ms(ev[0], ev[3]);
    *converged_out = rep->converged == 1;
    if (!*converged_out) {
        IPTGB_CUDA(cudaMemcpyAsync(X_fallback, O, elems * sizeof(double),
                                   cudaMemcpyDeviceToDevice, s));
        IPTGB_CUDA(cudaStreamSynchronize(s));
    }
    return IPT_CUDA_SUCCESS;
}

}  // namespace iptgb
