// abi_rayleigh.cu - the reference's Rayleigh-mixed entry point
// (IPT_C_GPU/src/mixed_precision/ipt_rayleigh_mixed_cuda.cu:19-41,274-400;
// the mixed-CholQR twin IPT_C_GPU/mixed/ipt_rayleigh_mixed_mpqr_cuda.cu:
// 169-386,406-538 exports the same symbol).
//
//   1. TF32 IPT of the k lowest diagonal positions on the tensor cores
//      (tcgen05, Delta with its diagonal zeroed) until the fixed-point
//      residual reaches tf32_tol;
//   2. an orthonormal basis Q of that block: CholQR2 with FP64 Gram matrices
//      (the mixed-CholQR twin's FP64 Gram + Cholesky), then the column signs
//      a Householder QR gives (below), so that Q equals the reference's
//      geqrf/orgqr factor, and the mixed-CholQR twin's Q = X (L^T R)^{-1}
//      whose R carries the same signs;
//   3. B = Q^T (H Q) in FP64, symmetrised ((B + B^T) / 2,
//      ipt_rayleigh_mixed_cuda.cu:84-106);
//   4. the FP64 plain IPT on the k x k matrix B to fp64_tol (the reference
//      calls its own ipt_cuda_device_tol there, :358), giving Z with
//      Z_jj = 1 and the values (B Z)_jj;
//   5. the vectors Q Z.
//
// Householder signs: for X = Q_c R_c with R_c's diagonal positive, LAPACK's
// Householder QR gives Q_h = Q_c S with S = diag(sign(R_h,jj)).  Each
// reflector maps the current column x to beta e_1 with beta = -sign(x_1)
// ||x|| (dlarfg), except when x has a single entry (no reflection, beta =
// x_1).  The current column of a Householder QR of Q_c itself is the Schur
// complement of the LU elimination of Q_c - S restricted to its top k x k
// block (the Householder reconstruction of Ballard, Demmel, Grigori,
// Jacobsen, Knight and Nguyen, IPDPS 2014), and scaling the columns of X by
// the positive R_c changes none of the signs, so S follows from a k x k
// elimination on the host: s_i = -sign(pivot_i) (the last row of a square
// block: +sign), pivot_i -= s_i, eliminate.
#include <cublas_v2.h>
#include <math.h>

#include <climits>
#include <memory>
#include <vector>

#include "../../include/ipt_block.h"
#include "block_ops.h"
#include "common.cuh"
#include "ipt_plain.h"
#include "lowp.h"
#include "rayleigh.h"

#define IPT_API extern "C" __attribute__((visibility("default")))

using namespace iptgb;

namespace iptgb {
int dense_plain_device_entry(const double *dH, int n, int k, const double *dX0, int maxiter,
                             double tol, int use_tol, double *X_out, double *values_out,
                             int *iterations_done, double *fixed_point_residual,
                             cudaStream_t stream);
}

namespace {

// Largest k: the Cholesky-inverse kernel of the CholQR holds two k x k FP64
// matrices in one CTA's shared memory.
constexpr int kRayleighMaxK = 112;

void reset_rayleigh(IPTRayleighMixedCudaDeviceResult *r)
{
    r->n = 0;
    r->k = 0;
    r->tf32_iterations = 0;
    r->fp64_iterations = 0;
    r->tf32_time_sec = NAN;
    r->orthogonalize_time_sec = NAN;
    r->rayleigh_transform_time_sec = NAN;
    r->fp64_time_sec = NAN;
    r->backtransform_time_sec = NAN;
    r->total_time_sec = NAN;
    r->tf32_fixed_point_residual = NAN;
    r->fp64_fixed_point_residual = NAN;
    r->d_vectors = nullptr;
    r->d_values = nullptr;
}

__global__ void symmetrize_kernel(double *B, int k)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= k * k) return;
    const int i = e % k, j = e / k;
    if (i < j) {
        const double a = 0.5 * (B[i + (size_t)j * k] + B[j + (size_t)i * k]);
        B[i + (size_t)j * k] = a;
        B[j + (size_t)i * k] = a;
    }
}

// Column signs of the Householder QR from the top k x k block T of the
// CholQR factor (column-major, ld k), rows = n.
void householder_signs(std::vector<double> T, int k, int n, std::vector<double> *s)
{
    s->assign((size_t)k, 1.0);
    for (int i = 0; i < k; ++i) {
        double &p = T[(size_t)i + (size_t)i * k];
        const double sg = p > 0.0 ? 1.0 : (p < 0.0 ? -1.0 : 0.0);
        double si;
        if (i == n - 1) {
            si = sg != 0.0 ? sg : 1.0;
        } else {
            si = sg != 0.0 ? -sg : -1.0;
        }
        (*s)[(size_t)i] = si;
        p -= si;
        if (p == 0.0) continue;
        for (int r = i + 1; r < k; ++r) {
            const double l = T[(size_t)r + (size_t)i * k] / p;
            if (l == 0.0) continue;
            for (int c = i + 1; c < k; ++c) {
                T[(size_t)r + (size_t)c * k] -= l * T[(size_t)i + (size_t)c * k];
            }
        }
    }
}

double seconds_between(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    return 1e-3 * ms;
}

// CholQR: dst = B R^{-1} with G = B^T B = R^T R in FP64.
int cholqr_fp64(BlockOps &ops, const double *B, int n, int k, double *dst, double *G,
                double *Rinv, int *st_dev, cudaStream_t s)
{
    IPTGB_CHECK(ops.gram(B, n, k, B, n, k, n, G, k));
    IPTGB_CHECK(ops.chol_inverse(G, k, Rinv, st_dev, nullptr, false));
    IPTGB_CHECK(ops.tall_gemm(B, n, Rinv, k, dst, n, n, k, k));
    int h = 0;
    IPTGB_CUDA(cudaMemcpyAsync(&h, st_dev, sizeof(int), cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    // a shifted factorisation would not be an orthonormal basis of the block
    return h == 0 ? IPT_CUDA_SUCCESS : IPT_CUDA_INVALID_ARGUMENT;
}

}  // namespace

namespace iptgb {

// Q = the orthonormal basis of X0 (n x k) with the column signs of LAPACK's
// Householder QR: CholQR2 in FP64, then the signs from the top k x k block.
// X0 is overwritten.
int householder_basis(BlockOps &ops, double *X0, int n, int k, double *Q, cudaStream_t s)
{
    DeviceBuffer<double> G, Rinv, sg;
    DeviceBuffer<int> idx, st;
    IPTGB_CHECK(G.alloc((size_t)k * k, s));
    IPTGB_CHECK(Rinv.alloc((size_t)k * k, s));
    IPTGB_CHECK(st.alloc(1, s));
    IPTGB_CHECK(cholqr_fp64(ops, X0, n, k, Q, G.ptr, Rinv.ptr, st.ptr, s));
    IPTGB_CHECK(cholqr_fp64(ops, Q, n, k, X0, G.ptr, Rinv.ptr, st.ptr, s));
    std::vector<double> top((size_t)k * k);
    IPTGB_CUDA(cudaMemcpy2DAsync(top.data(), (size_t)k * sizeof(double), X0,
                                 (size_t)n * sizeof(double), (size_t)k * sizeof(double), (size_t)k,
                                 cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    std::vector<double> signs;
    householder_signs(top, k, n, &signs);
    std::vector<int> id((size_t)k);
    for (int j = 0; j < k; ++j) id[(size_t)j] = j;
    IPTGB_CHECK(sg.alloc((size_t)k, s));
    IPTGB_CHECK(idx.alloc((size_t)k, s));
    IPTGB_CUDA(cudaMemcpyAsync(sg.ptr, signs.data(), (size_t)k * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    IPTGB_CUDA(cudaMemcpyAsync(idx.ptr, id.data(), (size_t)k * sizeof(int),
                               cudaMemcpyHostToDevice, s));
    IPTGB_CHECK(ops.gather_columns(X0, n, idx.ptr, sg.ptr, n, k, Q, n));
    // the host vectors must outlive the asynchronous copies
    IPTGB_CUDA(cudaStreamSynchronize(s));
    return IPT_CUDA_SUCCESS;
}

// B = (Q^T H Q + (Q^T H Q)^T) / 2 in FP64 (k x k), H column-major n x n.
int projected_matrix(BlockOps &ops, const double *dH, int n, const double *Q, int k, double *B,
                     cudaStream_t s)
{
    const size_t elems = (size_t)n * k;
    DeviceBuffer<double> AQ, P;
    IPTGB_CHECK(AQ.alloc(elems, s));
    const int S = dense64_split_for(n, k, ops.sms);
    IPTGB_CHECK(P.alloc((size_t)S * elems, s));
    IPTGB_CHECK(launch_dense64_partial(dH, n, n, Q, n, k, P.ptr, S, s));
    IPTGB_CHECK(launch_sum_partials(P.ptr, S, elems, AQ.ptr, s));
    IPTGB_CHECK(ops.gram(Q, n, k, AQ.ptr, n, k, n, B, k));
    symmetrize_kernel<<<(k * k + 255) / 256, 256, 0, s>>>(B, k);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

}  // namespace iptgb

namespace {

int rayleigh_run(const double *dH, int n, int k, double tf32_tol, int tf32_maxiter,
                 double fp64_tol, int fp64_maxiter, cudaStream_t s,
                 IPTRayleighMixedCudaDeviceResult *out)
{
    cudaEvent_t ev[10] = {};
    for (auto &e : ev) IPTGB_CUDA(cudaEventCreate(&e));
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard()
        {
            for (int i = 0; i < 10; ++i) cudaEventDestroy(e[i]);
        }
    } guard{ev};
    const size_t elems = (size_t)n * k;
    DeviceBuffer<double> d, X0, Q, B, Z;
    IPTGB_CHECK(d.alloc((size_t)n, s));
    IPTGB_CHECK(X0.alloc(elems, s));

    // 1. TF32 IPT on the tensor cores (ipt_tf32_initial_device_tol)
    IPTGB_CUDA(cudaEventRecord(ev[0], s));
    IPTGB_CHECK(launch_extract_diagonal(dH, n, n, d.ptr, s));
    {
        int status = IPT_CUDA_SUCCESS;
        std::unique_ptr<LowpDenseOperator> op(make_lowp_dense_operator(dH, n, kLowpTF32, s,
                                                                       &status));
        if (!op) return status != IPT_CUDA_SUCCESS ? status : IPT_CUDA_CUDA_ERROR;
        IPTGB_CHECK(op->set_width(k));
        IPTGB_CHECK(op->reset_identity(d.ptr));
        long long mv = 0;
        IPTGB_CHECK(run_lowp_ipt(*op, n, k, tf32_maxiter, tf32_tol, 1, X0.ptr,
                                 &out->tf32_iterations, &out->tf32_fixed_point_residual, &mv, s,
                                 false));
    }
    IPTGB_CUDA(cudaEventRecord(ev[1], s));

    // 2. orthonormal basis with the Householder column signs
    BlockOps ops;
    ops.stream = s;
    ops.sms = device_sm_count();
    struct OpsGuard {
        BlockOps *o;
        ~OpsGuard() { o->release(); }
    } og{&ops};
    IPTGB_CUDA(cudaEventRecord(ev[2], s));
    IPTGB_CHECK(Q.alloc(elems, s));
    IPTGB_CHECK(householder_basis(ops, X0.ptr, n, k, Q.ptr, s));
    IPTGB_CUDA(cudaEventRecord(ev[3], s));

    // 3. B = sym(Q^T H Q) in FP64
    IPTGB_CUDA(cudaEventRecord(ev[4], s));
    IPTGB_CHECK(B.alloc((size_t)k * k, s));
    IPTGB_CHECK(projected_matrix(ops, dH, n, Q.ptr, k, B.ptr, s));
    IPTGB_CUDA(cudaEventRecord(ev[5], s));

    // 4. FP64 IPT on the k x k matrix
    double *vals = nullptr, *vecs = nullptr;
    IPTGB_CHECK(Z.alloc((size_t)k * k, s));
    IPTGB_CUDA(cudaMalloc((void **)&vals, (size_t)k * sizeof(double)));
    if (cudaMalloc((void **)&vecs, elems * sizeof(double)) != cudaSuccess) {
        cudaFree(vals);
        return IPT_CUDA_CUDA_ERROR;
    }
    auto fail = [&](int code) {
        cudaStreamSynchronize(s);
        cudaFree(vals);
        cudaFree(vecs);
        return code;
    };
    cudaEventRecord(ev[6], s);
    int status = dense_plain_device_entry(B.ptr, k, k, nullptr, fp64_maxiter, fp64_tol, 1, Z.ptr,
                                          vals, &out->fp64_iterations,
                                          &out->fp64_fixed_point_residual, s);
    if (status != IPT_CUDA_SUCCESS) return fail(status);
    cudaEventRecord(ev[7], s);

    // 5. vectors = Q Z
    cudaEventRecord(ev[8], s);
    status = ops.tall_gemm(Q.ptr, n, Z.ptr, k, vecs, n, n, k, k);
    if (status != IPT_CUDA_SUCCESS) return fail(status);
    cudaEventRecord(ev[9], s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return fail(IPT_CUDA_CUDA_ERROR);
    out->tf32_time_sec = seconds_between(ev[0], ev[1]);
    out->orthogonalize_time_sec = seconds_between(ev[2], ev[3]);
    out->rayleigh_transform_time_sec = seconds_between(ev[4], ev[5]);
    out->fp64_time_sec = seconds_between(ev[6], ev[7]);
    out->backtransform_time_sec = seconds_between(ev[8], ev[9]);
    out->total_time_sec = out->tf32_time_sec + out->orthogonalize_time_sec +
                          out->rayleigh_transform_time_sec + out->fp64_time_sec +
                          out->backtransform_time_sec;
    out->n = n;
    out->k = k;
    out->d_vectors = vecs;
    out->d_values = vals;
    return IPT_CUDA_SUCCESS;
}

}  // namespace

IPT_API int ipt_block_householder_signs(const double *top, int k, int n, double *signs)
{
    if (top == nullptr || signs == nullptr || k <= 0 || n < k) return IPT_CUDA_INVALID_ARGUMENT;
    std::vector<double> s;
    householder_signs(std::vector<double>(top, top + (size_t)k * k), k, n, &s);
    for (int j = 0; j < k; ++j) signs[j] = s[(size_t)j];
    return IPT_CUDA_SUCCESS;
}

IPT_API void ipt_rayleigh_mixed_cuda_free_device_result(IPTRayleighMixedCudaDeviceResult *result)
{
    if (result == nullptr) return;
    cudaFree(result->d_vectors);
    cudaFree(result->d_values);
    reset_rayleigh(result);
}

IPT_API int ipt_rayleigh_mixed_tf32_cuda_device_tol(const double *d_matrix_col_major, int n,
                                                    int k, double tf32_tol, int tf32_maxiter,
                                                    double fp64_tol, int fp64_maxiter,
                                                    cublasHandle_t handle,
                                                    IPTRayleighMixedCudaDeviceResult *result)
{
    if (result == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    reset_rayleigh(result);
    if (d_matrix_col_major == nullptr || handle == nullptr || n <= 0 || k <= 0 || k > n ||
        !(tf32_tol > 0.0) || !(fp64_tol > 0.0) || tf32_maxiter <= 0 || fp64_maxiter <= 0) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    if ((size_t)n * (size_t)k > (size_t)INT_MAX || (size_t)k * (size_t)k > (size_t)INT_MAX) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    if (k > kRayleighMaxK) {
        fprintf(stderr, "ipt_gb300: ipt_rayleigh_mixed_tf32_cuda_device_tol supports k <= %d "
                        "(got %d)\n", kRayleighMaxK, k);
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = nullptr;
    if (cublasGetStream(handle, &s) != CUBLAS_STATUS_SUCCESS) {
        return IPT_CUDA_CUBLAS_ERROR;
    }
    const int status = rayleigh_run(d_matrix_col_major, n, k, tf32_tol, tf32_maxiter, fp64_tol,
                                    fp64_maxiter, s, result);
    if (status != IPT_CUDA_SUCCESS) {
        reset_rayleigh(result);
    }
    return status;
}
