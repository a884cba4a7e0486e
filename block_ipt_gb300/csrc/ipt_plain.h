// ipt_plain.h - FP64 plain-IPT drivers behind the reference ABI (internal).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "kernels.cuh"

namespace iptgb {

// One application of the IPT map X' = F(X) in FP64, plus (H X)_jj.
struct Fp64Operator {
    virtual ~Fp64Operator() = default;
    // Xn = F(X); with want_norms the step leaves ||Xn - X||_F, ||X||_F in ns->norms.
    virtual int step(const double *X, double *Xn, const double *d, int want_norms,
                     NormScratch *ns) = 0;
    // values[j] = (H X)_jj.
    virtual int diag_values(const double *X, double *values) = 0;
};

struct DenseFp64Operator final : Fp64Operator {
    const double *H = nullptr;
    long long ldh = 0;
    int n = 0, k = 0, S = 1;
    double *P = nullptr;  // S * n * k partial slices
    cudaStream_t stream = nullptr;
    int step(const double *X, double *Xn, const double *d, int want_norms,
             NormScratch *ns) override;
    int diag_values(const double *X, double *values) override;
};

struct CsrFp64Operator final : Fp64Operator {
    const int *row_ptr = nullptr;
    const int *col_ind = nullptr;
    const double *vals = nullptr;
    int n = 0, k = 0;
    double *Y = nullptr;  // n * k
    cudaStream_t stream = nullptr;
    int step(const double *X, double *Xn, const double *d, int want_norms,
             NormScratch *ns) override;
    int diag_values(const double *X, double *values) override;
};

// Scratch owned by a solve: norm reduction slots + readback.
struct SolveScratch {
    NormScratch ns;
    // the read-backs land in pageable memory: each is followed by a stream
    // synchronisation anyway, and a pinned allocation (with the device-wide
    // synchronisation of its release) per solve cost more than it saved
    double host_norms[2] = {0.0, 0.0};
    std::vector<double> host_hist;
    int init(size_t max_elems, cudaStream_t stream);
    void release(cudaStream_t stream);
    // zeroed history for up to `steps` steps with the device-side stop at tol
    int arm_history(int steps, double tol, cudaStream_t stream);
    // the first `count` history entries: *stopped_at = first step that met
    // the tolerance (-1: none), *rel = its ||delta||/||X|| (else the last
    // entry's); synchronises the stream
    int read_history(int count, int *stopped_at, double *rel, cudaStream_t stream);
};

// The reference's plain IPT loop (IPT_C_GPU/src/ipt_cuda.cu:1644-1703):
// X_a holds the start block on entry; on success *X_final points at the
// buffer (X_a or X_b) holding the returned block.  In tolerance mode the loop
// stops once ||F(X)-X||_F / ||X||_F <= tol and returns F(X).
int run_plain_ipt(Fp64Operator &op, int n, int k, const double *d, int maxiter, double tol,
                  int use_tol, double *X_a, double *X_b, double **X_final,
                  int *iterations_done, double *fixed_point_residual, SolveScratch *scratch,
                  cudaStream_t stream);

int device_sm_count();

}  // namespace iptgb
