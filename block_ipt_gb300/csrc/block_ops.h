// block_ops.h - FP64 block operations (CholQR, Rayleigh-Ritz, Davidson).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace iptgb {

// Launch wrapper bound to one stream; owns a reusable partial-sum buffer.
// All matrices are column-major doubles with explicit leading dimensions.
struct BlockOps {
    cudaStream_t stream = nullptr;
    int sms = 148;
    double *partials = nullptr;
    size_t partials_capacity = 0;
    double *eig_scratch = nullptr;
    size_t eig_capacity = 0;
    // gram / tall_gemm in double-float arithmetic on the FP32 pipe (about
    // 48 bits, several times faster on GB300) instead of FP64 FMAs
    bool df_products = false;

    // C = alpha * A^T B + beta * C, A: n x ma, B: n x mb, C: ma x mb.
    int gram(const double *A, long long lda, int ma, const double *B, long long ldb, int mb, int n,
             double *C, long long ldc, double alpha = 1.0, double beta = 0.0);
    // C = alpha * A B + beta * C, A: n x m, B: m x p, C: n x p.
    int tall_gemm(const double *A, long long lda, const double *B, long long ldb, double *C,
                  long long ldc, int n, int m, int p, double alpha = 1.0, double beta = 0.0);
    // G = R^T R (one CTA); Rinv = R^{-1}; status_dev[0] = shifts used or -1.
    // cond_bound (device, optional): (1 + e) / (1 - e) with e the Frobenius
    // distance of the unit-diagonal scaled G from I (infinite for e >= 1), a
    // bound of that matrix's condition number; m <= 32 and no shift only,
    // NaN otherwise.
    // df: for m <= 32, factor in double-float arithmetic (about 48 bits, several
    // times faster on GB300 than the FP64 one-warp kernel); FP64 otherwise.
    int chol_inverse(const double *G, int m, double *Rinv, int *status_dev,
                     double *cond_bound = nullptr, bool df = false);
    // Symmetric eigensolve for m <= 112: FP32 Jacobi + FP64 refinement +
    // FP64 cluster polish (k_eig.cu).  Ascending w, eigenvectors Z.
    int symmetric_eig(const double *T, int m, double *w, double *Z, int *sweeps_dev);
    // R = AX - X diag(theta); rnorm[j] = ||r_j||; scaled[j] as the reference.
    int residuals(const double *X, const double *AX, const double *theta, int n, int k,
                  long long ldx, double hnorm, double *R, double *rnorm, double *scaled);
    // T[:, c] = R[:, sel[c]] / clip(d - theta[sel[c]]).
    int diag_correction(const double *R, const double *d, const double *theta, const int *sel,
                        int nsel, int n, double clip, double *T);
    int column_norms(const double *A, long long lda, int n, int c, double *out);
    int gather_columns(const double *src, long long lds, const int *idx, const double *scale,
                       int n, int c, double *dst, long long ldd);
    // Incremental projection T = V^T H V held in Tf (ld): insert the border
    // B = V[:, :m0+c]^T (HV)[:, m0:m0+c]; copy the leading m x m block out;
    // reset the leading m x m block to diag(theta) after a restart.
    int proj_insert(const double *B, int m0, int c, double *Tf, int ld);
    int proj_compact(const double *Tf, int ld, int m, double *Tm);
    int proj_diag(const double *theta, int m, double *Tf, int ld);

    int ensure_partials(size_t count);
    void release();
};

}  // namespace iptgb
