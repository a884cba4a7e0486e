// block_solver.h - IPT stage + CholQR2 + Rayleigh-Ritz + Davidson (internal).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "../../include/ipt_block.h"
#include "block_ops.h"
#include "kernels.cuh"

namespace iptgb {

// FP64-accurate block product AV = H V (V, AV: n x c, ld = n).
struct Fp64Apply {
    virtual ~Fp64Apply() = default;
    virtual int apply(const double *V, int c, double *AV) = 0;
};

// The IPT stage: iterate the IPT map on the p lowest diagonal positions from
// the identity start and leave the final block, in FP64, in X (n x p).
struct IptStage {
    virtual ~IptStage() = default;
    virtual int run(int p, int maxiter, double tol, int check_every, double *X, int *iterations,
                    double *fixed_point_residual, long long *matvecs) = 0;
};

// Learned Davidson correction (k_mlp.cu): T[:, c] from features of the
// residual rows; returns IPT_CUDA_SUCCESS or an error.
// Inputs of a Davidson correction for the selected Ritz pairs sel[0..nsel):
// residuals R and Ritz vectors X (n x k), diagonal d, Ritz values theta,
// residual norms rnorm (k), the clip of the diagonal correction, and the
// current orthonormal search space V (n x m).
struct CorrectionArgs {
    // products H T for the correction's own terms (a preconditioner may use
    // a lower-precision operator than the solve's FP64-accurate one)
    Fp64Apply *apply = nullptr;
    const double *V = nullptr;
    int m = 0;
    const double *R = nullptr;
    const double *X = nullptr;
    const double *d = nullptr;
    const double *theta = nullptr;
    const double *rnorm = nullptr;
    const int *sel = nullptr;
    int nsel = 0;
    int n = 0;
    double clip = 0.0;
};

// A replacement for the plain diagonal correction (k_mlp.cu).  bind() gives
// the per-row off-diagonal coupling ||H[i, j != i]||_2 (device) and
// ||H||_inf before the solve; learned() says whether the Davidson solver should
// check the step (accept, or reject and redo it with the plain correction).
struct LearnedCorrection {
    virtual ~LearnedCorrection() = default;
    virtual void bind(const double *row_coupling, double hnorm) = 0;
    virtual bool learned() const = 0;
    virtual int correct(const CorrectionArgs &a, double *T) = 0;
};

LearnedCorrection *make_learned_correction(const float *params, cudaStream_t stream);
// Training-data collector: records rows (6 features, target, weight) against
// the converged vectors Xstar and returns the plain correction, or the
// learned one when params is not null.
LearnedCorrection *make_mlp_collector(const double *Xstar, int kstar, float *out,
                                      long long capacity, const float *params,
                                      cudaStream_t stream);
long long mlp_collector_count(const LearnedCorrection *collector);
int launch_csr_row_coupling(const int *row_ptr, const int *col_ind, const double *vals, int n,
                            double *sigma, cudaStream_t s);
int launch_dense_row_coupling(const double *H, int n, double *sigma, cudaStream_t s);

struct LowpDenseOperator;

// Orthogonality of a Rayleigh-Ritz basis and of its Ritz vectors: the
// Frobenius norm and the largest entry of C^T C - I over the columns C, and
// whether C held a non-finite entry (both figures NaN then), as the
// reference's IPT_RR_HOST_ORTHOGONALITY_STATS report
// (IPT_C_GPU/src/ipt_cuda.cu:2489-2524, 3191-3268).
struct OrthFigure {
    double frobenius = NAN;
    double max_abs = NAN;
    int invalid = 0;
};
struct OrthStats {
    // the first basis figure describes the start block as given, before its
    // orthogonalisation (the reference's Gram + generalized eigensolve on the
    // raw cluster basis); otherwise the orthonormalised basis (its
    // IPT_BLOCK_CLUSTER_QR path)
    bool raw_first_basis = true;
    OrthFigure basis;
    OrthFigure ritz;
};

struct BlockSolveInput {
    const double *initial = nullptr;  // optional start block (n x initial_cols), skips the IPT stage
    int initial_cols = 0;
    Fp64Apply *apply = nullptr;
    // operator for the learned correction's products (nullptr: `apply`)
    Fp64Apply *precond_apply = nullptr;
    IptStage *ipt = nullptr;
    LearnedCorrection *learned = nullptr;
    const double *d = nullptr;  // device diagonal, ascending
    int n = 0;
    int k = 0;
    double hnorm = 1.0;         // ||H||_inf
    IPTBlockOptions opt{};
    int lowp = 0;               // 1 if the IPT stage is low precision (report only)
    // Ritz vectors a thick restart keeps at most (0: as many as leave room
    // for the next block).  A restart costs two n x m x keep products; where
    // an operator product is cheap (sparse H) a small restart can save more
    // than the extra steps it causes (FCI-like n = 63,504, k = 16, keep 2k:
    // 28.5 ms and 11 steps against 33.7 ms and 10), where it is dear
    // (matrix-free sigma) the opposite.  Every entry leaves it at 0; tuning
    // knob IPT_GB300_RESTART_KEEP sets it.
    int restart_keep = 0;
    // when set, receives the orthogonality figures of the Rayleigh-Ritz step
    // whose pairs are returned (computed in FP64 after every such step)
    OrthStats *orth = nullptr;
};

int block_solve(const BlockSolveInput &in, double *X_out, double *values_out,
                IPTBlockReport *report, cudaStream_t stream);

struct RefineInput {
    Fp64Apply *apply = nullptr;
    IptStage *ipt = nullptr;            // low-precision IPT start, or nullptr (identity start)
    LowpDenseOperator *lowp = nullptr;  // correction solver, or nullptr (plain FP64 IPT steps)
    const double *d = nullptr;
    int n = 0;
    int k = 0;
    double hnorm = 1.0;
    int max_outer = 8;
    int inner_maxiter = 64;
    double inner_tol = 1e-3;
    bool mixing = false;                // the low-precision iterations mix (lowp.h set_mixing)
    IPTBlockOptions opt{};
};

// Refinement driver (refine.cu).  On return *converged tells whether the
// Ritz pairs in X_out / values_out met the tolerance; if not, X_fallback
// (n x k) holds the best block for a Davidson restart.
int refine_solve(const RefineInput &in, double *X_out, double *values_out, IPTBlockReport *report,
                 cudaStream_t stream, bool *converged, double *X_fallback);

// IPT stage running on an existing low-precision operator (not owned).
IptStage *make_lowp_stage_on(LowpDenseOperator *op, const double *d, int n, cudaStream_t stream);

void fill_default_options(IPTBlockOptions *opt);

// Large bases: the Davidson solver's Gram and tall products and the sparse
// products run in double-float on the FP32 pipe (~48 bits, far below the
// 1e-8 residual they serve; several times faster on GB300); small problems
// keep FP64, where these products cost little.  From 16384 rows; tuning
// knob IPT_GB300_DF_DAVIDSON (0 off, 1 always).
bool davidson_df_products(int n);

// Low-precision dense IPT stage on the tensor cores (k_tc.cu); nullptr if the
// precision is not supported on this device.
IptStage *make_lowp_dense_stage(const double *dH, int n, const double *d, int precision,
                                cudaStream_t stream, int *status);

// FP64 IPT stages on the plain operators.
IptStage *make_fp64_dense_stage(const double *dH, int n, const double *d, cudaStream_t stream);
IptStage *make_fp64_csr_stage(const int *row_ptr, const int *col_ind, const double *vals, int n,
                              const double *d, cudaStream_t stream);

}  // namespace iptgb
