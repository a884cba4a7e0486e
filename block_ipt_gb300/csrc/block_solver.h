// block_solver.h - IPT stage + CholQR2 + Rayleigh-Ritz + Davidson (internal).
#pragma once

#include <cuda_runtime.h>

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
struct LearnedCorrection {
    virtual ~LearnedCorrection() = default;
    virtual int correct(const double *R, const double *d, const double *theta, const int *sel,
                        int nsel, int n, double clip, double *T) = 0;
};

struct LowpDenseOperator;

struct BlockSolveInput {
    const double *initial = nullptr;  // optional start block (n x initial_cols), skips the IPT stage
    int initial_cols = 0;
    Fp64Apply *apply = nullptr;
    IptStage *ipt = nullptr;
    LearnedCorrection *learned = nullptr;
    const double *d = nullptr;  // device diagonal, ascending
    int n = 0;
    int k = 0;
    double hnorm = 1.0;         // ||H||_inf
    IPTBlockOptions opt{};
    int lowp = 0;               // 1 if the IPT stage is low precision (report only)
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

// Low-precision dense IPT stage on the tensor cores (k_tc.cu); nullptr if the
// precision is not supported on this device.
IptStage *make_lowp_dense_stage(const double *dH, int n, const double *d, int precision,
                                cudaStream_t stream, int *status);

// FP64 IPT stages on the plain operators.
IptStage *make_fp64_dense_stage(const double *dH, int n, const double *d, cudaStream_t stream);
IptStage *make_fp64_csr_stage(const int *row_ptr, const int *col_ind, const double *vals, int n,
                              const double *d, cudaStream_t stream);

}  // namespace iptgb
