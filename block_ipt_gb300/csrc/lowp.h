// lowp.h - low-precision (tensor-core) dense IPT operator (internal).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "ipt_plain.h"
#include "kernels.cuh"

namespace iptgb {

// Operand formats of the tensor-core product.
enum { kLowpF16 = 0, kLowpBF16 = 1, kLowpTF32 = 2, kLowpF32 = 3 };

// The IPT map X' = E + G o (Delta X - X diag(Delta X)) with Delta X on the
// tensor cores.  The block lives inside the operator as an FP32 master copy
// plus the low-precision operand copy; set_width() sizes it, reset_identity()
// starts from the unit vectors of the first p diagonal positions.
struct LowpDenseOperator {
    virtual ~LowpDenseOperator() = default;
    virtual int set_width(int p) = 0;
    virtual int reset_identity(const double *d) = 0;
    virtual int product() = 0;                               // partials of Delta X only
    virtual int step(int want_norms, NormScratch *ns) = 0;   // product + update
    virtual int read_error(int *host_err) = 0;               // async copy of the error flag
    virtual int export_fp64(double *X) = 0;                  // current block -> FP64
    virtual int export_fp64_prev(double *X) = 0;             // previous block -> FP64
    virtual const float *partials() const = 0;               // [split][col][row] FP32
    virtual int num_splits() const = 0;
    virtual double streamed_bytes() const { return 0.0; }    // operator bytes per product

    // Correction solve of the mixed refinement (after set_width/reset_identity
    // sized the block).  With the FP64 defect R0 = F(X) - X of the current
    // FP64 block X and c_j = (Delta X)_jj, iterate in low precision
    //   delta <- R0 + G o (B - X diag(b) - delta diag(c + b)),  B = Delta delta,
    // b_j = B_jj, which converges to the exact correction X* - X of the IPT
    // fixed point.  The operand copy of column j is scaled by sigma_j (a
    // power of two chosen from max |R0_j|) to use the FP16 range.
    virtual int refine_begin(const double *R0, const double *X, const double *c,
                             const float *sigma) = 0;
    virtual int refine_step(int want_norms, NormScratch *ns) = 0;
    virtual int refine_apply(double *X) = 0;  // X += delta (FP64)
    // Anderson mixing of depth one, column by column, after every step of
    // the IPT iteration and of the correction solve (with host-read checks):
    // with the map's value f = F(x) and g = f - x of this step and of the
    // previous one, x+ = f - theta (f - f_prev), theta = <g, g - g_prev> /
    // ||g - g_prev||^2 (Walker and Ni, SIAM J. Numer. Anal. 49 (2011)).  Off
    // by default: the reference's IPT entry points iterate the plain map.
    virtual void set_mixing(bool on) { (void)on; }
};

// Statistics of a dense symmetric H (device, zero-initialised before use):
// the largest column sum of |H|, the largest off-diagonal |H_il| (non-negative
// doubles order like their bit patterns) and the count of descents
// d_{i+1} < d_i of the diagonal.
struct DenseStats {
    unsigned long long hnorm_bits;
    unsigned long long maxabs_bits;
    unsigned long long descents;
};

// Largest n the fused setup pass handles (one column of H in shared memory).
constexpr int kFusedSetupMaxN = 16384;

// Optional inputs and outputs of the operator's one pass over H.
struct LowpDenseSetup {
    double maxabs = -1.0;           // >= 0: max |H_il| (l != i) is known (no extra pass)
    bool symmetric = false;         // H exactly symmetric: columns of H stream as rows of Delta
    float *split_hi = nullptr;      // symmetric only: the pass also writes the double-FP32
    float *split_lo = nullptr;      //   split of H (column-major)
    double *colsum_part = nullptr;  // symmetric only: partial column sums of |H|,
                                    //   [chunk][column], chunk = 2048 rows
    int colsum_chunks = 0;          // out: chunks written to colsum_part
    bool split_done = false;        // out: split_hi/lo written
    // Fused setup (symmetric, n <= kFusedSetupMaxN): one CTA per column of
    // fused_src (device memory or mapped pinned host memory) writes row c of
    // Delta with its own power-of-two scale (no global maximum needed, so no
    // pass before it), the split, the diagonal and the statistics; with
    // fused_copy also the FP64 matrix itself (when fused_src is host memory).
    const double *fused_src = nullptr;
    double *fused_copy = nullptr;
    // fused setup from pinned host memory read by its upper triangle only
    // (device-accessible pointer; H symmetric): column chunks of the upper
    // triangle cross the host link in decreasing column order into
    // fused_copy, mirrored there into the full matrix, and the setup of each
    // chunk runs on a second stream while the next chunk crosses the link
    // (fused_src is then not used)
    const double *upper_host = nullptr;
    double *diag = nullptr;         // n entries
    DenseStats *stats = nullptr;    // device, zeroed by the caller
    bool fused_done = false;        // out
    // fused setup only: the digit slices of Delta for the FP64-accurate
    // tensor-core product ([kOzSlices][n][ldp] FP16, ldp = n rounded up to
    // 64) and their row exponents (oz.cuh)
    __half *oz = nullptr;
    int *oz_rowexp = nullptr;
    bool oz_done = false;           // out
};
constexpr int kLowpColsumChunk = 2048;
LowpDenseOperator *make_lowp_dense_operator(const double *dH, int n, int kind, cudaStream_t s,
                                            int *status, LowpDenseSetup *setup = nullptr);

// Whether an iteration on `op` should use the device-side stop (NormScratch
// history): the per-step norm reduction costs a few microseconds, the
// pass-through steps after convergence save about one check interval of
// products; worth it once a product streams clearly more than L2 holds.
// Tuning knob IPT_GB300_DEVICE_STOP (0 = off, 1 = on).
bool lowp_device_stop(const LowpDenseOperator &op);

int run_lowp_ipt(LowpDenseOperator &op, int n, int p, int maxiter, double tol, int check_every,
                 double *X, int *iterations, double *fpres_out, long long *matvecs,
                 cudaStream_t s, bool guard);

}  // namespace iptgb
