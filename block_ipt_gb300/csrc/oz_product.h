// oz_product.h - FP64-accurate dense block product on the tensor cores
// (internal; k_oz.cu, operand splitting in oz.cuh).
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "common.cuh"

namespace iptgb {

// The digit slices of Delta = H - diag(H): kOzSlices FP16 matrices
// [slice][row][ldp] (ldp = n rounded up to 64, zero beyond n and on the
// diagonal) and one exponent per row, with the TMA map the product streams.
struct OzDelta {
    int n = 0;
    int ldp = 0;
    DeviceBuffer<__half> A;
    DeviceBuffer<int> rowexp;
    CUtensorMap mapA;
    // storage and tensor map only (the fused setup pass writes the slices)
    int init_storage(int n, cudaStream_t s);
    // slices of a column-major n x n H (any H; the diagonal is left out)
    int split_from(const double *H, int n, cudaStream_t s);
};

// Y = (diag(d) + Delta) X for an n x C block X (column-major, ld ldx), in
// groups of at most kOzMaxCols columns; d may be null (Y = Delta X).
struct OzProduct {
    const OzDelta *dl = nullptr;
    const double *d = nullptr;
    cudaStream_t s = nullptr;
    int sms = 148;
    int cp_cur = 0;
    DeviceBuffer<__half> B;
    DeviceBuffer<int> colexp;
    DeviceBuffer<unsigned long long> colmax;
    DeviceBuffer<double> P;
    DeviceBuffer<int> err;
    CUtensorMap mapB;
    int bind(const OzDelta *delta, const double *diag, cudaStream_t stream);
    int apply(const double *X, long long ldx, int C, double *Y, long long ldy);
    // the kernel's error flag (non-zero: a bounded wait gave up)
    int read_error(int *host_err);

  private:
    int apply_group(const double *X, long long ldx, int C, double *Y, long long ldy);
};

}  // namespace iptgb
