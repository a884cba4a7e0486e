// k_csr64.cu - FP64 sparse kernels of the plain CSR IPT path.
//
// The reference multiplies through cuSPARSE SpMM with the CSC arrays passed
// as CSR and OP_T (IPT_C_GPU/src/ipt_cuda.cu:1535-1559).  Here the host
// preparation produces a true CSR of the (sorted) matrix, so the product is a
// gather: one warp per row, lanes stride over the row's nonzeros, every lane
// keeps BN column accumulators in registers and the warp reduces them with
// shuffles.  Works for any sparsity pattern; rows are independent, so no
// atomics and deterministic results.
#include "common.cuh"
#include "kernels.cuh"
#include "reduce.cuh"

namespace iptgb {

constexpr int kCsrWarpsPerBlock = 8;

template <int BN>
__global__ void __launch_bounds__(kCsrWarpsPerBlock * 32)
csr64_spmm_kernel(const int *__restrict__ row_ptr, const int *__restrict__ col_ind,
                  const double *__restrict__ vals, int n, const double *__restrict__ X,
                  int k, double *__restrict__ Y)
{
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * kCsrWarpsPerBlock + (threadIdx.x >> 5);
    const int c0 = blockIdx.y * BN;
    if (row >= n) {
        return;
    }
    double acc[BN];
#pragma unroll
    for (int j = 0; j < BN; ++j) {
        acc[j] = 0.0;
    }
    const int pbeg = row_ptr[row];
    const int pend = row_ptr[row + 1];
    for (int p = pbeg + lane; p < pend; p += 32) {
        const double v = __ldg(vals + p);
        const int c = __ldg(col_ind + p);
        const double *xc = X + c;
#pragma unroll
        for (int j = 0; j < BN; ++j) {
            if (c0 + j < k) {
                acc[j] = fma(v, __ldg(xc + (size_t)(c0 + j) * (size_t)n), acc[j]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < BN; ++j) {
        acc[j] = warp_sum(acc[j]);
    }
    // lane j writes column c0 + j (BN <= 32)
#pragma unroll
    for (int j = 0; j < BN; ++j) {
        if (lane == j && c0 + j < k) {
            Y[(size_t)row + (size_t)(c0 + j) * (size_t)n] = acc[j];
        }
    }
}

int launch_csr64_spmm(const int *row_ptr, const int *col_ind, const double *vals, int n,
                      const double *X, int k, double *Y, cudaStream_t stream)
{
    const int bn = k <= 4 ? 4 : (k <= 8 ? 8 : 16);
    dim3 grid((n + kCsrWarpsPerBlock - 1) / kCsrWarpsPerBlock, (k + bn - 1) / bn);
    const int threads = kCsrWarpsPerBlock * 32;
    if (bn == 4) {
        csr64_spmm_kernel<4><<<grid, threads, 0, stream>>>(row_ptr, col_ind, vals, n, X, k, Y);
    } else if (bn == 8) {
        csr64_spmm_kernel<8><<<grid, threads, 0, stream>>>(row_ptr, col_ind, vals, n, X, k, Y);
    } else {
        csr64_spmm_kernel<16><<<grid, threads, 0, stream>>>(row_ptr, col_ind, vals, n, X, k, Y);
    }
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

int launch_ipt_update_from_y(const double *Y, int n, int k, const double *X, const double *d,
                             double *Xn, int want_norms, NormScratch *ns, cudaStream_t stream)
{
    // A full product block is a single "slice" of the split-K layout.
    return launch_dense64_update(Y, 1, n, k, X, d, Xn, want_norms, ns, stream);
}

// d[i] = H_ii (first stored diagonal entry of row i, 0 if none), matching
// extract_csc_diagonal_kernel (IPT_C_GPU/src/ipt_cuda.cu:1469-1489).
__global__ void csr64_diagonal_kernel(const int *row_ptr, const int *col_ind,
                                      const double *vals, int n, double *d)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    double v = 0.0;
    for (int p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
        if (col_ind[p] == i) {
            v = vals[p];
            break;
        }
    }
    d[i] = v;
}

int launch_csr64_diagonal(const int *row_ptr, const int *col_ind, const double *vals, int n,
                          double *d, cudaStream_t stream)
{
    csr64_diagonal_kernel<<<blocks_for(n), kThreads, 0, stream>>>(row_ptr, col_ind, vals, n, d);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

// values[j] = (H X)_jj = row j of H dotted with column j of X; one warp per j.
__global__ void csr64_diag_values_kernel(const int *__restrict__ row_ptr,
                                         const int *__restrict__ col_ind,
                                         const double *__restrict__ vals, int n,
                                         const double *__restrict__ X, int k, double *values)
{
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (j >= k) {
        return;
    }
    double s = 0.0;
    for (int p = row_ptr[j] + lane; p < row_ptr[j + 1]; p += 32) {
        s = fma(vals[p], X[(size_t)col_ind[p] + (size_t)j * (size_t)n], s);
    }
    s = warp_sum(s);
    if (lane == 0) {
        values[j] = s;
    }
}

int launch_csr64_diag_values(const int *row_ptr, const int *col_ind, const double *vals, int n,
                             const double *X, int k, double *values, cudaStream_t stream)
{
    const int warps = 8;
    csr64_diag_values_kernel<<<(k + warps - 1) / warps, warps * 32, 0, stream>>>(
        row_ptr, col_ind, vals, n, X, k, values);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

}  // namespace iptgb
