// k_csr64.cu - FP64 sparse kernels of the plain CSR IPT path.
//
// The reference multiplies through cuSPARSE SpMM with the CSC arrays passed
// as CSR and OP_T (IPT_C_GPU/src/ipt_cuda.cu:1535-1559).  Here the host
// preparation produces a true CSR of the (sorted) matrix, so the product is a
// gather, one warp per row.  X is first copied to a row-major block Xr
// (row c holds the k entries X[c, :], padded), so that the BN values a
// nonzero multiplies sit in one cache line: with column-major X every
// nonzero would touch BN different lines.  Within the warp, BN/4 lanes share
// a nonzero (each owns 4 columns, loaded as two 16-byte vectors) and 32/(BN/4)
// nonzeros are in flight; the partial sums are reduced over the nonzero
// streams with shuffles.  Works for any sparsity pattern; rows are
// independent, so no atomics and deterministic results.
#include "common.cuh"
#include "dfloat.cuh"
#include "kernels.cuh"
#include "reduce.cuh"

namespace iptgb {

constexpr int kCsrWarpsPerBlock = 8;

// Xr[c * ldr + j] = X[c + j * n] (j < k), 0 for k <= j < ldr; 32 x 32 tiles.
__global__ void rowmajor_copy_kernel(const double *__restrict__ X, int n, int k,
                                     double *__restrict__ Xr, int ldr)
{
    __shared__ double t[32][33];
    const int r0 = blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int j = c0 + y;
        const int r = r0 + threadIdx.x;
        t[y][threadIdx.x] = (j < k && r < n) ? X[(size_t)r + (size_t)j * n] : 0.0;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y;
        const int j = c0 + threadIdx.x;
        if (r < n && j < ldr) Xr[(size_t)r * ldr + j] = t[threadIdx.x][y];
    }
}

template <int BN>
__global__ void __launch_bounds__(kCsrWarpsPerBlock * 32)
csr64_spmm_kernel(const int *__restrict__ row_ptr, const int *__restrict__ col_ind,
                  const double *__restrict__ vals, int n, const double *__restrict__ Xr,
                  int ldr, int k, double *__restrict__ Y)
{
    constexpr int LPN = BN / 4;          // lanes per nonzero
    constexpr int STREAMS = 32 / LPN;    // nonzeros in flight per warp
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * kCsrWarpsPerBlock + (threadIdx.x >> 5);
    if (row >= n) {
        return;
    }
    const int sub = lane % LPN;
    const int q = lane / LPN;
    const int col0 = blockIdx.y * BN + 4 * sub;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    const int pbeg = row_ptr[row];
    const int pend = row_ptr[row + 1];
    const double *xb = Xr + col0;
    for (int p = pbeg + q; p < pend; p += STREAMS) {
        const double v = __ldg(vals + p);
        const int c = __ldg(col_ind + p);
        const double2 *x = reinterpret_cast<const double2 *>(xb + (size_t)c * ldr);
        const double2 x01 = __ldg(x);
        const double2 x23 = __ldg(x + 1);
        a0 = fma(v, x01.x, a0);
        a1 = fma(v, x01.y, a1);
        a2 = fma(v, x23.x, a2);
        a3 = fma(v, x23.y, a3);
    }
#pragma unroll
    for (int off = 16; off >= LPN; off >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, off);
        a1 += __shfl_xor_sync(0xffffffffu, a1, off);
        a2 += __shfl_xor_sync(0xffffffffu, a2, off);
        a3 += __shfl_xor_sync(0xffffffffu, a3, off);
    }
    if (q == 0) {
        double *y = Y + row;
        if (col0 + 0 < k) y[(size_t)(col0 + 0) * n] = a0;
        if (col0 + 1 < k) y[(size_t)(col0 + 1) * n] = a1;
        if (col0 + 2 < k) y[(size_t)(col0 + 2) * n] = a2;
        if (col0 + 3 < k) y[(size_t)(col0 + 3) * n] = a3;
    }
}

int launch_csr64_spmm(const int *row_ptr, const int *col_ind, const double *vals, int n,
                      const double *X, int k, double *Y, cudaStream_t stream)
{
    if (n <= 0 || k <= 0) {
        return IPT_CUDA_SUCCESS;
    }
    const int bn = k <= 4 ? 4 : (k <= 8 ? 8 : 16);
    const int nblk = (k + bn - 1) / bn;
    const int ldr = nblk * bn;
    DeviceBuffer<double> Xr;
    IPTGB_CHECK(Xr.alloc((size_t)n * ldr, stream));
    rowmajor_copy_kernel<<<dim3((n + 31) / 32, (ldr + 31) / 32), dim3(32, 8), 0, stream>>>(
        X, n, k, Xr.ptr, ldr);
    IPTGB_LAUNCH();
    dim3 grid((n + kCsrWarpsPerBlock - 1) / kCsrWarpsPerBlock, nblk);
    const int threads = kCsrWarpsPerBlock * 32;
    if (bn == 4) {
        csr64_spmm_kernel<4><<<grid, threads, 0, stream>>>(row_ptr, col_ind, vals, n, Xr.ptr, ldr,
                                                            k, Y);
    } else if (bn == 8) {
        csr64_spmm_kernel<8><<<grid, threads, 0, stream>>>(row_ptr, col_ind, vals, n, Xr.ptr, ldr,
                                                            k, Y);
    } else {
        csr64_spmm_kernel<16><<<grid, threads, 0, stream>>>(row_ptr, col_ind, vals, n, Xr.ptr,
                                                             ldr, k, Y);
    }
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------
// The same SpMM in double-float arithmetic on the FP32 pipe: the values as
// (hi, lo) floats split once per solve, X as a row-major block of (hi, lo)
// pairs, df_acc per term (~48 bits).  On GB300 the FP64 kernel above is bound
// by the FP64 pipe at ~81 % of its peak; this one does ~5x more terms per
// second and is limited by the gathers of X instead.
// ---------------------------------------------------------------------------
// Xr2[c * ldr + j] = split(X[c + j * n]) as float2 (hi, lo); 0 beyond k.
__global__ void rowmajor_split_kernel(const double *__restrict__ X, int n, int k,
                                      float2 *__restrict__ Xr2, int ldr)
{
    __shared__ double t[32][33];
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const int r0 = blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int j = c0 + y;
        const int r = r0 + threadIdx.x;
        t[y][threadIdx.x] = (j < k && r < n) ? X[(size_t)r + (size_t)j * n] : 0.0;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y;
        const int j = c0 + threadIdx.x;
        if (r < n && j < ldr) {
            const dfloat v = df_from_double(t[threadIdx.x][y]);
            Xr2[(size_t)r * ldr + j] = make_float2(v.hi, v.lo);
        }
    }
}

template <int BN>
__global__ void __launch_bounds__(kCsrWarpsPerBlock * 32)
csr_df_spmm_kernel(const int *__restrict__ row_ptr, const int *__restrict__ col_ind,
                   const float *__restrict__ vh, const float *__restrict__ vl, int n,
                   const float2 *__restrict__ Xr2, int ldr, int k, double *__restrict__ Y)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    constexpr int LPN = BN / 4;          // lanes per nonzero
    constexpr int STREAMS = 32 / LPN;    // nonzeros in flight per warp
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * kCsrWarpsPerBlock + (threadIdx.x >> 5);
    if (row >= n) {
        return;
    }
    const int sub = lane % LPN;
    const int q = lane / LPN;
    const int col0 = blockIdx.y * BN + 4 * sub;
    float S[4] = {0.f, 0.f, 0.f, 0.f}, s[4] = {0.f, 0.f, 0.f, 0.f};
    const int pbeg = row_ptr[row];
    const int pend = row_ptr[row + 1];
    const float2 *xb = Xr2 + col0;
    for (int p = pbeg + q; p < pend; p += STREAMS) {
        const float h = __ldg(vh + p);
        const float l = __ldg(vl + p);
        const int c = __ldg(col_ind + p);
        const float4 *x = reinterpret_cast<const float4 *>(xb + (size_t)c * ldr);
        const float4 x01 = __ldg(x);      // (hi, lo) of columns col0, col0 + 1
        const float4 x23 = __ldg(x + 1);  // and col0 + 2, col0 + 3
        df_acc(S[0], s[0], h, l, x01.x, x01.y);
        df_acc(S[1], s[1], h, l, x01.z, x01.w);
        df_acc(S[2], s[2], h, l, x23.x, x23.y);
        df_acc(S[3], s[3], h, l, x23.z, x23.w);
    }
#pragma unroll
    for (int off = 16; off >= LPN; off >>= 1) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const dfloat o = {__shfl_xor_sync(0xffffffffu, S[j], off),
                              __shfl_xor_sync(0xffffffffu, s[j], off)};
            const dfloat t = df_add(dfloat{S[j], s[j]}, o);
            S[j] = t.hi;
            s[j] = t.lo;
        }
    }
    if (q == 0) {
        double *y = Y + row;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (col0 + j < k) y[(size_t)(col0 + j) * n] = (double)S[j] + (double)s[j];
        }
    }
}

int launch_csr_df_spmm(const int *row_ptr, const int *col_ind, const float *vh, const float *vl,
                       int n, const double *X, int k, double *Y, cudaStream_t stream)
{
    if (n <= 0 || k <= 0) {
        return IPT_CUDA_SUCCESS;
    }
    const int bn = k <= 4 ? 4 : (k <= 8 ? 8 : 16);
    const int nblk = (k + bn - 1) / bn;
    const int ldr = nblk * bn;
    DeviceBuffer<float2> Xr2;
    IPTGB_CHECK(Xr2.alloc((size_t)n * ldr, stream));
    IPTGB_CHECK(launch_pdl(rowmajor_split_kernel, dim3((n + 31) / 32, (ldr + 31) / 32),
                           dim3(32, 8), 0, stream, X, n, k, Xr2.ptr, ldr));
    dim3 grid((n + kCsrWarpsPerBlock - 1) / kCsrWarpsPerBlock, nblk);
    const dim3 threads(kCsrWarpsPerBlock * 32);
    auto kernel = bn == 4 ? csr_df_spmm_kernel<4>
                  : bn == 8 ? csr_df_spmm_kernel<8>
                            : csr_df_spmm_kernel<16>;
    return launch_pdl(kernel, grid, threads, 0, stream, row_ptr, col_ind, vh, vl, n,
                      (const float2 *)Xr2.ptr, ldr, k, Y);
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
