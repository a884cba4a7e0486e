// k_dense64.cu - FP64 kernels of the plain dense IPT path.
//
// The per-iteration block product Y = H X (reference: cublasDgemm in
// IPT_C_GPU/src/ipt_cuda.cu:1649,1888) is written for GB300's FP64 pipe,
// which retires ~1.2 TFLOP/s: a split-K SIMT kernel keeps every SM's DFMA
// pipe busy (the skinny N = k product has too few output tiles otherwise),
// writes per-slice partial blocks, and a second kernel sums the partials in a
// fixed order and applies the IPT update (reference kernels
// column_diagonal_after_d_kernel / ipt_update_kernel / fixed_point_delta_kernel,
// IPT_C_GPU/src/ipt_cuda.cu:1403-1467) together with both Frobenius norms.
#include "common.cuh"
#include "kernels.cuh"
#include "reduce.cuh"

namespace iptgb {

// ---------------------------------------------------------------------------
// Split-K partial product.  Block = 256 threads, one output row per thread,
// BN output columns per thread held in registers.  Grid: (row blocks, S
// slices, column tiles).  P is laid out [slice][column][row].
// ---------------------------------------------------------------------------
constexpr int kD64Rows = 256;
constexpr int kD64Chunk = 32;

template <typename T, int BN>
__global__ void __launch_bounds__(kD64Rows)
dense64_partial_kernel(const T *__restrict__ H, int n, long long ldh,
                       const T *__restrict__ X, long long ldx, int k,
                       T *__restrict__ P, int kslice)
{
    __shared__ T xs[kD64Chunk][BN];
    const int row = blockIdx.x * kD64Rows + threadIdx.x;
    const int s = blockIdx.y;
    const int c0 = blockIdx.z * BN;
    const int kbeg = s * kslice;
    const int kend = min(n, kbeg + kslice);
    T acc[BN];
#pragma unroll
    for (int j = 0; j < BN; ++j) {
        acc[j] = T(0);
    }
    const bool active = row < n;
    const T *hrow = H + (active ? row : 0);

    for (int l0 = kbeg; l0 < kend; l0 += kD64Chunk) {
        const int lc = min(kD64Chunk, kend - l0);
        __syncthreads();
        for (int e = threadIdx.x; e < kD64Chunk * BN; e += kD64Rows) {
            const int ll = e % kD64Chunk;
            const int j = e / kD64Chunk;
            T v = T(0);
            if (ll < lc && c0 + j < k) {
                v = X[(size_t)(l0 + ll) + (size_t)(c0 + j) * (size_t)ldx];
            }
            xs[ll][j] = v;
        }
        __syncthreads();
        if (active) {
            const T *hp = hrow + (size_t)l0 * (size_t)ldh;
            if (lc == kD64Chunk) {
                T h[kD64Chunk];
#pragma unroll
                for (int ll = 0; ll < kD64Chunk; ++ll) {
                    h[ll] = __ldg(hp + (size_t)ll * (size_t)ldh);
                }
#pragma unroll
                for (int ll = 0; ll < kD64Chunk; ++ll) {
#pragma unroll
                    for (int j = 0; j < BN; ++j) {
                        acc[j] = fma(h[ll], xs[ll][j], acc[j]);
                    }
                }
            } else {
                for (int ll = 0; ll < lc; ++ll) {
                    const T h = __ldg(hp + (size_t)ll * (size_t)ldh);
#pragma unroll
                    for (int j = 0; j < BN; ++j) {
                        acc[j] = fma(h, xs[ll][j], acc[j]);
                    }
                }
            }
        }
    }
    if (active) {
#pragma unroll
        for (int j = 0; j < BN; ++j) {
            if (c0 + j < k) {
                P[((size_t)s * (size_t)k + (size_t)(c0 + j)) * (size_t)n + row] = acc[j];
            }
        }
    }
}

static int pick_bn(int k)
{
    if (k <= 4) return 4;
    if (k <= 8) return 8;
    if (k <= 16) return 16;
    return 32;
}

int dense64_split_for(int n, int k, int sms)
{
    const int row_blocks = (n + kD64Rows - 1) / kD64Rows;
    const int bn = pick_bn(k);
    const int col_tiles = (k + bn - 1) / bn;
    // Aim at ~4 resident 256-thread blocks per SM; FP64 work per block must
    // stay well above the partial-store cost, so slices are >= 128 deep.
    int want = (4 * sms + row_blocks * col_tiles - 1) / (row_blocks * col_tiles);
    int max_s = (n + 127) / 128;
    if (want > max_s) want = max_s;
    if (want < 1) want = 1;
    return want;
}

template <typename T>
static int launch_partial_t(const T *H, int n, long long ldh, const T *X, long long ldx, int k,
                            T *P, int S, cudaStream_t stream)
{
    int kslice = (n + S - 1) / S;
    kslice = ((kslice + kD64Chunk - 1) / kD64Chunk) * kD64Chunk;
    const int row_blocks = (n + kD64Rows - 1) / kD64Rows;
    const int bn = pick_bn(k);
    dim3 grid(row_blocks, S, (k + bn - 1) / bn);
    switch (bn) {
    case 4:
        dense64_partial_kernel<T, 4><<<grid, kD64Rows, 0, stream>>>(H, n, ldh, X, ldx, k, P, kslice);
        break;
    case 8:
        dense64_partial_kernel<T, 8><<<grid, kD64Rows, 0, stream>>>(H, n, ldh, X, ldx, k, P, kslice);
        break;
    case 16:
        dense64_partial_kernel<T, 16><<<grid, kD64Rows, 0, stream>>>(H, n, ldh, X, ldx, k, P, kslice);
        break;
    default:
        dense64_partial_kernel<T, 32><<<grid, kD64Rows, 0, stream>>>(H, n, ldh, X, ldx, k, P, kslice);
        break;
    }
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

int launch_dense64_partial(const double *H, int n, long long ldh, const double *X,
                           long long ldx, int k, double *P, int S, cudaStream_t stream)
{
    return launch_partial_t<double>(H, n, ldh, X, ldx, k, P, S, stream);
}

// FP32 SIMT variant of the same split-K product (the reference's FP32
// "pedantic" GemmEx path, IPT_C_GPU/src/mixed_precision/ipt_mixed_precision_cuda.cu:802-815).
int launch_dense32_partial(const float *H, int n, long long ldh, const float *X, long long ldx,
                           int k, float *P, int S, cudaStream_t stream)
{
    return launch_partial_t<float>(H, n, ldh, X, ldx, k, P, S, stream);
}

// ---------------------------------------------------------------------------
// Sum the S partial slices into Y (fixed slice order => deterministic).
// ---------------------------------------------------------------------------
__global__ void sum_partials_kernel(const double *__restrict__ P, int S, size_t elems,
                                    double *__restrict__ Y)
{
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= elems) {
        return;
    }
    double y = 0.0;
    for (int s = 0; s < S; ++s) {
        y += P[(size_t)s * elems + idx];
    }
    Y[idx] = y;
}

int launch_sum_partials(const double *P, int S, size_t elems, double *Y, cudaStream_t stream)
{
    sum_partials_kernel<<<blocks_for(elems), kThreads, 0, stream>>>(P, S, elems, Y);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------
// IPT update from the partial slices of Y = H X.
//   y      = sum_s P[s]                              (H X)_ij
//   c_j    = y_jj - d_j X_jj                          (Delta X)_jj
//   X'_ij  = (y - d_i X_ij - X_ij c_j) * g_ij,  g_ij = 1 / (d_j - d_i)
//   X'_jj  = 1
// (IPT_C_GPU/src/ipt_cuda.cu:1369-1443).  A zero or non-finite gap gives NaN,
// like build_g_kernel with min_gap_allowed = 0.
// With want_norms, also ||X' - X||_F and ||X||_F (ipt_cuda.cu:1457-1467,1663-1688).
// ---------------------------------------------------------------------------
__global__ void dense64_update_kernel(const double *__restrict__ P, int S, int n, int k,
                                      const double *__restrict__ X, const double *__restrict__ d,
                                      double *__restrict__ Xn, int want_norms,
                                      double2 *partials, unsigned int *counter, double *norms)
{
    const size_t elems = (size_t)n * (size_t)k;
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    double dsq = 0.0, xsq = 0.0;
    if (idx < elems) {
        const int row = (int)(idx % (size_t)n);
        const int col = (int)(idx / (size_t)n);
        const double x = X[idx];
        double out;
        if (row == col) {
            out = 1.0;
        } else {
            double y = 0.0;
            double yjj = 0.0;
            const size_t didx = (size_t)col + (size_t)col * (size_t)n;
            for (int s = 0; s < S; ++s) {
                y += P[(size_t)s * elems + idx];
                yjj += P[(size_t)s * elems + didx];
            }
            const double c = yjj - d[col] * X[didx];
            const double gap = d[col] - d[row];
            const double g = (isfinite(gap) && gap != 0.0) ? 1.0 / gap : NAN;
            out = (y - d[row] * x - x * c) * g;
        }
        Xn[idx] = out;
        if (want_norms) {
            const double diff = out - x;
            dsq = diff * diff;
            xsq = x * x;
        }
    }
    if (want_norms) {
        double2 t = block_sum2(dsq, xsq);
        grid_finish_norms2(t, partials, counter, norms);
    }
}

int launch_dense64_update(const double *P, int S, int n, int k, const double *X,
                          const double *d, double *Xn, int want_norms, NormScratch *ns,
                          cudaStream_t stream)
{
    const size_t elems = (size_t)n * (size_t)k;
    const int grid = blocks_for(elems);
    if (want_norms && grid > ns->capacity) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    dense64_update_kernel<<<grid, kThreads, 0, stream>>>(
        P, S, n, k, X, d, Xn, want_norms, ns->partials, ns->counter, ns->norms);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------
// Small helpers.
// ---------------------------------------------------------------------------
__global__ void set_identity_kernel(double *x, int n, int k)
{
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < (size_t)n * (size_t)k) {
        int row = (int)(idx % (size_t)n);
        int col = (int)(idx / (size_t)n);
        x[idx] = row == col ? 1.0 : 0.0;
    }
}

int launch_set_identity(double *x, int n, int k, cudaStream_t stream)
{
    set_identity_kernel<<<blocks_for((size_t)n * k), kThreads, 0, stream>>>(x, n, k);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

__global__ void extract_diagonal_kernel(const double *H, long long ldh, int n, double *d)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        d[i] = H[(size_t)i + (size_t)i * (size_t)ldh];
    }
}

int launch_extract_diagonal(const double *H, long long ldh, int n, double *d, cudaStream_t stream)
{
    extract_diagonal_kernel<<<blocks_for(n), kThreads, 0, stream>>>(H, ldh, n, d);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

// values[j] = (H X)_jj = sum_l H[j,l] X[l,j]: one block per column (reference:
// final product + gather_values_kernel, IPT_C_GPU/src/ipt_cuda.cu:1934-1942).
__global__ void dense64_diag_values_kernel(const double *__restrict__ H, long long ldh, int n,
                                           const double *__restrict__ X, int k, double *values)
{
    const int j = blockIdx.x;
    double s = 0.0;
    for (int l = threadIdx.x; l < n; l += blockDim.x) {
        s = fma(H[(size_t)j + (size_t)l * (size_t)ldh], X[(size_t)l + (size_t)j * (size_t)n], s);
    }
    double2 t = block_sum2(s, 0.0);
    if (threadIdx.x == 0 && j < k) {
        values[j] = t.x;
    }
}

int launch_dense64_diag_values(const double *H, long long ldh, int n, const double *X, int k,
                               double *values, cudaStream_t stream)
{
    dense64_diag_values_kernel<<<k, kThreads, 0, stream>>>(H, ldh, n, X, k, values);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

}  // namespace iptgb
