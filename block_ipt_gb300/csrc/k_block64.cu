// k_block64.cu - FP64 block kernels for CholQR, Rayleigh-Ritz and Davidson.
//
// These are the steps whose stability needs FP64 (Gram matrices, the
// projected matrix and its eigensolve, residual norms, the correction step).
// Reference counterparts: Householder QR / Gram + sygvd Rayleigh-Ritz
// (IPT_C_GPU/src/ipt_cuda.cu:3039-3316), mixed CholQR
// (IPT_C_GPU/mixed/ipt_rayleigh_mixed_mpqr_cuda.cu:169-386), residual kernels
// (ipt_cuda.cu:2399-2447,2608-2709) and the Davidson correction
// (ipt_cuda.cu:2449-2465,2711-2780,3389-3403).
//
// GB300 retires ~8 GFLOP/s of FP64 per SM, so every O(n m^2) kernel here is
// spread over all SMs (row-chunk partials reduced in a fixed order), and the
// O(m^3) kernels run in one CTA on data held in shared memory.
#include <math.h>

#include "block_ops.h"
#include "common.cuh"
#include "dfloat.cuh"
#include "reduce.cuh"

namespace iptgb {

// ---------------------------------------------------------------------------
// Gram-type products C = A^T B (A: n x ma, B: n x mb, column-major).
// Grid: (row chunks, output tiles of 32x32).  Partials [chunk][mb][ma].
// ---------------------------------------------------------------------------
constexpr int kGramRows = 64;
constexpr int kGramTile = 32;

__global__ void __launch_bounds__(256)
gram_partial_kernel(const double *__restrict__ A, long long lda, int ma,
                    const double *__restrict__ B, long long ldb, int mb, int n, int chunks_per_block,
                    double *__restrict__ P)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    __shared__ double as[kGramRows][kGramTile + 1];
    __shared__ double bs[kGramRows][kGramTile + 1];
    const int tiles_i = (ma + kGramTile - 1) / kGramTile;
    const int ti = blockIdx.y % tiles_i;
    const int tj = blockIdx.y / tiles_i;
    const int i0 = ti * kGramTile;
    const int j0 = tj * kGramTile;
    // thread -> 4 outputs: (li, lj + 8q), q = 0..3
    const int li = threadIdx.x % kGramTile;
    const int lj = threadIdx.x / kGramTile;  // 0..7
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int c = 0; c < chunks_per_block; ++c) {
        const int r0 = (blockIdx.x * chunks_per_block + c) * kGramRows;
        if (r0 >= n) {
            break;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < kGramRows * kGramTile; e += blockDim.x) {
            const int r = e % kGramRows;
            const int col = e / kGramRows;
            const int row = r0 + r;
            as[r][col] = (row < n && i0 + col < ma) ? A[(size_t)row + (size_t)(i0 + col) * lda] : 0.0;
            bs[r][col] = (row < n && j0 + col < mb) ? B[(size_t)row + (size_t)(j0 + col) * ldb] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int r = 0; r < kGramRows; ++r) {
            const double a = as[r][li];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                acc[q] = fma(a, bs[r][lj + 8 * q], acc[q]);
            }
        }
    }
    const size_t mm = (size_t)ma * (size_t)mb;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = i0 + li;
        const int j = j0 + lj + 8 * q;
        if (i < ma && j < mb) {
            P[(size_t)blockIdx.x * mm + (size_t)j * ma + i] = acc[q];
        }
    }
}

__global__ void reduce_slices_kernel(const double *__restrict__ P, int slices, size_t elems,
                                     double *__restrict__ out, long long ldo, int rows,
                                     double alpha, double beta)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= elems) {
        return;
    }
    double s = 0.0;
    for (int b = 0; b < slices; ++b) {
        s += P[(size_t)b * elems + e];
    }
    const size_t i = e % (size_t)rows;
    const size_t j = e / (size_t)rows;
    double *o = out + i + j * (size_t)ldo;
    *o = beta == 0.0 ? alpha * s : alpha * s + beta * *o;
}

// The same partial Gram products in double-float arithmetic on the FP32
// pipe (BlockOps::df_products): tiles split into (hi, lo) floats when staged,
// df_acc per term; GB300's FP32 pipe runs ~5x more of these terms per second
// than its FP64 pipe runs FMAs.
__global__ void __launch_bounds__(256)
gram_partial_df_kernel(const double *__restrict__ A, long long lda, int ma,
                       const double *__restrict__ B, long long ldb, int mb, int n,
                       int chunks_per_block, double *__restrict__ P)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    // (hi, lo) pairs: one 8-byte load per entry
    __shared__ float2 as2[kGramRows][kGramTile + 1];
    __shared__ float2 bs2[kGramRows][kGramTile + 1];
    const int tiles_i = (ma + kGramTile - 1) / kGramTile;
    const int ti = blockIdx.y % tiles_i;
    const int tj = blockIdx.y / tiles_i;
    const int i0 = ti * kGramTile;
    const int j0 = tj * kGramTile;
    const int li = threadIdx.x % kGramTile;
    const int lj = threadIdx.x / kGramTile;  // 0..7
    float S[4] = {0.f, 0.f, 0.f, 0.f}, sl[4] = {0.f, 0.f, 0.f, 0.f};
    for (int c = 0; c < chunks_per_block; ++c) {
        const int r0 = (blockIdx.x * chunks_per_block + c) * kGramRows;
        if (r0 >= n) {
            break;
        }
        __syncthreads();
        // loads first (all in flight), then the splits into shared memory
        constexpr int kPer = kGramRows * kGramTile / 256;
        double av[kPer], bv[kPer];
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const int e = threadIdx.x + q * 256;
            const int r = e % kGramRows;
            const int col = e / kGramRows;
            const int row = r0 + r;
            av[q] = (row < n && i0 + col < ma) ? A[(size_t)row + (size_t)(i0 + col) * lda] : 0.0;
            bv[q] = (row < n && j0 + col < mb) ? B[(size_t)row + (size_t)(j0 + col) * ldb] : 0.0;
        }
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const int e = threadIdx.x + q * 256;
            const int r = e % kGramRows;
            const int col = e / kGramRows;
            const dfloat a = df_from_double(av[q]);
            const dfloat b = df_from_double(bv[q]);
            as2[r][col] = make_float2(a.hi, a.lo);
            bs2[r][col] = make_float2(b.hi, b.lo);
        }
        __syncthreads();
#pragma unroll 4
        for (int r = 0; r < kGramRows; ++r) {
            const float2 a = as2[r][li];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float2 b = bs2[r][lj + 8 * q];
                df_acc(S[q], sl[q], a.x, a.y, b.x, b.y);
            }
        }
    }
    const size_t mm = (size_t)ma * (size_t)mb;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = i0 + li;
        const int j = j0 + lj + 8 * q;
        if (i < ma && j < mb) {
            P[(size_t)blockIdx.x * mm + (size_t)j * ma + i] = (double)S[q] + (double)sl[q];
        }
    }
}

// Slice sums with one warp per output: lanes take every 32nd slice, then a
// fixed shuffle tree (deterministic; many slices reduce in parallel instead
// of one thread's FP64 chain).
__global__ void reduce_slices_warp_kernel(const double *__restrict__ P, int slices, size_t elems,
                                          double *__restrict__ out, long long ldo, int rows,
                                          double alpha, double beta)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const size_t e = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (e >= elems) return;  // whole warps leave together
    double s = 0.0;
    for (int b = lane; b < slices; b += 32) s += P[(size_t)b * elems + e];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) {
        const size_t i = e % (size_t)rows;
        const size_t j = e / (size_t)rows;
        double *o = out + i + j * (size_t)ldo;
        *o = beta == 0.0 ? alpha * s : alpha * s + beta * *o;
    }
}

int BlockOps::gram(const double *A, long long lda, int ma, const double *B, long long ldb, int mb,
                   int n, double *C, long long ldc, double alpha, double beta)
{
    if (ma <= 0 || mb <= 0) {
        return IPT_CUDA_SUCCESS;
    }
    const int chunks = (n + kGramRows - 1) / kGramRows;
    const int tiles = ((ma + kGramTile - 1) / kGramTile) * ((mb + kGramTile - 1) / kGramTile);
    // ~2 blocks per SM in total, each taking consecutive row chunks
    int blocks_x = (2 * sms + tiles - 1) / tiles;
    if (blocks_x > chunks) blocks_x = chunks;
    if (blocks_x < 1) blocks_x = 1;
    const int per_block = (chunks + blocks_x - 1) / blocks_x;
    blocks_x = (chunks + per_block - 1) / per_block;
    const size_t mm = (size_t)ma * (size_t)mb;
    IPTGB_CHECK(ensure_partials((size_t)blocks_x * mm));
    KernelTimerScope timer(kProfGram, stream);
    if (df_products) {
        IPTGB_CHECK(launch_pdl(gram_partial_df_kernel, dim3(blocks_x, tiles), dim3(256), 0, stream,
                               A, lda, ma, B, ldb, mb, n, per_block, partials));
        IPTGB_CHECK(launch_pdl(reduce_slices_warp_kernel, dim3(blocks_for(mm * 32)),
                               dim3(kThreads), 0, stream, (const double *)partials, blocks_x, mm, C,
                               ldc, ma, alpha, beta));
        return IPT_CUDA_SUCCESS;
    }
    IPTGB_CHECK(launch_pdl(gram_partial_kernel, dim3(blocks_x, tiles), dim3(256), 0, stream, A,
                           lda, ma, B, ldb, mb, n, per_block, partials));
    IPTGB_CHECK(launch_pdl(reduce_slices_kernel, dim3(blocks_for(mm)), dim3(kThreads), 0, stream,
                           (const double *)partials, blocks_x, mm, C, ldc, ma, alpha, beta));
    return IPT_CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------
// Tall-by-small product C = alpha * A B + beta * C
// (A: n x m, B: m x p, C: n x p, column-major).  One row per thread, 32
// output columns per block column; B tile staged in shared memory.
// ---------------------------------------------------------------------------
constexpr int kTallK = 32;
constexpr int kTallThreads = 128;

// TC output columns per thread: fewer columns give more CTAs, so that the
// FP64 pipes of every SM take part when n is only a few thousand rows.
template <int TC>
__global__ void __launch_bounds__(kTallThreads)
    tall_gemm_kernel(const double *__restrict__ A, long long lda, const double *__restrict__ B,
                     long long ldb, double *__restrict__ C, long long ldc, int n, int m, int p,
                     double alpha, double beta)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    __shared__ double bs[kTallK][TC];
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    const int c0 = blockIdx.y * TC;
    double acc[TC];
#pragma unroll
    for (int j = 0; j < TC; ++j) {
        acc[j] = 0.0;
    }
    for (int l0 = 0; l0 < m; l0 += kTallK) {
        __syncthreads();
        for (int e = threadIdx.x; e < kTallK * TC; e += blockDim.x) {
            const int l = e % kTallK;
            const int j = e / kTallK;
            bs[l][j] = (l0 + l < m && c0 + j < p) ? B[(size_t)(l0 + l) + (size_t)(c0 + j) * ldb] : 0.0;
        }
        __syncthreads();
        if (row < n) {
            const int lc = min(kTallK, m - l0);
            // unrolled so that several A loads are in flight per thread
#pragma unroll 8
            for (int l = 0; l < lc; ++l) {
                const double a = A[(size_t)row + (size_t)(l0 + l) * lda];
#pragma unroll
                for (int j = 0; j < TC; ++j) {
                    acc[j] = fma(a, bs[l][j], acc[j]);
                }
            }
        }
    }
    if (row < n) {
#pragma unroll
        for (int j = 0; j < TC; ++j) {
            if (c0 + j < p) {
                double *o = C + (size_t)row + (size_t)(c0 + j) * ldc;
                *o = beta == 0.0 ? alpha * acc[j] : alpha * acc[j] + beta * *o;
            }
        }
    }
}

// tall_gemm_kernel in double-float arithmetic (BlockOps::df_products): the
// B tile split into (hi, lo) floats in shared memory, interleaved so that one
// 16-byte load brings two columns' pairs (every thread of the CTA reads the
// same address: a broadcast), each A entry split once per row and used for TC
// columns.
template <int TC>
__global__ void __launch_bounds__(kTallThreads)
    tall_gemm_df_kernel(const double *__restrict__ A, long long lda, const double *__restrict__ B,
                        long long ldb, double *__restrict__ C, long long ldc, int n, int m, int p,
                        double alpha, double beta)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    __shared__ float4 bs4[kTallK][TC / 2];  // (hi_j, lo_j, hi_j+1, lo_j+1)
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    const int c0 = blockIdx.y * TC;
    float S[TC], sl[TC];
#pragma unroll
    for (int j = 0; j < TC; ++j) {
        S[j] = 0.f;
        sl[j] = 0.f;
    }
    for (int l0 = 0; l0 < m; l0 += kTallK) {
        __syncthreads();
        for (int e = threadIdx.x; e < kTallK * TC / 2; e += blockDim.x) {
            const int l = e % kTallK;
            const int j = 2 * (e / kTallK);
            const bool row_ok = l0 + l < m;
            const dfloat b0 = df_from_double(
                (row_ok && c0 + j < p) ? B[(size_t)(l0 + l) + (size_t)(c0 + j) * ldb] : 0.0);
            const dfloat b1 = df_from_double(
                (row_ok && c0 + j + 1 < p) ? B[(size_t)(l0 + l) + (size_t)(c0 + j + 1) * ldb]
                                           : 0.0);
            bs4[l][j / 2] = make_float4(b0.hi, b0.lo, b1.hi, b1.lo);
        }
        __syncthreads();
        if (row < n) {
            const int lc = min(kTallK, m - l0);
            // groups of 8 A values in flight per thread: enough loads per
            // warp without the register cost of a whole chunk (which limits
            // the resident warps)
#pragma unroll
            for (int g = 0; g < kTallK; g += 8) {
                double av[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    av[u] = g + u < lc ? A[(size_t)row + (size_t)(l0 + g + u) * lda] : 0.0;
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    if (g + u < lc) {
                        const dfloat a = df_from_double(av[u]);
#pragma unroll
                        for (int q = 0; q < TC / 2; ++q) {
                            const float4 b = bs4[g + u][q];
                            df_acc(S[2 * q], sl[2 * q], a.hi, a.lo, b.x, b.y);
                            df_acc(S[2 * q + 1], sl[2 * q + 1], a.hi, a.lo, b.z, b.w);
                        }
                    }
                }
            }
        }
    }
    if (row < n) {
#pragma unroll
        for (int j = 0; j < TC; ++j) {
            if (c0 + j < p) {
                double *o = C + (size_t)row + (size_t)(c0 + j) * ldc;
                const double v = (double)S[j] + (double)sl[j];
                *o = beta == 0.0 ? alpha * v : alpha * v + beta * *o;
            }
        }
    }
}

int BlockOps::tall_gemm(const double *A, long long lda, const double *B, long long ldb, double *C,
                        long long ldc, int n, int m, int p, double alpha, double beta)
{
    if (p <= 0) {
        return IPT_CUDA_SUCCESS;
    }
    const int row_blocks = (n + kTallThreads - 1) / kTallThreads;
    const int want = 2 * std::max(1, sms);
    KernelTimerScope timer(kProfTallGemm, stream);
    // column group: the widest that still gives the grid enough CTAs
    int tc = 0;
    void (*kernel)(const double *, long long, const double *, long long, double *, long long, int,
                   int, int, double, double) = nullptr;
    if (df_products) {
        // several CTAs per SM hide the latency of the double-float chains:
        // narrower column groups until the grid has about four per SM
        if ((long long)row_blocks * ((p + 15) / 16) >= 2 * want) {
            tc = 16;
            kernel = tall_gemm_df_kernel<16>;
        } else if ((long long)row_blocks * ((p + 7) / 8) >= 2 * want) {
            tc = 8;
            kernel = tall_gemm_df_kernel<8>;
        } else {
            tc = 4;
            kernel = tall_gemm_df_kernel<4>;
        }
    } else if ((long long)row_blocks * ((p + 31) / 32) >= want) {
        tc = 32;
        kernel = tall_gemm_kernel<32>;
    } else if ((long long)row_blocks * ((p + 15) / 16) >= want) {
        tc = 16;
        kernel = tall_gemm_kernel<16>;
    } else {
        tc = 8;
        kernel = tall_gemm_kernel<8>;
    }
    return launch_pdl(kernel, dim3(row_blocks, (p + tc - 1) / tc), dim3(kTallThreads), 0, stream,
                      A, lda, B, ldb, C, ldc, n, m, p, alpha, beta);
}

// ---------------------------------------------------------------------------
// One-CTA Cholesky of an m x m SPD matrix G (column-major, ld = m) and the
// inverse of its upper factor: G = R^T R, Rinv = R^{-1} (upper triangular).
// If G is not numerically positive definite, G + shift*I is factored with a
// shift grown from 1e-14 * trace(G) until it succeeds; status[0] gets the
// number of shifts used (0 = plain), or -1 if it never succeeded.
// Dynamic shared memory: 2 * m * m doubles.
// ---------------------------------------------------------------------------
__device__ void chol_inverse_block(const double *__restrict__ G, int m, double *__restrict__ Rinv,
                                   int *status, double *sm)
{
    double *L = sm;          // lower factor, row-major [i*m + j]
    double *W = sm + m * m;  // inverse of L, row-major
    __shared__ int fail;
    __shared__ double shift;
    __shared__ int attempts;
    const int tid = threadIdx.x;
    const int nt = blockDim.x;
    if (tid == 0) {
        double tr = 0.0;
        for (int i = 0; i < m; ++i) {
            tr += fabs(G[(size_t)i * m + i]);
        }
        shift = 0.0;
        attempts = 0;
        // remember the trace for shift growth
        W[0] = tr > 0.0 ? tr : 1.0;
    }
    __syncthreads();
    const double trace = W[0];
    for (;;) {
        for (int e = tid; e < m * m; e += nt) {
            const int i = e / m;
            const int j = e % m;
            L[e] = G[(size_t)j * m + i] + (i == j ? shift : 0.0);
        }
        if (tid == 0) {
            fail = 0;
        }
        __syncthreads();
        for (int j = 0; j < m; ++j) {
            if (tid == 0) {
                const double a = L[j * m + j];
                if (!(a > 0.0) || !isfinite(a)) {
                    fail = 1;
                } else {
                    L[j * m + j] = sqrt(a);
                }
            }
            __syncthreads();
            if (fail) {
                break;
            }
            const double ljj = L[j * m + j];
            for (int i = j + 1 + tid; i < m; i += nt) {
                L[i * m + j] /= ljj;
            }
            __syncthreads();
            // trailing update of the lower triangle: L[i][l] -= L[i][j] L[l][j], j < l <= i
            const int rem = m - j - 1;
            for (int e = tid; e < rem * rem; e += nt) {
                const int i = j + 1 + e / rem;
                const int l = j + 1 + e % rem;
                if (l <= i) {
                    L[i * m + l] -= L[i * m + j] * L[l * m + j];
                }
            }
            __syncthreads();
        }
        if (!fail) {
            break;
        }
        __syncthreads();
        if (tid == 0) {
            attempts += 1;
            shift = shift == 0.0 ? 1e-14 * trace : shift * 100.0;
        }
        __syncthreads();
        if (attempts > 12) {
            if (tid == 0) {
                status[0] = -1;
            }
            return;
        }
    }
    // W = L^{-1} by forward substitution, one column per thread.
    for (int c = tid; c < m; c += nt) {
        for (int i = 0; i < m; ++i) {
            double v = (i == c) ? 1.0 : 0.0;
            for (int l = c; l < i; ++l) {
                v -= L[i * m + l] * W[l * m + c];
            }
            W[i * m + c] = i < c ? 0.0 : v / L[i * m + i];
        }
    }
    __syncthreads();
    // R = L^T, so R^{-1} = (L^{-1})^T: Rinv[i][j] = W[j][i]; column-major out.
    for (int e = tid; e < m * m; e += nt) {
        const int i = e % m;
        const int j = e / m;
        Rinv[(size_t)j * m + i] = W[j * m + i];
    }
    if (tid == 0) {
        status[0] = attempts;
    }
}

__global__ void chol_inverse_kernel(const double *__restrict__ G, int m, double *__restrict__ Rinv,
                                    int *status, double *cond_bound)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    extern __shared__ double sm[];
    chol_inverse_block(G, m, Rinv, status, sm);
    if (cond_bound != nullptr && threadIdx.x == 0) *cond_bound = NAN;  // not estimated here
}


// ---------------------------------------------------------------------------
// Cholesky + inverse for m <= 32 with one thread per matrix entry (1024
// threads, 32 x 32 padded to the identity beyond m): the same right-looking
// factorisation as chol_inverse_block, then the column-oriented forward
// substitution W = L^{-1}; two barriers per column.  GB300's FP64 pipe
// holds its partition for 64 cycles per warp instruction, so spreading the
// trailing updates over all 32 warps (all four partitions) instead of one
// warp is what makes the kernel fast.  Arithmetic T: double (FP64, the
// divisions of chol_inverse_block) or dfloat (double-float on the FP32 pipe,
// about 48 bits, with the pivot reciprocal formed once).  A matrix that
// needs a diagonal shift goes through chol_inverse_block (FP64, its shift
// retries and status) instead.
// ---------------------------------------------------------------------------
struct CholF64 {
    typedef double T;
    static __device__ __forceinline__ T load(double v) { return v; }
    static __device__ __forceinline__ T value(float v) { return (double)v; }
    static __device__ __forceinline__ bool positive(T v) { return v > 0.0 && isfinite(v); }
    static __device__ __forceinline__ T sqrt_(T v) { return sqrt(v); }
    static __device__ __forceinline__ T scale(T a, T piv, T) { return a / piv; }
    static __device__ __forceinline__ T fms(T a, T x, T y) { return a - x * y; }
    static __device__ __forceinline__ T recip(T) { return 0.0; }  // unused: divides
    static __device__ __forceinline__ double store(T v) { return v; }
    static __device__ __forceinline__ float lead(T v) { return (float)v; }
};

struct CholDF {
    typedef dfloat T;
    static __device__ __forceinline__ T load(double v) { return df_from_double(v); }
    static __device__ __forceinline__ T value(float v) { return {v, 0.0f}; }
    static __device__ __forceinline__ bool positive(T v) { return v.hi > 0.0f && isfinite(v.hi); }
    static __device__ __forceinline__ T sqrt_(T v) { return df_sqrt(v); }
    static __device__ __forceinline__ T scale(T a, T, T inv) { return df_mul(a, inv); }
    static __device__ __forceinline__ T fms(T a, T x, T y) { return df_sub(a, df_mul(x, y)); }
    static __device__ __forceinline__ T recip(T v) { return df_recip(v); }
    static __device__ __forceinline__ double store(T v) { return df_to_double(v); }
    static __device__ __forceinline__ float lead(T v) { return v.hi; }
};

template <typename Ops>
__global__ void __launch_bounds__(1024)
    chol_inverse32x32_kernel(const double *__restrict__ G, int m, double *__restrict__ Rinv,
                             int *status, double *cond_bound)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    typedef typename Ops::T T;
    __shared__ T col[32];      // the current column of L
    __shared__ T piv[2];       // pivot and its reciprocal
    __shared__ T Ls[32][33];   // L after the factorisation
    __shared__ T Wrow[32];     // the current row of W
    __shared__ float red[32];
    __shared__ int fail;
    const int tid = threadIdx.x;
    const int r = tid >> 5;  // row
    const int c = tid & 31;  // column
    T a = (r < m && c < m) ? Ops::load(G[(size_t)c * m + r]) : Ops::value(r == c ? 1.0f : 0.0f);
    if (tid == 0) fail = 0;
    if (cond_bound != nullptr) {
        // e = ||D^{-1/2} G D^{-1/2} - I||_F (D = diag G): the eigenvalues of
        // the unit-diagonal G lie in [1 - e, 1 + e], so its condition number
        // (which governs the orthogonality CholQR leaves) is at most
        // (1 + e) / (1 - e); a few digits suffice, so FP32
        const float grr = (float)G[(size_t)min(r, m - 1) * (m + 1)];
        const float gcc = (float)G[(size_t)min(c, m - 1) * (m + 1)];
        const float g = Ops::lead(a);
        float t = (r != c && r < m && c < m) ? g * g / (grr * gcc) : 0.0f;
        const bool bad = r == c && r < m && !(grr > 0.0f);
        for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
        const bool wbad = __any_sync(0xffffffffu, bad);
        if (c == 0) red[r] = wbad ? INFINITY : t;
        __syncthreads();
        if (r == 0) {
            float v = red[c];
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (c == 0) {
                const double e = sqrt((double)v);
                *cond_bound = e < 1.0 ? (1.0 + e) / (1.0 - e) : INFINITY;  // NaN/inf: INFINITY
            }
        }
    }
    __syncthreads();
    for (int j = 0; j < 32; ++j) {
        if (r == j && c == j) {
            if (!Ops::positive(a)) {
                fail = 1;
                a = Ops::value(1.0f);
            }
            a = Ops::sqrt_(a);
            piv[0] = a;
            piv[1] = Ops::recip(a);
        }
        __syncthreads();
        if (fail) break;  // uniform: read after the barrier
        if (c == j && r > j) {
            a = Ops::scale(a, piv[0], piv[1]);
            col[r] = a;
        }
        __syncthreads();
        if (c > j && r >= c) a = Ops::fms(a, col[r], col[c]);
    }
    if (fail) {
        __shared__ double sm[2 * 32 * 32];
        __syncthreads();
        chol_inverse_block(G, m, Rinv, status, sm);
        if (cond_bound != nullptr && tid == 0) *cond_bound = NAN;  // shifted: not estimated
        return;
    }
    Ls[r][c] = a;
    // W = L^{-1}, thread (r, c) holds W[r][c]; column-oriented substitution
    T w = Ops::value(r == c ? 1.0f : 0.0f);
    __syncthreads();
    for (int l = 0; l < 32; ++l) {
        if (r == l) {
            w = Ops::scale(w, Ls[l][l], Ops::recip(Ls[l][l]));
            Wrow[c] = w;
        }
        __syncthreads();
        if (r > l) w = Ops::fms(w, Ls[r][l], Wrow[c]);
        __syncthreads();
    }
    // R^{-1} = W^T (upper triangular), column-major: Rinv[c + r m] = W[r][c]
    if (r < m && c < m) Rinv[(size_t)r * m + c] = r < c ? 0.0 : Ops::store(w);
    if (tid == 0) status[0] = 0;
}

// ---------------------------------------------------------------------------
// Residual block R = AX - X diag(theta) and per-column partial sums of
// ||r_j||^2, ||x_j||^2.  Grid: (row chunks, k).  Partials [chunk][k][2].
// ---------------------------------------------------------------------------
__global__ void residual_partial_kernel(const double *__restrict__ X, const double *__restrict__ AX,
                                        const double *__restrict__ theta, int n, long long ldx,
                                        double *__restrict__ R, int rows_per_block,
                                        double2 *__restrict__ P)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const int j = blockIdx.y;
    const int r0 = blockIdx.x * rows_per_block;
    const int r1 = min(n, r0 + rows_per_block);
    const double th = theta[j];
    double rs = 0.0, xs = 0.0;
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const size_t idx = (size_t)i + (size_t)j * ldx;
        const double x = X[idx];
        const double r = AX[idx] - x * th;
        R[(size_t)i + (size_t)j * n] = r;
        rs = fma(r, r, rs);
        xs = fma(x, x, xs);
    }
    double2 t = block_sum2(rs, xs);
    if (threadIdx.x == 0) {
        P[(size_t)blockIdx.x * gridDim.y + j] = t;
    }
}

// norms[j] = (||r_j||, ||x_j||), scaled[j] = ||r_j|| / (max(1,hnorm) max(1,||x_j||))
// (scaling of IPT_C_GPU/src/ipt_cuda.cu:2684-2697).
__global__ void residual_finish_kernel(const double2 *__restrict__ P, int chunks, int k,
                                       double hnorm, double *__restrict__ rnorm,
                                       double *__restrict__ scaled)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k) {
        return;
    }
    double rs = 0.0, xs = 0.0;
    for (int c = 0; c < chunks; ++c) {
        const double2 p = P[(size_t)c * k + j];
        rs += p.x;
        xs += p.y;
    }
    const double r = sqrt(rs);
    const double x = sqrt(xs);
    rnorm[j] = r;
    scaled[j] = r / (fmax(1.0, hnorm) * fmax(1.0, x));
}

int BlockOps::residuals(const double *X, const double *AX, const double *theta, int n, int k,
                        long long ldx, double hnorm, double *R, double *rnorm, double *scaled)
{
    const int rows_per_block = 2048;
    const int chunks = (n + rows_per_block - 1) / rows_per_block;
    IPTGB_CHECK(ensure_partials((size_t)chunks * k * 2));
    IPTGB_CHECK(launch_pdl(residual_partial_kernel, dim3(chunks, k), dim3(256), 0, stream, X, AX,
                           theta, n, ldx, R, rows_per_block, (double2 *)partials));
    IPTGB_CHECK(launch_pdl(residual_finish_kernel, dim3(blocks_for(k)), dim3(kThreads), 0, stream,
                           (const double2 *)partials, chunks, k, hnorm, rnorm, scaled));
    return IPT_CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------
// Diagonal Davidson correction for the selected Ritz pairs:
//   T[:, c] = R[:, sel[c]] / clip(d_i - theta_sel[c])
// with |denominator| clipped below at `clip` keeping its sign
// (IPT_C_GPU/src/ipt_cuda.cu:2449-2465, clip rule :3389-3403).
// ---------------------------------------------------------------------------
__global__ void diag_correction_kernel(const double *__restrict__ R, const double *__restrict__ d,
                                       const double *__restrict__ theta, const int *__restrict__ sel,
                                       int nsel, int n, double clip, double *__restrict__ T)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)n * (size_t)nsel) {
        return;
    }
    const int i = (int)(idx % (size_t)n);
    const int c = (int)(idx / (size_t)n);
    const int j = sel[c];
    double den = d[i] - theta[j];
    if (fabs(den) < clip) {
        den = den < 0.0 ? -clip : clip;
    }
    T[idx] = R[(size_t)i + (size_t)j * n] / den;
}

int BlockOps::diag_correction(const double *R, const double *d, const double *theta,
                              const int *sel, int nsel, int n, double clip, double *T)
{
    diag_correction_kernel<<<blocks_for((size_t)n * nsel), kThreads, 0, stream>>>(
        R, d, theta, sel, nsel, n, clip, T);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

// Column norms of an n x c block (2-pass deterministic).
__global__ void colnorm_partial_kernel(const double *__restrict__ A, long long lda, int n,
                                       int rows_per_block, double *__restrict__ P)
{
    const int j = blockIdx.y;
    const int r0 = blockIdx.x * rows_per_block;
    const int r1 = min(n, r0 + rows_per_block);
    double s = 0.0;
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        const double a = A[(size_t)i + (size_t)j * lda];
        s = fma(a, a, s);
    }
    double2 t = block_sum2(s, 0.0);
    if (threadIdx.x == 0) {
        P[(size_t)blockIdx.x * gridDim.y + j] = t.x;
    }
}

__global__ void colnorm_finish_kernel(const double *__restrict__ P, int chunks, int c,
                                      double *__restrict__ out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= c) {
        return;
    }
    double s = 0.0;
    for (int b = 0; b < chunks; ++b) {
        s += P[(size_t)b * c + j];
    }
    out[j] = sqrt(s);
}

int BlockOps::column_norms(const double *A, long long lda, int n, int c, double *out)
{
    const int rows_per_block = 2048;
    const int chunks = (n + rows_per_block - 1) / rows_per_block;
    IPTGB_CHECK(ensure_partials((size_t)chunks * c));
    colnorm_partial_kernel<<<dim3(chunks, c), 256, 0, stream>>>(A, lda, n, rows_per_block,
                                                                partials);
    IPTGB_LAUNCH();
    colnorm_finish_kernel<<<blocks_for(c), kThreads, 0, stream>>>(partials, chunks, c, out);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

// Gather/scale columns: dst[:, c] = src[:, idx[c]] * (scale ? scale[c] : 1).
__global__ void gather_columns_kernel(const double *__restrict__ src, long long lds,
                                      const int *__restrict__ idx, const double *__restrict__ scale,
                                      int n, int c, double *__restrict__ dst, long long ldd)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n * (size_t)c) {
        return;
    }
    const int i = (int)(e % (size_t)n);
    const int j = (int)(e / (size_t)n);
    const double s = scale != nullptr ? scale[j] : 1.0;
    dst[(size_t)i + (size_t)j * ldd] = src[(size_t)i + (size_t)idx[j] * lds] * s;
}

int BlockOps::gather_columns(const double *src, long long lds, const int *idx, const double *scale,
                             int n, int c, double *dst, long long ldd)
{
    if (c <= 0) {
        return IPT_CUDA_SUCCESS;
    }
    gather_columns_kernel<<<blocks_for((size_t)n * c), kThreads, 0, stream>>>(src, lds, idx, scale,
                                                                           n, c, dst, ldd);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------
// Incremental Rayleigh-Ritz projection.  Tf (ld) holds T = V^T (H V) of the
// current basis.  After c columns are appended at m0, B = V[:, :m0+c]^T
// (H V)[:, m0:m0+c] (ld m0+c) fills the new border of T: rows i < m0 are
// mirrored into the new rows, the new c x c block is symmetrised.
// ---------------------------------------------------------------------------
__global__ void proj_insert_kernel(const double *__restrict__ B, int m0, int c,
                                   double *__restrict__ Tf, int ld)
{
    const int mt = m0 + c;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= mt * c) return;
    const int j = e / mt;  // new column
    const int i = e - j * mt;
    const double b = B[e];
    if (i < m0) {
        Tf[(size_t)(m0 + j) * ld + i] = b;
        Tf[(size_t)i * ld + m0 + j] = b;
    } else {
        const int ii = i - m0;
        Tf[(size_t)(m0 + j) * ld + i] = 0.5 * (b + B[(size_t)ii * mt + m0 + j]);
    }
}

// Tm (ld m) = Tf[:m, :m]
__global__ void proj_compact_kernel(const double *__restrict__ Tf, int ld, int m,
                                    double *__restrict__ Tm)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m * m) return;
    const int j = e / m;
    const int i = e - j * m;
    Tm[e] = Tf[(size_t)j * ld + i];
}

// Tf[:m, :m] = diag(theta[:m]): the projection onto V Z of the Ritz vectors
__global__ void proj_diag_kernel(const double *__restrict__ theta, int m, double *__restrict__ Tf,
                                 int ld)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m * m) return;
    const int j = e / m;
    const int i = e - j * m;
    Tf[(size_t)j * ld + i] = i == j ? theta[i] : 0.0;
}

int BlockOps::proj_insert(const double *B, int m0, int c, double *Tf, int ld)
{
    proj_insert_kernel<<<blocks_for((size_t)(m0 + c) * c), kThreads, 0, stream>>>(B, m0, c, Tf, ld);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

int BlockOps::proj_compact(const double *Tf, int ld, int m, double *Tm)
{
    proj_compact_kernel<<<blocks_for((size_t)m * m), kThreads, 0, stream>>>(Tf, ld, m, Tm);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

int BlockOps::proj_diag(const double *theta, int m, double *Tf, int ld)
{
    proj_diag_kernel<<<blocks_for((size_t)m * m), kThreads, 0, stream>>>(theta, m, Tf, ld);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

int BlockOps::chol_inverse(const double *G, int m, double *Rinv, int *status_dev, double *cond_bound,
                           bool df)
{
    if (m <= 32) {
        return launch_pdl(df ? chol_inverse32x32_kernel<CholDF> : chol_inverse32x32_kernel<CholF64>,
                          dim3(1), dim3(1024), 0, stream, G, m, Rinv, status_dev, cond_bound);
    }
    const size_t smem = 2 * (size_t)m * (size_t)m * sizeof(double);
    if (smem > 200 * 1024) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    IPTGB_CUDA(cudaFuncSetAttribute(chol_inverse_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return launch_pdl(chol_inverse_kernel, dim3(1), dim3(256), smem, stream, G, m, Rinv,
                      status_dev, cond_bound);
}

int BlockOps::ensure_partials(size_t count)
{
    if (count <= partials_capacity) {
        return IPT_CUDA_SUCCESS;
    }
    if (partials != nullptr) {
        cudaFreeAsync(partials, stream);
        partials = nullptr;
    }
    size_t want = count < (size_t)1 << 16 ? (size_t)1 << 16 : count;
    IPTGB_CUDA(cudaMallocAsync((void **)&partials, want * sizeof(double), stream));
    partials_capacity = want;
    return IPT_CUDA_SUCCESS;
}

void BlockOps::release()
{
    if (partials != nullptr) {
        cudaFreeAsync(partials, stream);
        partials = nullptr;
        partials_capacity = 0;
    }
    if (eig_scratch != nullptr) {
        cudaFreeAsync(eig_scratch, stream);
        eig_scratch = nullptr;
        eig_capacity = 0;
    }
}

}  // namespace iptgb
