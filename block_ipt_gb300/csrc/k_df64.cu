// k_df64.cu - FP64-accurate dense block product on the FP32 pipe.
//
// GB300 retires FP32 FMAs at 64x its FP64 rate, so the accurate products of
// the mixed-precision solve (the FP64 defect HX of the refinement and the
// final certification; the reference forms these with cublasDgemm,
// IPT_C_GPU/src/ipt_cuda.cu:1649,1888) are computed in double-FP32
// ("double-float") arithmetic: H and X are held as unevaluated sums of two
// floats, hi + lo (H split once per solve, X per product), and every term
//   h x = hh xh + (hh xl + hl xh) + O(2^-48 |h x|)
// is formed with an exact two-product (p = hh xh, e = fma(hh, xh, -p)) and
// added to a double-float accumulator (S, s) with an exact two-sum
// (Knuth), ~12 FP32 operations per term.  The result carries ~48 bits, far
// below the 1e-8 eigen-residual the products certify; the split-K layout
// and the FP64 partial sums are those of the FP64 kernel (k_dense64.cu).
#include <string.h>

#include <algorithm>

#include "common.cuh"
#include "dfloat.cuh"
#include "fpconv.cuh"
#include "kernels.cuh"

namespace iptgb {

constexpr int kDfRows = 256;
constexpr int kDfChunk = 32;

// hi = float(a), lo = float(a - hi)
__global__ void df_split_kernel(const double *__restrict__ A, size_t count,
                                float *__restrict__ hi, float *__restrict__ lo)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    const double a = A[e];
    uint32_t hb, lb;
    if (split_double_bits((unsigned long long)__double_as_longlong(a), &hb, &lb)) {
        hi[e] = __uint_as_float(hb);
        lo[e] = __uint_as_float(lb);
    } else {
        const float h = __double2float_rn(a);
        hi[e] = h;
        lo[e] = __double2float_rn(a - (double)h);
    }
}

__device__ __forceinline__ void df_term(float &S, float &s, float hh, float hl, float xh, float xl)
{
    df_acc(S, s, hh, hl, xh, xl);
}

// Split-K partial product, one output row per thread, BN columns in
// double-float registers; X chunk (hi, lo) staged in shared memory.
// P[slice][column][row] = the slice's partial sum as a double-float pair
// (float2 hi, lo; summed by df_sum_partials_kernel).
// Three CTAs per SM for BN <= 16 (80 registers, no spills): six warps per
// scheduler hide the latency of the H loads and of the staging barrier
// better than four.
template <int BN>
__global__ void __launch_bounds__(kDfRows, BN <= 16 ? 3 : 1)
df64_partial_kernel(const float *__restrict__ Hh, const float *__restrict__ Hl, int n,
                    long long ldh, const float *__restrict__ Xh, const float *__restrict__ Xl,
                    long long ldx, int k, float2 *__restrict__ P, int kslice)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    __shared__ float xsh[kDfChunk][BN];
    __shared__ float xsl[kDfChunk][BN];
    const int row = blockIdx.x * kDfRows + threadIdx.x;
    const int sl = blockIdx.y;
    const int c0 = blockIdx.z * BN;
    const int kbeg = sl * kslice;
    const int kend = min(n, kbeg + kslice);
    float S[BN], s[BN];
#pragma unroll
    for (int j = 0; j < BN; ++j) {
        S[j] = 0.f;
        s[j] = 0.f;
    }
    const bool active = row < n;
    const size_t rofs = active ? (size_t)row : 0;
    for (int l0 = kbeg; l0 < kend; l0 += kDfChunk) {
        const int lc = min(kDfChunk, kend - l0);
        __syncthreads();
        for (int e = threadIdx.x; e < kDfChunk * BN; e += kDfRows) {
            const int ll = e % kDfChunk;
            const int j = e / kDfChunk;
            float vh = 0.f, vl = 0.f;
            if (ll < lc && c0 + j < k) {
                const size_t o = (size_t)(l0 + ll) + (size_t)(c0 + j) * (size_t)ldx;
                vh = Xh[o];
                vl = Xl[o];
            }
            xsh[ll][j] = vh;
            xsl[ll][j] = vl;
        }
        __syncthreads();
        if (active) {
#pragma unroll 4
            for (int ll = 0; ll < lc; ++ll) {
                const size_t o = rofs + (size_t)(l0 + ll) * (size_t)ldh;
                const float hh = __ldg(Hh + o);
                const float hl = __ldg(Hl + o);
#pragma unroll
                for (int j = 0; j < BN; ++j) df_term(S[j], s[j], hh, hl, xsh[ll][j], xsl[ll][j]);
            }
        }
    }
    if (active) {
#pragma unroll
        for (int j = 0; j < BN; ++j) {
            if (c0 + j < k) {
                P[((size_t)sl * (size_t)k + (size_t)(c0 + j)) * (size_t)n + row] =
                    make_float2(S[j], s[j]);
            }
        }
    }
}

// Y = sum over the S double-float slices (fixed order, accurate double-float
// additions on the FP32 pipe), then one conversion to FP64 per entry.
__global__ void df_sum_partials_kernel(const float2 *__restrict__ P, int S, size_t elems,
                                       double *__restrict__ Y)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= elems) return;
    const float2 p0 = P[idx];
    dfloat y = {p0.x, p0.y};
    for (int sl = 1; sl < S; ++sl) {
        const float2 p = P[(size_t)sl * elems + idx];
        y = df_add(y, dfloat{p.x, p.y});
    }
    Y[idx] = df_to_double(y);
}

int launch_df_sum_partials(const double *P, int S, size_t elems, double *Y, cudaStream_t stream)
{
    if (S <= 0 || elems == 0) return IPT_CUDA_SUCCESS;
    IPTGB_CHECK(launch_pdl(df_sum_partials_kernel, dim3(blocks_for(elems)), dim3(kThreads), 0,
                           stream, reinterpret_cast<const float2 *>(P), S, elems, Y));
    return IPT_CUDA_SUCCESS;
}

int launch_df_split(const double *A, size_t count, float *hi, float *lo, cudaStream_t stream)
{
    IPTGB_CHECK(launch_pdl(df_split_kernel, dim3(blocks_for(count)), dim3(kThreads), 0, stream, A,
                           count, hi, lo));
    return IPT_CUDA_SUCCESS;
}

static int df64_tile_width(int k)
{
    int bn = k <= 8 ? 8 : 16;
    const int over = env_int("IPT_GB300_DF_BN", 0);  // tuning override: 8, 16 or 32
    if (over == 8 || over == 16 || over == 32) bn = over;
    return bn;
}

int df64_split_for(int n, int k, int sms)
{
    // K slices so that the grid is a whole number of waves of the resident
    // CTAs (3 per SM at BN <= 16): two waves by default (tuning knob
    // IPT_GB300_DF_WAVES), slices at least 64 deep
    const int bn = df64_tile_width(k);
    const int row_blocks = (n + kDfRows - 1) / kDfRows;
    const int tiles = row_blocks * ((k + bn - 1) / bn);
    const int per_sm = bn <= 16 ? 3 : 1;
    const int waves = std::max(1, env_int("IPT_GB300_DF_WAVES", 2));
    int S = (waves * per_sm * std::max(1, sms)) / std::max(1, tiles);
    S = std::min(S, std::max(1, n / 64));
    return std::max(1, S);
}

int launch_df64_partial(const float *Hh, const float *Hl, int n, long long ldh, const float *Xh,
                        const float *Xl, long long ldx, int k, double *P, int S,
                        cudaStream_t stream)
{
    int kslice = (n + S - 1) / S;
    kslice = ((kslice + kDfChunk - 1) / kDfChunk) * kDfChunk;
    const int row_blocks = (n + kDfRows - 1) / kDfRows;
    // 16-column tiles also for wider blocks: H is re-read per tile (from L2 /
    // HBM, cheap next to the FP32 work) but 80 instead of 148 registers let
    // three CTAs share an SM (measured faster at n = 8192, k = 32)
    const int bn = df64_tile_width(k);
    dim3 grid(row_blocks, S, (k + bn - 1) / bn);
    // the double-float partials (float2) fill the same bytes as FP64 ones
    float2 *P2 = reinterpret_cast<float2 *>(P);
    auto kernel = bn == 8 ? df64_partial_kernel<8>
                  : bn == 16 ? df64_partial_kernel<16>
                             : df64_partial_kernel<32>;
    return launch_pdl(kernel, grid, dim3(kDfRows), 0, stream, Hh, Hl, n, ldh, Xh, Xl, ldx, k, P2,
                      kslice);
}

}  // namespace iptgb

#define IPT_API extern "C" __attribute__((visibility("default")))

// hi = RN_float(a), lo = RN_float(a - hi) for `count` doubles on the device
// (the double-FP32 operands of the FP64-accurate products).
IPT_API int ipt_block_split_double(const double *d_in, long long count, float *d_hi, float *d_lo,
                                   void *stream)
{
    if (count < 0 || (count > 0 && (d_in == nullptr || d_hi == nullptr || d_lo == nullptr))) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    if (count == 0) return IPT_CUDA_SUCCESS;
    return iptgb::launch_df_split(d_in, (size_t)count, d_hi, d_lo, (cudaStream_t)stream);
}

// The same split on the host, through the same integer-pipe helper (the
// device kernels' conversion restated for checking on machines without a GPU).
IPT_API int ipt_block_split_double_host(const double *in, long long count, float *hi, float *lo)
{
    if (count < 0 || (count > 0 && (in == nullptr || hi == nullptr || lo == nullptr))) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    for (long long e = 0; e < count; ++e) {
        uint64_t b;
        memcpy(&b, &in[e], sizeof(b));
        uint32_t hb, lb;
        if (iptgb::split_double_bits(b, &hb, &lb)) {
            memcpy(&hi[e], &hb, sizeof(float));
            memcpy(&lo[e], &lb, sizeof(float));
        } else {
            const float h = (float)in[e];
            hi[e] = h;
            lo[e] = (float)(in[e] - (double)h);
        }
    }
    return IPT_CUDA_SUCCESS;
}
