// k_oz.cu - FP64-accurate block product Y = H X on the FP16 tensor cores.
//
// Replaces the reference's FP64 cublasDgemm of the mixed refinement
// (IPT_C_GPU/src/mixed_precision/ipt_mixed_precision_cuda.cu:917,958) and of
// the Rayleigh-Ritz products.  H = D + Delta: the diagonal part is applied
// in FP64, Delta X by the split-operand scheme of oz.cuh:
//
//  * Delta is split once per matrix into kOzSlices FP16 digit slices
//    A_s (row-major, K-major for the MMA, [slice][row][ldp]) with one
//    exponent per row; X is split per product into B_t ([slice][col][ldp]
//    concatenated as 6 * cp rows, cp = columns padded to 16) with one
//    exponent per column (oz_slice_x_kernel);
//  * oz_product_kernel is persistent: one CTA per SM walks a contiguous range
//    of (128-row tile, 128-element K period) items.  Warp 4 streams the A
//    slices (each byte of A is read once per product, L2 evict_first) and
//    the B chunk through TMA into shared memory; warp 5 issues tcgen05.mma:
//    per A slice s and K step one MMA of N = (6 - s) cp (two above N = 256)
//    that adds every pair (s, t), t <= 5 - s, into the TMEM accumulator of
//    level s + t (the B slices are consecutive rows, the level accumulators
//    consecutive columns).  One thread issues every MMA of the SM and each
//    issue costs it about 50-65 cycles whatever N, so the kernel issues as
//    few and as wide MMAs as the level structure allows (24 per 64-element K
//    chunk; one per pair took 84).  Two accumulator sets when they fit in
//    TMEM, so the MMAs of the next period run while the last one drains;
//    warps 0-3 drain the six level
//    accumulators after every period, combine them in double-float
//    arithmetic and keep a running sum per (row, column) until the CTA
//    leaves the tile, then write one FP64 partial per (tile, CTA);
//  * oz_finish_kernel adds the partials of each tile in a fixed order,
//    scales by 2^(e_i + f_c - 16) and adds d_i X_ic.
//
// Every mbarrier wait is bounded; a timeout sets the error flag, the CTA
// drains its own copies and MMAs (bounded), frees TMEM and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <climits>

#include "common.cuh"
#include "ipt_plain.h"
#include "kernels.cuh"
#include "oz.cuh"
#include "oz_product.h"
#include "tcgen05.cuh"

namespace iptgb {

namespace oz {

constexpr int kBM = 128;                      // UMMA M: rows per tile
constexpr int kChunk = 64;                    // K elements per TMA chunk (128 B of FP16)
constexpr uint32_t kABytes = kBM * 128;       // one slice of one chunk: 16 KB
constexpr int kThreads = 192;                 // warps 0-3 epilogue, 4 producer, 5 MMA
constexpr int kProducerWarp = 4;
constexpr int kMmaWarp = 5;
constexpr int kMaxASlots = 12;  // A ring depth (slices in flight), set by the shared memory left
constexpr int kMaxBSlots = 2;   // B ring depth (chunks)
constexpr int kChunksPerPeriod = kOzPeriod / kChunk;

struct Params {
    int n, C, cp;
    int a_slots;   // A ring depth
    int b_slots;   // B ring depth
    int acc_bufs;  // TMEM accumulator sets (2: the epilogue drains one while the MMAs fill the other)
    int nchunks, periods;
    long long items;
    int maxslots;
    uint32_t b_bytes;
    uint32_t idesc;  // M = 128, N = cp, FP16 x FP16 -> FP32
};

using tc::owner_of;

using tc::mbar_arrive;

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

template <int CP>
__global__ void __launch_bounds__(kThreads, 1)
oz_product_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  const __grid_constant__ Params prm, double *__restrict__ P, int *err)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
    const int kBSlots = prm.b_slots;
    const int kASlots = prm.a_slots;
    uint8_t *a_ring = smem;
    uint8_t *b_ring = smem + (size_t)kASlots * kABytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(b_ring + (size_t)kBSlots * prm.b_bytes);
    uint32_t *tmem_slot =
        reinterpret_cast<uint32_t *>(bars + 2 * kMaxASlots + 2 * kMaxBSlots + 5);
    __shared__ volatile int abort_flag;
    __shared__ int a_issued, b_issued;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const long long G = gridDim.x;
    const long long it0 = (long long)blockIdx.x * prm.items / G;
    const long long it1 = ((long long)blockIdx.x + 1) * prm.items / G;
    const uint32_t bar0 = tc::smem_u32(bars);
    auto a_full = [&](int q) { return bar0 + 8u * (uint32_t)q; };
    auto a_empty = [&](int q) { return bar0 + 8u * (uint32_t)(kMaxASlots + q); };
    auto b_full = [&](int q) { return bar0 + 8u * (uint32_t)(2 * kMaxASlots + q); };
    auto b_empty = [&](int q) {
        return bar0 + 8u * (uint32_t)(2 * kMaxASlots + kMaxBSlots + q);
    };
    // acc_full(b), acc_empty(b) for the accumulator sets b = 0, 1; mma_done
    const uint32_t acc_base = bar0 + 8u * (uint32_t)(2 * kMaxASlots + 2 * kMaxBSlots);
    auto acc_full = [&](int b) { return acc_base + 8u * (uint32_t)b; };
    auto acc_empty = [&](int b) { return acc_base + 16u + 8u * (uint32_t)b; };
    const uint32_t mma_done = acc_base + 32u;
    const uint32_t a_base = tc::smem_u32(a_ring);
    const uint32_t b_base = tc::smem_u32(b_ring);

    if (threadIdx.x == 0) {
        for (int q = 0; q < kASlots; ++q) {
            tc::mbar_init(a_full(q), 1);
            tc::mbar_init(a_empty(q), 1);
        }
        for (int q = 0; q < kBSlots; ++q) {
            tc::mbar_init(b_full(q), 1);
            tc::mbar_init(b_empty(q), 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(acc_full(b), 1);
            tc::mbar_init(acc_empty(b), 4);  // one arrival per epilogue warp
        }
        tc::mbar_init(mma_done, 1);
        abort_flag = 0;
        a_issued = 0;
        b_issued = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == kProducerWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         tc::smem_u32(tmem_slot)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == kProducerWarp && lane == 0) {
        // ---- TMA producer: per chunk the B chunk, then the six A slices ----
        const uint64_t pol = tc::l2_stream_policy();
        int ac = 0, bc = 0;
        int aq = 0, bq = 0;            // ring slots of copy ac / bc
        uint32_t apar = 0, bpar = 0;   // parities of their rounds
        bool waited = false;
        for (long long it = it0; it < it1 && !abort_flag; ++it) {
            const int tile = (int)(it / prm.periods);
            const int per = (int)(it % prm.periods);
            const int c0 = per * kChunksPerPeriod;
            const int c1 = min(prm.nchunks, c0 + kChunksPerPeriod);
            for (int c = c0; c < c1 && !abort_flag; ++c) {
                if (!waited) {
                    // Delta's slices do not depend on the preceding kernel: the
                    // first chunk's slices are requested before waiting for the
                    // grid that wrote the X slices
                    for (int s = 0; s < kOzSlices; ++s) {
                        tc::mbar_expect_tx(a_full(s), kABytes);
                        tc::tma_load_3d_hint(a_base + (uint32_t)s * kABytes, &tmA, c * kChunk,
                                             tile * kBM, s, a_full(s), pol);
                    }
                    ac = kOzSlices;
                    aq = kOzSlices % kASlots;
                    apar = kOzSlices >= kASlots ? 1u : 0u;
                    pdl_wait();
                    waited = true;
                    const uint32_t dst = b_base;
                    tc::mbar_expect_tx(b_full(0), prm.b_bytes);
                    tc::tma_load_2d(dst, &tmB, c * kChunk, 0, b_full(0));
                    tc::tma_load_2d(dst + (uint32_t)(3 * CP * 128), &tmB, c * kChunk, 3 * CP,
                                    b_full(0));
                    bc = 1;
                    bq = 1 % kBSlots;
                    bpar = kBSlots == 1 ? 1u : 0u;
                    continue;
                }
                {
                    // slot bq of the B ring, round bc / kBSlots (kept incrementally:
                    // this one thread issues every copy of the SM)
                    if (bc >= kBSlots &&
                        !tc::mbar_wait(b_empty(bq), bpar ^ 1u, err, 12, false)) {
                        abort_flag = 1;
                        break;
                    }
                    const uint32_t dst = b_base + (uint32_t)bq * prm.b_bytes;
                    tc::mbar_expect_tx(b_full(bq), prm.b_bytes);
                    tc::tma_load_2d(dst, &tmB, c * kChunk, 0, b_full(bq));
                    tc::tma_load_2d(dst + (uint32_t)(3 * CP * 128), &tmB, c * kChunk, 3 * CP,
                                    b_full(bq));
                    ++bc;
                    if (++bq == kBSlots) {
                        bq = 0;
                        bpar ^= 1u;
                    }
                }
                for (int s = 0; s < kOzSlices; ++s) {
                    if (ac >= kASlots &&
                        !tc::mbar_wait(a_empty(aq), apar ^ 1u, err, 11, false)) {
                        abort_flag = 1;
                        break;
                    }
                    tc::mbar_expect_tx(a_full(aq), kABytes);
                    tc::tma_load_3d_hint(a_base + (uint32_t)aq * kABytes, &tmA, c * kChunk,
                                         tile * kBM, s, a_full(aq), pol);
                    ++ac;
                    if (++aq == kASlots) {
                        aq = 0;
                        apar ^= 1u;
                    }
                }
            }
        }
        if (!waited) pdl_wait();
        a_issued = ac;
        b_issued = bc;
    } else if (warp == kMmaWarp && lane == 0) {
        // ---- tcgen05.mma issuer ----
        // instruction descriptor without its N field (bits 17-22)
        const uint32_t ibase = prm.idesc & ~(0x3Fu << 17);
        int ac = 0, bc = 0;
        int aq = 0, bq = 0;
        uint32_t apar = 0, bpar = 0;
        int k = 0;
        const int nb = prm.acc_bufs;
        for (long long it = it0; it < it1 && !abort_flag; ++it, ++k) {
            // accumulator set k % nb: wait until the epilogue has drained its
            // previous use (item k - nb)
            const int ab = k % nb;
            const int use = k / nb;
            if (use > 0 &&
                !tc::mbar_wait(acc_empty(ab), (uint32_t)((use - 1) & 1), err, 13, false)) {
                abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t acc_tmem = tmem + (uint32_t)(ab * kOzSlices * CP);
            const int per = (int)(it % prm.periods);
            const int c0 = per * kChunksPerPeriod;
            const int c1 = min(prm.nchunks, c0 + kChunksPerPeriod);
            bool first = true;
            for (int c = c0; c < c1 && !abort_flag; ++c) {
                const int qb = bq;
                if (!tc::mbar_wait(b_full(qb), bpar, err, 14, false)) {
                    abort_flag = 1;
                    break;
                }
                const uint32_t bsm = b_base + (uint32_t)qb * prm.b_bytes;
                for (int s = 0; s < kOzSlices; ++s) {
                    const int qa = aq;
                    if (!tc::mbar_wait(a_full(qa), apar, err, 15, false)) {
                        abort_flag = 1;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint64_t ad = tc::sw128_desc(a_base + (uint32_t)qa * kABytes);
                    // one MMA for every pair (s, t <= 5 - s): the B slices t
                    // lie in consecutive rows, so an MMA of N = (6 - s) cp
                    // rows written at column s cp puts pair (s, t) into the
                    // accumulator of level s + t (two MMAs when N exceeds
                    // 256).  The first K step of an item (s = 0, which covers
                    // every level) initialises the accumulators.
                    const int nt = kOzSlices - s;
                    const int t1 = nt * CP > 256 ? nt / 2 : nt;
                    const uint64_t bd0 = tc::sw128_desc(bsm);
                    const uint64_t bd1 = tc::sw128_desc(bsm + (uint32_t)(t1 * CP) * 128u);
                    const uint32_t id0 = ibase | ((uint32_t)(t1 * CP) >> 3 << 17);
                    const uint32_t id1 = ibase | ((uint32_t)((nt - t1) * CP) >> 3 << 17);
                    const uint32_t acc_first = (first && s == 0) ? 0u : 1u;
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        const uint32_t accum = kk > 0 ? 1u : acc_first;
                        tc::umma<kLowpF16>(acc_tmem + (uint32_t)(s * CP), ad + (uint64_t)(2 * kk),
                                           bd0 + (uint64_t)(2 * kk), id0, accum);
                        if (t1 < nt) {
                            tc::umma<kLowpF16>(acc_tmem + (uint32_t)((s + t1) * CP),
                                               ad + (uint64_t)(2 * kk), bd1 + (uint64_t)(2 * kk),
                                               id1, accum);
                        }
                    }
                    tc::umma_commit(a_empty(qa));
                    ++ac;
                    if (++aq == kASlots) {
                        aq = 0;
                        apar ^= 1u;
                    }
                }
                tc::umma_commit(b_empty(qb));
                ++bc;
                if (++bq == kBSlots) {
                    bq = 0;
                    bpar ^= 1u;
                }
                first = false;
            }
            if (abort_flag) break;
            tc::umma_commit(acc_full(ab));
        }
        tc::umma_commit(mma_done);
    } else if (warp < 4) {
        // ---- epilogue: drain the six level accumulators every period ----
        float Hs[CP], Ls[CP];
#pragma unroll
        for (int j = 0; j < CP; ++j) {
            Hs[j] = 0.0f;
            Ls[j] = 0.0f;
        }
        const int row_local = warp * 32 + lane;
        const int nb = prm.acc_bufs;
        int k = 0;
        for (long long it = it0; it < it1; ++it, ++k) {
            const int ab = k % nb;
            const uint32_t lane_addr =
                tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(ab * kOzSlices * CP);
            const bool ok =
                tc::mbar_wait(acc_full(ab), (uint32_t)((k / nb) & 1), err, 16, true);
            // warp-uniform decision: the TMEM loads below are warp-collective
            if (__any_sync(0xffffffffu, !ok || abort_flag)) {
                abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int g = 0; g < CP / 16; ++g) {
                float v0[16], v1[16], v2[16];
                tc::tmem_ld_16cols_x3(lane_addr + (uint32_t)(16 * g), CP, v0, v1, v2);
                float hh[16], ll[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    float h, e1, e2;
                    two_sum(v0[j], v1[j] * 0x1p-8f, h, e1);
                    two_sum(h, v2[j] * 0x1p-16f, hh[j], e2);
                    ll[j] = e1 + e2;
                }
                tc::tmem_ld_16cols_x3(lane_addr + (uint32_t)(3 * CP + 16 * g), CP, v0, v1, v2);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const float l = ll[j] + (v0[j] * 0x1p-24f + (v1[j] * 0x1p-32f +
                                                                 v2[j] * 0x1p-40f));
                    float s, e;
                    two_sum(Hs[16 * g + j], hh[j], s, e);
                    Hs[16 * g + j] = s;
                    Ls[16 * g + j] += l + e;
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(acc_empty(ab));
            const long long tile = it / prm.periods;
            const bool last = (it + 1 == it1) || ((it + 1) / prm.periods != tile);
            if (last) {
                const long long slot = (long long)blockIdx.x -
                                       owner_of(tile * prm.periods, prm.items, G);
                double *dst = P + ((size_t)(tile * prm.maxslots + slot) * prm.C) * kBM + row_local;
#pragma unroll
                for (int j = 0; j < CP; ++j) {
                    if (j < prm.C) dst[(size_t)j * kBM] = (double)Hs[j] + (double)Ls[j];
                    Hs[j] = 0.0f;
                    Ls[j] = 0.0f;
                }
            }
        }
    }
    __syncwarp();
    pdl_trigger();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == kProducerWarp && lane == 0) {
        // every MMA this CTA issued has completed before TMEM is released
        tc::mbar_wait(mma_done, 0u, err, 17, true);
        if (abort_flag) {
            // drain the copies still in flight (bounded)
            const int ai = a_issued, bi = b_issued;
            for (int i = max(0, ai - prm.a_slots); i < ai; ++i) {
                tc::mbar_wait(a_full(i % prm.a_slots), (uint32_t)((i / prm.a_slots) & 1), err, 18,
                              true);
            }
            for (int i = max(0, bi - prm.b_slots); i < bi; ++i) {
                tc::mbar_wait(b_full(i % prm.b_slots), (uint32_t)((i / prm.b_slots) & 1), err,
                              19, true);
            }
        }
    }
    __syncthreads();
    if (warp == kProducerWarp) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512)
                     : "memory");
    }
}

// Column maxima of |X| as bit patterns (colmax zeroed by the caller): grid
// (column, row chunk), atomicMax per CTA.
__global__ void oz_colmax_kernel(const double *__restrict__ X, long long ldx, int n,
                                 unsigned long long *__restrict__ colmax)
{
    pdl_wait();
    const int c = blockIdx.x;
    const double *xc = X + (size_t)c * ldx;
    unsigned long long m = 0;
    for (int j = blockIdx.y * blockDim.x + threadIdx.x; j < n; j += gridDim.y * blockDim.x) {
        const unsigned long long a =
            (unsigned long long)__double_as_longlong(xc[j]) & 0x7FFFFFFFFFFFFFFFULL;
        m = a > m ? a : m;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, m, off);
        m = o > m ? o : m;
    }
    if ((threadIdx.x & 31) == 0 && m != 0) atomicMax(colmax + c, m);
    pdl_trigger();
}

// B slices of X (columns c < C; zero rows for C <= c < cp): row t * cp + c
// of B holds digit t of column c along K, zero beyond n.  Grid (column, K
// chunk); colexp[c] records the column's exponent.
__global__ void oz_slice_x_kernel(const double *__restrict__ X, long long ldx, int n, int C,
                                  int cp, int ldp, const unsigned long long *__restrict__ colmax,
                                  __half *__restrict__ B, int *__restrict__ colexp)
{
    pdl_wait();
    const int c = blockIdx.x;
    const int e = c < C ? oz_exponent(colmax[c]) : 0;
    if (blockIdx.y == 0 && threadIdx.x == 0 && c < C) colexp[c] = e;
    const double *xc = X + (size_t)c * ldx;
    __half2 *row = reinterpret_cast<__half2 *>(B + (size_t)c * ldp);
    const size_t stride = (size_t)cp * (size_t)ldp / 2;
    for (int j = 2 * (blockIdx.y * blockDim.x + threadIdx.x); j < ldp;
         j += 2 * gridDim.y * blockDim.x) {
        const double v0 = (c < C && j < n) ? xc[j] : 0.0;
        const double v1 = (c < C && j + 1 < n) ? xc[j + 1] : 0.0;
        oz_store_pair(v0, v1, e, row + j / 2, stride);
    }
    pdl_trigger();
}

// Y[:, c] = 2^(e_i + f_c - 16) (sum of the tile's partials) + d_i X[:, c].
__global__ void oz_finish_kernel(const double *__restrict__ P, const int *__restrict__ rowexp,
                                 const int *__restrict__ colexp, const double *__restrict__ d,
                                 const double *__restrict__ X, long long ldx, int n, int C,
                                 int periods, long long items, long long G, int maxslots,
                                 double *__restrict__ Y, long long ldy)
{
    pdl_wait();
    pdl_trigger();
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n * (size_t)C) return;
    const int i = (int)(e % (size_t)n);
    const int c = (int)(e / (size_t)n);
    const long long tile = i / kBM;
    const int r = i - (int)tile * kBM;
    const long long first = owner_of(tile * periods, items, G);
    const long long last = owner_of(tile * periods + periods - 1, items, G);
    double s = 0.0;
    for (long long q = 0; q <= last - first; ++q) {
        s += P[((size_t)(tile * maxslots + q) * C + c) * kBM + r];
    }
    const int ei = rowexp[i], fc = colexp[c];
    double y = (ei == kOzNonFinite || fc == kOzNonFinite) ? NAN : ldexp(s, ei + fc - 16);
    if (d != nullptr) y = fma(d[i], X[(size_t)i + (size_t)c * ldx], y);
    Y[(size_t)i + (size_t)c * ldy] = y;
}

// Row maxima of |H_il| (l != i) of a column-major H, as bit patterns.
__global__ void oz_rowmax_kernel(const double *__restrict__ H, int n,
                                 unsigned long long *__restrict__ rowmax)
{
    const int i = blockIdx.y * 32 + threadIdx.x;
    const int l0 = blockIdx.x * 32;
    if (i >= n) return;
    unsigned long long m = 0;
    for (int l = l0 + threadIdx.y; l < min(n, l0 + 32); l += blockDim.y) {
        if (l == i) continue;
        const unsigned long long a =
            (unsigned long long)__double_as_longlong(H[(size_t)i + (size_t)l * n]) &
            0x7FFFFFFFFFFFFFFFULL;
        m = a > m ? a : m;
    }
    if (m != 0) atomicMax(rowmax + i, m);
}

// A slices of a column-major H: tile of 32 rows x 64 columns, read along
// rows (coalesced), digits staged in shared memory, written along K.
__global__ void oz_slice_h_kernel(const double *__restrict__ H, int n, int ldp,
                                  const unsigned long long *__restrict__ rowmax,
                                  __half *__restrict__ A, int *__restrict__ rowexp)
{
    __shared__ short dg[kOzSlices][32][66];
    const int i0 = blockIdx.y * 32;
    const int l0 = blockIdx.x * 64;
    const int tx = threadIdx.x;  // 0..31
    const int i = i0 + tx;
    const int e = i < n ? oz_exponent(rowmax[i]) : 0;
    if (blockIdx.x == 0 && threadIdx.y == 0 && i < n) rowexp[i] = e;
    for (int ly = threadIdx.y; ly < 64; ly += blockDim.y) {
        const int l = l0 + ly;
        const double v = (i < n && l < n && l != i) ? H[(size_t)i + (size_t)l * n] : 0.0;
        int dd[kOzSlices];
        oz_digits_fast(v, e, dd);
#pragma unroll
        for (int s = 0; s < kOzSlices; ++s) dg[s][tx][ly] = (short)dd[s];
    }
    __syncthreads();
    // write: thread (tx, ty) covers column pair 2*tx of rows ty, ty + 8, ...
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int row = i0 + r;
        if (row >= n) continue;
        const int l = l0 + 2 * tx;
        if (l >= ldp) continue;
#pragma unroll
        for (int s = 0; s < kOzSlices; ++s) {
            reinterpret_cast<__half2 *>(A + ((size_t)s * n + row) * ldp + l)[0] =
                oz_digit_pair(dg[s][r][2 * tx], dg[s][r][2 * tx + 1]);
        }
    }
}

}  // namespace oz

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
int OzDelta::init_storage(int n_, cudaStream_t s)
{
    n = n_;
    ldp = (n + 63) / 64 * 64;
    IPTGB_CHECK(A.alloc((size_t)kOzSlices * n * ldp, s));
    IPTGB_CHECK(rowexp.alloc((size_t)n, s));
    return make_map_3d(&mapA, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, A.ptr, ldp, n, kOzSlices,
                       oz::kBM);
}

int OzDelta::split_from(const double *H, int n_, cudaStream_t s)
{
    IPTGB_CHECK(init_storage(n_, s));
    DeviceBuffer<unsigned long long> rm;
    IPTGB_CHECK(rm.alloc((size_t)n, s));
    IPTGB_CUDA(cudaMemsetAsync(rm.ptr, 0, (size_t)n * sizeof(unsigned long long), s));
    const dim3 g1((n + 31) / 32, (n + 31) / 32);
    oz::oz_rowmax_kernel<<<g1, dim3(32, 8), 0, s>>>(H, n, rm.ptr);
    IPTGB_LAUNCH();
    const dim3 g2(ldp / 64, (n + 31) / 32);
    oz::oz_slice_h_kernel<<<g2, dim3(32, 8), 0, s>>>(H, n, ldp, rm.ptr, A.ptr, rowexp.ptr);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

namespace {

template <int CP>
int launch_product(const CUtensorMap &mapA, const CUtensorMap &mapB, const oz::Params &prm,
                   int grid, size_t smem, double *P, int *err, cudaStream_t s)
{
    auto kfn = oz::oz_product_kernel<CP>;
    IPTGB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return launch_pdl(kfn, dim3(grid), dim3(oz::kThreads), smem, s, mapA, mapB, prm, P, err);
}

}  // namespace

int OzProduct::bind(const OzDelta *delta, const double *diag, cudaStream_t stream)
{
    dl = delta;
    d = diag;
    s = stream;
    sms = device_sm_count();
    if (err.ptr == nullptr) {
        IPTGB_CHECK(err.alloc(1, s));
        IPTGB_CUDA(cudaMemsetAsync(err.ptr, 0, sizeof(int), s));
    }
    return IPT_CUDA_SUCCESS;
}

int OzProduct::apply_group(const double *X, long long ldx, int C, double *Y, long long ldy)
{
    const int n = dl->n;
    const int ldp = dl->ldp;
    const int cp = (C + 15) / 16 * 16;
    if (C <= 0 || cp > kOzMaxCols) return IPT_CUDA_INVALID_ARGUMENT;
    if (cp != cp_cur) {
        IPTGB_CHECK(B.alloc((size_t)kOzSlices * cp * ldp, s));
        IPTGB_CHECK(colexp.alloc((size_t)cp, s));
        IPTGB_CHECK(colmax.alloc((size_t)cp, s));
        IPTGB_CHECK(make_map(&mapB, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, B.ptr, ldp, kOzSlices * cp,
                             3 * cp));
        cp_cur = cp;
    }
    oz::Params prm = {};
    prm.n = n;
    prm.C = C;
    prm.cp = cp;
    prm.nchunks = ldp / oz::kChunk;
    prm.periods = (prm.nchunks + oz::kChunksPerPeriod - 1) / oz::kChunksPerPeriod;
    const int tiles = (n + oz::kBM - 1) / oz::kBM;
    prm.items = (long long)tiles * prm.periods;
    const int grid = (int)std::min<long long>(sms, prm.items);
    int maxslots = 1;
    for (int t = 0; t < tiles; ++t) {
        const long long f = tc::owner_of((long long)t * prm.periods, prm.items, grid);
        const long long l = tc::owner_of((long long)t * prm.periods + prm.periods - 1, prm.items,
                                         grid);
        maxslots = std::max(maxslots, (int)(l - f + 1));
    }
    prm.maxslots = maxslots;
    prm.b_bytes = (uint32_t)(kOzSlices * cp * 128);
    prm.b_slots = oz::kMaxBSlots;
    // as many A slices in flight as the shared memory holds (>= one chunk)
    const size_t budget = 225u * 1024u - (size_t)prm.b_slots * prm.b_bytes;
    prm.a_slots = (int)std::min<size_t>(oz::kMaxASlots, budget / oz::kABytes);
    if (prm.a_slots < kOzSlices) return IPT_CUDA_INVALID_ARGUMENT;
    prm.acc_bufs = 2 * kOzSlices * cp <= 512 ? 2 : 1;
    prm.idesc = (1u << 4) | ((uint32_t)(cp >> 3) << 17) | ((uint32_t)(oz::kBM >> 4) << 24);
    const size_t pneed = (size_t)tiles * maxslots * C * oz::kBM;
    if (P.count < pneed) IPTGB_CHECK(P.alloc(pneed, s));
    const size_t smem = 1024 + (size_t)prm.a_slots * oz::kABytes +
                        (size_t)prm.b_slots * prm.b_bytes +
                        (2 * oz::kMaxASlots + 2 * oz::kMaxBSlots + 5) * 8 + 16;

    // X split: column maxima, then the digit slices (grids of about 4 CTAs per SM)
    IPTGB_CUDA(cudaMemsetAsync(colmax.ptr, 0, (size_t)cp * sizeof(unsigned long long), s));
    const int ychunks = std::max(1, std::min((n + 2047) / 2048, (4 * sms + cp - 1) / cp));
    IPTGB_CHECK(launch_pdl(oz::oz_colmax_kernel, dim3(C, ychunks), dim3(256), 0, s, X, ldx, n,
                           colmax.ptr));
    IPTGB_CHECK(launch_pdl(oz::oz_slice_x_kernel, dim3(cp, ychunks), dim3(256), 0, s, X, ldx, n,
                           C, cp, ldp, (const unsigned long long *)colmax.ptr, B.ptr,
                           colexp.ptr));
    int st;
    switch (cp) {
    case 16: st = launch_product<16>(dl->mapA, mapB, prm, grid, smem, P.ptr, err.ptr, s); break;
    case 32: st = launch_product<32>(dl->mapA, mapB, prm, grid, smem, P.ptr, err.ptr, s); break;
    case 48: st = launch_product<48>(dl->mapA, mapB, prm, grid, smem, P.ptr, err.ptr, s); break;
    default: st = launch_product<64>(dl->mapA, mapB, prm, grid, smem, P.ptr, err.ptr, s); break;
    }
    IPTGB_CHECK(st);
    return launch_pdl(oz::oz_finish_kernel, dim3(blocks_for((size_t)n * C)), dim3(kThreads), 0, s,
                      (const double *)P.ptr, (const int *)dl->rowexp.ptr,
                      (const int *)colexp.ptr, d, X, ldx, n, C, prm.periods, prm.items,
                      (long long)grid, maxslots, Y, ldy);
}

int OzProduct::apply(const double *X, long long ldx, int C, double *Y, long long ldy)
{
    for (int c0 = 0; c0 < C; c0 += kOzMaxCols) {
        const int cc = std::min(kOzMaxCols, C - c0);
        IPTGB_CHECK(apply_group(X + (size_t)c0 * ldx, ldx, cc, Y + (size_t)c0 * ldy, ldy));
    }
    return IPT_CUDA_SUCCESS;
}

int OzProduct::read_error(int *host_err)
{
    IPTGB_CUDA(cudaMemcpyAsync(host_err, err.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    return IPT_CUDA_SUCCESS;
}

}  // namespace iptgb

// ---------------------------------------------------------------------------
// Exported entry points (include/ipt_block.h)
// ---------------------------------------------------------------------------
#define IPT_API extern "C" __attribute__((visibility("default")))

IPT_API int ipt_block_accurate_product(const double *d_H, int n, const double *d_X, int c,
                                       double *d_Y, void *stream)
{
    using namespace iptgb;
    if (d_H == nullptr || d_X == nullptr || d_Y == nullptr || n <= 0 || c <= 0 ||
        (size_t)n * (size_t)c > (size_t)INT_MAX) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    OzDelta delta;
    IPTGB_CHECK(delta.split_from(d_H, n, s));
    DeviceBuffer<double> d;
    IPTGB_CHECK(d.alloc((size_t)n, s));
    IPTGB_CHECK(launch_extract_diagonal(d_H, n, n, d.ptr, s));
    OzProduct prod;
    IPTGB_CHECK(prod.bind(&delta, d.ptr, s));
    IPTGB_CHECK(prod.apply(d_X, n, c, d_Y, n));
    int herr = 0;
    IPTGB_CHECK(prod.read_error(&herr));
    if (herr != 0) {
        fprintf(stderr, "ipt_gb300: accurate product: bounded wait gave up (code %d)\n", herr);
        return IPT_CUDA_CUDA_ERROR;
    }
    IPTGB_CUDA(cudaGetLastError());
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_block_accurate_split_host(const double *values, long long count, double max_abs,
                                          int *exponent_out, int *digits_out)
{
    using namespace iptgb;
    if (count < 0 || exponent_out == nullptr || (count > 0 && (values == nullptr ||
                                                               digits_out == nullptr))) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    uint64_t mb;
    memcpy(&mb, &max_abs, sizeof(mb));
    const int e = oz_exponent(mb & 0x7FFFFFFFFFFFFFFFULL);
    *exponent_out = e;
    for (long long i = 0; i < count; ++i) {
        int dg[kOzSlices];
        oz_digits_of(oz_fixed(values[i], e), dg);
        for (int s = 0; s < kOzSlices; ++s) digits_out[i * kOzSlices + s] = dg[s];
    }
    return IPT_CUDA_SUCCESS;
}
