// k_tc.cu - low-precision dense IPT stage on the GB300 tensor cores.
//
// Block product Y = Delta X for the IPT map (reference: cublasGemmEx FP16 /
// TF32 on the off-diagonal copy, IPT_C_GPU/src/mixed_precision/
// ipt_mixed_precision_cuda.cu:189-216,520-523,713-716), written for sm_103a:
//
//  * Delta (diagonal zeroed, power-of-two scaled for FP16) is stored once per
//    solve row-major ("K-major") in FP16, BF16 or TF32-rounded FP32, with a
//    leading dimension padded to 64 elements;
//  * each CTA owns 128 rows and a K-range (split-K so that the grid covers
//    the 152 SMs); warp 0 streams 128-byte-wide K chunks of Delta and X
//    through a multi-stage TMA pipeline (cp.async.bulk.tensor, SWIZZLE_128B,
//    mbarrier complete_tx), warp 1 issues tcgen05.mma (M = 128, N = padded
//    block width, FP32 accumulators in TMEM), and all four warps drain TMEM
//    with tcgen05.ld into per-split FP32 partial blocks;
//  * a second kernel sums the split partials in a fixed order, applies the
//    IPT update X' = (Y - X c) * G (c_j = Y_jj, G_ij = 1/(d_j - d_i)) in FP32,
//    writes the FP32 master block and the low-precision operand copy for the
//    next product, and reduces ||X' - X||_F and ||X||_F.
//
// Every mbarrier wait is bounded; a timeout sets an error flag, the CTA
// drains its own outstanding copies (bounded), frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <utility>
#include <vector>

#include "block_solver.h"
#include "common.cuh"
#include "dfloat.cuh"
#include "fpconv.cuh"
#include "lowp.h"
#include "oz.cuh"
#include "reduce.cuh"
#include "tcgen05.cuh"

namespace iptgb {

namespace tc {

constexpr int kBM = 128;         // UMMA M: rows of Delta per CTA
constexpr int kRowBytes = 128;   // one SWIZZLE_128B row per K chunk
constexpr int kThreads = 128;

// ---------------------------------------------------------------------------
// Split-K partial product P[split] = Delta[rows, Ksplit] X[Ksplit, :].
// Grid (row blocks, splits); 128 threads; dynamic smem = stages * stage bytes
// + 1 KB alignment slack + barriers.  P layout: [split][col][row], ld = n.
// ---------------------------------------------------------------------------
template <int KIND>
__global__ void __launch_bounds__(kThreads, 1)
tc_partial_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  int n, int p, int p_pad, int stages, int tmem_cols, int chunks_total,
                  int chunks_per_split, int kchunk_elems, uint32_t idesc, float *__restrict__ P,
                  int *err, float a_keep, const double *hist, int step, double stop_tol,
                  long long spin)
{
    // the iteration already met its tolerance on the device: nothing to do
    // (the history is written by the previous update: wait for it first)
    if (hist != nullptr) {
        pdl_wait();
        if (hist_stopped(hist, step, stop_tol)) return;
    }
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte alignment of the shared-window address (SWIZZLE_128B atoms)
    uint8_t *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const uint32_t a_bytes = kBM * kRowBytes;
    const uint32_t b_bytes = (uint32_t)p_pad * kRowBytes;
    const uint32_t stage_bytes = a_bytes + b_bytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (size_t)stages * stage_bytes);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * stages + 1);
    __shared__ int abort_flag;
    __shared__ int issued_count;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int rb = blockIdx.x;
    const int split = blockIdx.y;
    const int c0 = split * chunks_per_split;
    const int c1 = min(chunks_total, c0 + chunks_per_split);
    const int nchunks = c1 - c0;
    const uint32_t smem_base = smem_u32(smem);
    const uint32_t bar_base = smem_u32(bars);
    auto full_bar = [&](int s) { return bar_base + 8u * (uint32_t)s; };
    auto empty_bar = [&](int s) { return bar_base + 8u * (uint32_t)(stages + s); };
    const uint32_t accum_bar = bar_base + 8u * (uint32_t)(2 * stages);

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(full_bar(s), 1);
            mbar_init(empty_bar(s), 1);
        }
        mbar_init(accum_bar, 1);
        abort_flag = 0;
        issued_count = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        const uint64_t a_pol = a_keep > 0.0f ? l2_keep_policy(fminf(a_keep, 1.0f)) : 0ull;
        // ---- TMA producer ----
        // Delta does not depend on the previous kernel: the first stages' Delta
        // tiles are requested before waiting for the grid that wrote X (with a
        // programmatic dependent launch that grid may still be running)
        const int pre = min(stages, nchunks);
        for (int q = 0; q < pre; ++q) {
            const uint32_t sa = smem_base + (uint32_t)q * stage_bytes;
            const int kx = (c0 + q) * kchunk_elems;
            mbar_expect_tx(full_bar(q), stage_bytes);
            if (a_keep > 0.0f) {
                tma_load_2d_hint(sa, &tmA, kx, rb * kBM, full_bar(q), a_pol);
            } else {
                tma_load_2d(sa, &tmA, kx, rb * kBM, full_bar(q));
            }
        }
        pdl_wait();
        for (int q = 0; q < pre; ++q) {
            const uint32_t sb = smem_base + (uint32_t)q * stage_bytes + a_bytes;
            tma_load_2d(sb, &tmB, (c0 + q) * kchunk_elems, 0, full_bar(q));
        }
        int i = pre;
        for (; i < nchunks; ++i) {
            const int s = i % stages;
            const int r = i / stages;
            if (r > 0 && !mbar_wait(empty_bar(s), (uint32_t)((r - 1) & 1), err, 1, false, spin)) {
                abort_flag = 1;
                break;
            }
            if (abort_flag) {
                break;
            }
            const uint32_t sa = smem_base + (uint32_t)s * stage_bytes;
            const uint32_t sb = sa + a_bytes;
            const int kx = (c0 + i) * kchunk_elems;
            mbar_expect_tx(full_bar(s), stage_bytes);
            if (a_keep > 0.0f) {
                tma_load_2d_hint(sa, &tmA, kx, rb * kBM, full_bar(s), a_pol);
            } else {
                tma_load_2d(sa, &tmA, kx, rb * kBM, full_bar(s));
            }
            tma_load_2d(sb, &tmB, kx, 0, full_bar(s));
        }
        issued_count = i;
        pdl_trigger();
    } else if (warp == 1 && lane == 0) {
        // ---- tcgen05.mma issuer ----
        for (int i = 0; i < nchunks; ++i) {
            const int s = i % stages;
            const int r = i / stages;
            if (!mbar_wait(full_bar(s), (uint32_t)(r & 1), err, 2, false, spin)) {
                abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_base + (uint32_t)s * stage_bytes;
            const uint32_t sb = sa + a_bytes;
            const uint64_t ad = sw128_desc(sa);
            const uint64_t bd = sw128_desc(sb);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                // advance 32 bytes along K inside the swizzle atom
                umma<KIND>(tmem, ad + (uint64_t)(2 * kk), bd + (uint64_t)(2 * kk), idesc,
                           (i > 0 || kk > 0) ? 1u : 0u);
            }
            umma_commit(empty_bar(s));
        }
        umma_commit(accum_bar);
    }
    __syncwarp();

    // ---- epilogue: TMEM -> registers -> partial block ----
    const bool ok0 = mbar_wait(accum_bar, 0u, err, 3, true, spin);
    // warp-uniform: the TMEM loads below are warp-collective
    const bool ok = __all_sync(0xffffffffu, ok0 && !abort_flag);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        const int row = rb * kBM + warp * 32 + lane;
        for (int cb = 0; cb < p_pad; cb += 32) {
            float v[32];
            tmem_ld_32cols(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, v);
            if (row < n) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    if (cb + j < p) {
                        P[((size_t)split * p + (size_t)(cb + j)) * (size_t)n + row] = v[j];
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (abort_flag && threadIdx.x == 0) {
        // before TMEM and shared memory are released: the MMAs this CTA
        // issued (the issuer always commits the accumulator barrier last) and
        // the copies it may still have in flight, each with the full bound
        mbar_wait(accum_bar, 0u, err, 5, true);
        const int issued = issued_count;
        for (int i = max(0, issued - stages); i < issued; ++i) {
            mbar_wait(full_bar(i % stages), (uint32_t)((i / stages) & 1), err, 4, true);
        }
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(tmem_cols)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
// Persistent (stream-K) form of the same product: G CTAs (one per SM) walk
// contiguous ranges of the (128-row tile, K chunk) items, so every SM
// streams the same number of Delta bytes whatever the tile count, through
// a deeper TMA ring than the split-K grid can hold.  A CTA's range crosses
// tile boundaries: each piece of a tile it covers (a segment) accumulates
// in one of two TMEM accumulators, so the MMAs of the next segment run
// while the epilogue warps drain the last one into partial slot
// (CTA - first CTA of the tile) of that tile.  The slots a tile never uses
// are never written (the caller zeroes them once), so the update sums a
// fixed number of slots in a fixed order, as for split-K.
// Warps 0-3 epilogue, warp 4 TMA producer, warp 5 MMA issuer.
// ---------------------------------------------------------------------------
constexpr int kStreamThreads = 192;
constexpr int kStreamProducer = 4;
constexpr int kStreamMma = 5;

struct StreamParams {
    int n, p, p_pad, stages;
    int acc_cols;    // TMEM columns of one accumulator
    int acc_bufs;    // accumulators (2: drain one while the other fills)
    int tmem_cols;   // allocation (power of two >= acc_bufs * acc_cols)
    int chunks;      // K chunks per tile
    int kchunk;      // elements per K chunk (128 bytes)
    long long items; // tiles * chunks
    uint32_t idesc;
};

template <int KIND>
__global__ void __launch_bounds__(kStreamThreads, 1)
tc_stream_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                 const __grid_constant__ StreamParams prm, float *__restrict__ P, int *err,
                 float a_keep, const double *hist, int step, double stop_tol, long long spin,
                 int reverse)
{
    if (hist != nullptr) {
        pdl_wait();
        if (hist_stopped(hist, step, stop_tol)) return;
    }
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int stages = prm.stages;
    const uint32_t a_bytes = kBM * kRowBytes;
    const uint32_t stage_bytes = a_bytes + (uint32_t)prm.p_pad * kRowBytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (size_t)stages * stage_bytes);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * stages + 5);
    __shared__ volatile int abort_flag;
    __shared__ int issued_count;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const long long G = gridDim.x;
    const long long it0 = (long long)blockIdx.x * prm.items / G;
    const long long it1 = ((long long)blockIdx.x + 1) * prm.items / G;
    const uint32_t smem_base = smem_u32(smem);
    const uint32_t bar0 = smem_u32(bars);
    auto full_bar = [&](int q) { return bar0 + 8u * (uint32_t)q; };
    auto empty_bar = [&](int q) { return bar0 + 8u * (uint32_t)(stages + q); };
    auto acc_full = [&](int b) { return bar0 + 8u * (uint32_t)(2 * stages + b); };
    auto acc_empty = [&](int b) { return bar0 + 8u * (uint32_t)(2 * stages + 2 + b); };
    const uint32_t mma_done = bar0 + 8u * (uint32_t)(2 * stages + 4);

    if (threadIdx.x == 0) {
        for (int q = 0; q < stages; ++q) {
            mbar_init(full_bar(q), 1);
            mbar_init(empty_bar(q), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(acc_full(b), 1);
            mbar_init(acc_empty(b), 4);  // one arrival per epilogue warp
        }
        mbar_init(mma_done, 1);
        abort_flag = 0;
        issued_count = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == kStreamProducer) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(prm.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const int count = (int)(it1 - it0);
    // traversal direction: every other product walks its items backwards, so
    // it starts on the bytes of Delta the previous product read last (still
    // in L2)
    const long long first_it = reverse ? it1 - 1 : it0;
    // items of the segment (one tile's part of this CTA's range) that starts
    // at item `it` in traversal order
    auto seg_len_at = [&](long long it) {
        const long long tile = it / prm.chunks;
        return reverse ? (int)(it - max(it0, tile * prm.chunks) + 1)
                       : (int)(min(it1, (tile + 1) * prm.chunks) - it);
    };

    if (warp == kStreamProducer && lane == 0) {
        // the loop bodies keep their indices incremental: this one thread
        // issues every copy of the SM, so a division per chunk would slow it
        const uint64_t a_pol = a_keep > 0.0f ? l2_keep_policy(fminf(a_keep, 1.0f)) : 0ull;
        const int tile0 = (int)(first_it / prm.chunks);
        const int c00 = (int)(first_it - (long long)tile0 * prm.chunks);
        auto advance = [&](int &tile, int &c) {
            if (reverse) {
                if (c == 0) {
                    c = prm.chunks - 1;
                    --tile;
                } else {
                    --c;
                }
            } else if (++c == prm.chunks) {
                c = 0;
                ++tile;
            }
        };
        auto load_a = [&](int q, int tile, int c) {
            const uint32_t sa = smem_base + (uint32_t)q * stage_bytes;
            if (a_keep > 0.0f) {
                tma_load_2d_hint(sa, &tmA, c * prm.kchunk, tile * kBM, full_bar(q), a_pol);
            } else {
                tma_load_2d(sa, &tmA, c * prm.kchunk, tile * kBM, full_bar(q));
            }
        };
        auto load_b = [&](int q, int c) {
            tma_load_2d(smem_base + (uint32_t)q * stage_bytes + a_bytes, &tmB, c * prm.kchunk, 0,
                        full_bar(q));
        };
        // Delta does not depend on the preceding kernel: the first stages'
        // Delta tiles are requested before waiting for the grid that wrote X
        const int pre = min(stages, count);
        int tile = tile0, c = c00;
        for (int q = 0; q < pre; ++q) {
            mbar_expect_tx(full_bar(q), stage_bytes);
            load_a(q, tile, c);
            advance(tile, c);
        }
        pdl_wait();
        {
            int tb = tile0, cb = c00;
            for (int q = 0; q < pre; ++q) {
                load_b(q, cb);
                advance(tb, cb);
            }
        }
        int i = pre, q = 0;
        uint32_t parity = 0;  // of the empty barriers' first reuse
        for (; i < count; ++i) {
            if (!mbar_wait(empty_bar(q), parity, err, 21, false, spin)) {
                abort_flag = 1;
                break;
            }
            if (abort_flag) break;
            mbar_expect_tx(full_bar(q), stage_bytes);
            load_a(q, tile, c);
            load_b(q, c);
            advance(tile, c);
            if (++q == stages) {
                q = 0;
                parity ^= 1u;
            }
        }
        issued_count = i;
        pdl_trigger();
    } else if (warp == kStreamMma && lane == 0) {
        int q = 0, seg = 0;
        uint32_t parity = 0;
        long long it = first_it;
        for (int done = 0; done < count && !abort_flag; ++seg) {
            const int seg_len = seg_len_at(it);
            const int ab = seg & (prm.acc_bufs - 1);
            const int use = prm.acc_bufs == 2 ? seg >> 1 : seg;
            if (use > 0 &&
                !mbar_wait(acc_empty(ab), (uint32_t)((use - 1) & 1), err, 22, false, spin)) {
                abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t acc = tmem + (uint32_t)(ab * prm.acc_cols);
            for (int x = 0; x < seg_len; ++x) {
                if (!mbar_wait(full_bar(q), parity, err, 23, false, spin)) {
                    abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t sa = smem_base + (uint32_t)q * stage_bytes;
                const uint64_t ad = sw128_desc(sa);
                const uint64_t bd = sw128_desc(sa + a_bytes);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    umma<KIND>(acc, ad + (uint64_t)(2 * kk), bd + (uint64_t)(2 * kk), prm.idesc,
                               (x > 0 || kk > 0) ? 1u : 0u);
                }
                umma_commit(empty_bar(q));
                if (++q == stages) {
                    q = 0;
                    parity ^= 1u;
                }
            }
            if (abort_flag) break;
            it += reverse ? -seg_len : seg_len;
            done += seg_len;
            umma_commit(acc_full(ab));
        }
        umma_commit(mma_done);
    } else if (warp < 4) {
        // ---- epilogue: one segment at a time, TMEM -> partial slot ----
        int seg = 0;
        long long it = first_it;
        for (int done = 0; done < count; ++seg) {
            const long long tile = it / prm.chunks;
            const int seg_len = seg_len_at(it);
            it += reverse ? -seg_len : seg_len;
            done += seg_len;
            const int ab = seg % prm.acc_bufs;
            const bool ok0 =
                mbar_wait(acc_full(ab), (uint32_t)((seg / prm.acc_bufs) & 1), err, 24, true, spin);
            // warp-uniform: the TMEM loads below are warp-collective
            if (__any_sync(0xffffffffu, !ok0 || abort_flag)) {
                abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const long long slot = (long long)blockIdx.x - owner_of(tile * prm.chunks, prm.items, G);
            const int row = (int)tile * kBM + warp * 32 + lane;
            float *dst = P + (size_t)slot * prm.p * (size_t)prm.n + row;
            const uint32_t lane_addr =
                tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(ab * prm.acc_cols);
            for (int cb = 0; cb < prm.p_pad; cb += 32) {
                float v[32];
                tmem_ld_32cols(lane_addr + (uint32_t)cb, v);
                if (row < prm.n) {
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        if (cb + j < prm.p) dst[(size_t)(cb + j) * prm.n] = v[j];
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(acc_empty(ab));
        }
    }
    __syncwarp();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == kStreamProducer && lane == 0) {
        // every MMA this CTA issued has completed before TMEM is released
        mbar_wait(mma_done, 0u, err, 25, true);
        if (abort_flag) {
            // the copies still in flight (bounded)
            const int issued = issued_count;
            for (int i = max(0, issued - stages); i < issued; ++i) {
                mbar_wait(full_bar(i % stages), (uint32_t)((i / stages) & 1), err, 26, true);
            }
        }
    }
    __syncthreads();
    if (warp == kStreamProducer) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(prm.tmem_cols)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
// Symmetric form of the product (FP16 / BF16 Delta): Delta = Delta^T, so only
// its upper 128 x 128 tiles (ib <= jb) are read, each once, and used twice:
// as the K-major A operand for Y[ib] += T X[jb] and, through an MN-major
// descriptor of the same shared-memory tile (the TMA's 128-byte swizzled
// rows of 64 columns are MN-major atoms of the transpose: LBO = the 16 KB
// between the two 64-column halves, SBO = 1 KB per 8 rows), for
// Y[jb] += T^T X[ib].  Half of Delta's bytes per product, which at n = 8192
// (67 MB) stays resident in L2 across the products of a solve.
//
// Work: super-tiles (IB, JB), IB <= JB, of 4 x 4 tiles, one CTA each at a
// time; a super-tile keeps 4 row accumulators R[a] (MMA1, rows 4 IB + a) and
// 4 column accumulators C[b] (MMA2, rows 4 JB + b) in TMEM, and the 8 X blocks
// it needs in shared memory, while its tiles stream through a TMA ring.
// Output row block r (super-block R = r / 4) receives its R-partials in
// slots JB - R (JB = R .. nS - 1) and its C-partials in slots nS - R + IB
// (IB = 0 .. R): every one of the nS + 1 slots of every row block is written
// once per product (zeros for an accumulator no tile reaches), so the update
// sums a fixed number of slots in a fixed order.
// Warps 0-3 epilogue, warp 4 TMA producer, warp 5 MMA issuer.
// ---------------------------------------------------------------------------
constexpr int kSymG = 4;             // tiles per super-tile side
constexpr uint32_t kSymTileBytes = 2 * kBM * kRowBytes;  // 128 x 128 FP16 = 32 KB

struct SymParams {
    int n, p, p_pad, nb, nS, stages;
    int items;       // nS (nS + 1) / 2 super-tiles
    uint32_t idesc;  // M = 128, N = p_pad, K-major A
};

__device__ __forceinline__ uint64_t mn_sw128_desc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)(16384u >> 4) << 16;  // LBO: next 64 MN elements (the second half)
    d |= (uint64_t)(1024u >> 4) << 32;   // SBO: next 8 K rows
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// super-tile index -> (IB, JB), IB <= JB, row by row
__device__ __forceinline__ void sym_item(int it, int nS, int &IB, int &JB)
{
    int ib = 0, rem = it;
    while (rem >= nS - ib) {
        rem -= nS - ib;
        ++ib;
    }
    IB = ib;
    JB = ib + rem;
}

template <int KIND>
__global__ void __launch_bounds__(kStreamThreads, 1)
tc_sym_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
              const __grid_constant__ SymParams prm, float *__restrict__ P, int *err, float a_keep,
              const double *hist, int step, double stop_tol, long long spin)
{
    if (hist != nullptr) {
        pdl_wait();
        if (hist_stopped(hist, step, stop_tol)) return;
    }
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int stages = prm.stages;
    const uint32_t bbox = (uint32_t)prm.p_pad * kRowBytes;  // one 64-wide K box of X
    const uint32_t bblk = 2 * bbox;                          // one 128-row block of X
    uint8_t *a_ring = smem;
    uint8_t *b_area = smem + (size_t)stages * kSymTileBytes;  // 8 blocks: rows 0-3, cols 4-7
    uint64_t *bars = reinterpret_cast<uint64_t *>(b_area + (size_t)2 * kSymG * bblk);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * stages + 5);
    __shared__ volatile int abort_flag;
    __shared__ int issued_count;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t a_base = smem_u32(a_ring);
    const uint32_t b_base = smem_u32(b_area);
    const uint32_t bar0 = smem_u32(bars);
    auto full_bar = [&](int q) { return bar0 + 8u * (uint32_t)q; };
    auto empty_bar = [&](int q) { return bar0 + 8u * (uint32_t)(stages + q); };
    const uint32_t b_full = bar0 + 8u * (uint32_t)(2 * stages);
    const uint32_t b_free = b_full + 8u;    // MMAs of a super-tile done: X blocks reusable
    const uint32_t acc_full = b_full + 16u;
    const uint32_t acc_empty = b_full + 24u;
    const uint32_t mma_done = b_full + 32u;

    if (threadIdx.x == 0) {
        for (int q = 0; q < stages; ++q) {
            mbar_init(full_bar(q), 1);
            mbar_init(empty_bar(q), 1);
        }
        mbar_init(b_full, 1);
        mbar_init(b_free, 1);
        mbar_init(acc_full, 1);
        mbar_init(acc_empty, 4);
        mbar_init(mma_done, 1);
        abort_flag = 0;
        issued_count = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == kStreamProducer) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const int nb = prm.nb, nS = prm.nS;
    const int G = gridDim.x;
    // the tiles of super-tile (IB, JB) in order: a-major, then b
    auto tile_ok = [&](int IB, int JB, int a, int b) {
        const int ib = kSymG * IB + a, jb = kSymG * JB + b;
        return ib < nb && jb < nb && ib <= jb;
    };

    if (warp == kStreamProducer && lane == 0) {
        const uint64_t pol = a_keep > 0.0f ? l2_keep_policy(fminf(a_keep, 1.0f)) : 0ull;
        int q = 0;
        uint32_t parity = 0;
        int issued = 0;
        bool waited = false;
        int st = 0;
        for (int it = blockIdx.x; it < prm.items && !abort_flag; it += G, ++st) {
            int IB, JB;
            sym_item(it, nS, IB, JB);
            // Delta tiles first (no dependence on the preceding kernel); the
            // X blocks after the grid that wrote X is done and, from the
            // second super-tile on, after the MMAs of the previous one
            int pre_done = 0;
            auto issue_tile = [&](int a, int b) -> bool {
                if (issued >= stages &&
                    !mbar_wait(empty_bar(q), parity ^ 1u, err, 31, false, spin)) {
                    abort_flag = 1;
                    return false;
                }
                const uint32_t dst = a_base + (uint32_t)q * kSymTileBytes;
                const int row = (kSymG * IB + a) * kBM, col = (kSymG * JB + b) * kBM;
                mbar_expect_tx(full_bar(q), kSymTileBytes);
                if (a_keep > 0.0f) {
                    tma_load_2d_hint(dst, &tmA, col, row, full_bar(q), pol);
                    tma_load_2d_hint(dst + kSymTileBytes / 2, &tmA, col + 64, row, full_bar(q), pol);
                } else {
                    tma_load_2d(dst, &tmA, col, row, full_bar(q));
                    tma_load_2d(dst + kSymTileBytes / 2, &tmA, col + 64, row, full_bar(q));
                }
                ++issued;
                if (++q == stages) {
                    q = 0;
                    parity ^= 1u;
                }
                return true;
            };
            int a = 0, b = 0;
            // prefetch up to `stages` tiles before the X blocks
            for (; a < kSymG && pre_done < stages; ) {
                if (tile_ok(IB, JB, a, b)) {
                    if (!issue_tile(a, b)) break;
                    ++pre_done;
                }
                if (++b == kSymG) {
                    b = 0;
                    ++a;
                }
            }
            if (abort_flag) break;
            if (!waited) {
                pdl_wait();
                waited = true;
            }
            if (st > 0 && !mbar_wait(b_free, (uint32_t)((st - 1) & 1), err, 32, false, spin)) {
                abort_flag = 1;
                break;
            }
            mbar_expect_tx(b_full, 2u * kSymG * bblk);
            for (int g = 0; g < 2 * kSymG; ++g) {
                // blocks 0-3: X rows of row blocks 4 IB + g (MMA2's K); 4-7:
                // X rows of column blocks 4 JB + g - 4 (MMA1's K)
                const int blk = g < kSymG ? kSymG * IB + g : kSymG * JB + g - kSymG;
                const uint32_t dst = b_base + (uint32_t)g * bblk;
                tma_load_2d(dst, &tmB, blk * kBM, 0, b_full);
                tma_load_2d(dst + bbox, &tmB, blk * kBM + 64, 0, b_full);
            }
            for (; a < kSymG && !abort_flag; ) {
                if (tile_ok(IB, JB, a, b) && !issue_tile(a, b)) break;
                if (++b == kSymG) {
                    b = 0;
                    ++a;
                }
            }
        }
        if (!waited) pdl_wait();
        issued_count = issued;
        pdl_trigger();
    } else if (warp == kStreamMma && lane == 0) {
        const uint32_t id_k = prm.idesc;
        const uint32_t id_mn = prm.idesc | (1u << 15);  // A transposed (MN-major)
        int q = 0;
        uint32_t parity = 0;
        int st = 0;
        for (int it = blockIdx.x; it < prm.items && !abort_flag; it += G, ++st) {
            int IB, JB;
            sym_item(it, nS, IB, JB);
            if (st > 0 && !mbar_wait(acc_empty, (uint32_t)((st - 1) & 1), err, 33, false, spin)) {
                abort_flag = 1;
                break;
            }
            if (!mbar_wait(b_full, (uint32_t)(st & 1), err, 34, false, spin)) {
                abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            uint32_t r_started = 0, c_started = 0;
            for (int a = 0; a < kSymG && !abort_flag; ++a) {
                for (int b = 0; b < kSymG; ++b) {
                    if (!tile_ok(IB, JB, a, b)) continue;
                    if (!mbar_wait(full_bar(q), parity, err, 35, false, spin)) {
                        abort_flag = 1;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t ta = a_base + (uint32_t)q * kSymTileBytes;
                    const uint32_t xr = b_base + (uint32_t)a * bblk;            // X[ib]
                    const uint32_t xc = b_base + (uint32_t)(kSymG + b) * bblk;  // X[jb]
                    const uint32_t accR = tmem + (uint32_t)(a * prm.p_pad);
                    const uint32_t accC = tmem + (uint32_t)((kSymG + b) * prm.p_pad);
                    const bool diag = kSymG * IB + a == kSymG * JB + b;
#pragma unroll
                    for (int kk = 0; kk < 8; ++kk) {
                        const uint32_t h = (uint32_t)(kk >> 2), sub = (uint32_t)(kk & 3);
                        // Y[ib] += T X[jb]: K = columns j of the tile
                        umma<KIND>(accR, sw128_desc(ta + h * (kSymTileBytes / 2)) + 2 * sub,
                                   sw128_desc(xc + h * bbox) + 2 * sub, id_k,
                                   ((r_started >> a) & 1u) | (kk > 0 ? 1u : 0u));
                    }
                    r_started |= 1u << a;
                    if (!diag) {
#pragma unroll
                        for (int kk = 0; kk < 8; ++kk) {
                            const uint32_t h = (uint32_t)(kk >> 2), sub = (uint32_t)(kk & 3);
                            // Y[jb] += T^T X[ib]: K = rows i of the tile, 16 per step
                            umma<KIND>(accC, mn_sw128_desc(ta + (uint32_t)kk * 2048u),
                                       sw128_desc(xr + h * bbox) + 2 * sub, id_mn,
                                       ((c_started >> b) & 1u) | (kk > 0 ? 1u : 0u));
                        }
                        c_started |= 1u << b;
                    }
                    umma_commit(empty_bar(q));
                    if (++q == stages) {
                        q = 0;
                        parity ^= 1u;
                    }
                }
            }
            if (abort_flag) break;
            umma_commit(b_free);
            umma_commit(acc_full);
        }
        umma_commit(mma_done);
    } else if (warp < 4) {
        // ---- epilogue: 8 accumulators of a super-tile -> their slots ----
        int st = 0;
        for (int it = blockIdx.x; it < prm.items; it += G, ++st) {
            int IB, JB;
            sym_item(it, nS, IB, JB);
            const bool ok0 = mbar_wait(acc_full, (uint32_t)(st & 1), err, 36, true, spin);
            if (__any_sync(0xffffffffu, !ok0 || abort_flag)) {
                abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int g = 0; g < 2 * kSymG; ++g) {
                const bool row_role = g < kSymG;
                const int blk = row_role ? kSymG * IB + g : kSymG * JB + g - kSymG;
                if (blk >= nb) continue;
                // did any tile of the super-tile reach this accumulator?
                bool touched = false;
                for (int o = 0; o < kSymG; ++o) {
                    if (row_role) {
                        touched = touched || tile_ok(IB, JB, g, o);
                    } else {
                        touched = touched || (tile_ok(IB, JB, o, g - kSymG) &&
                                              kSymG * IB + o != blk);
                    }
                }
                const int R = blk / kSymG;
                const int slot = row_role ? JB - IB : nS - R + IB;
                const int row = blk * kBM + warp * 32 + lane;
                float *dst = P + (size_t)slot * prm.p * (size_t)prm.n + row;
                for (int cb = 0; cb < prm.p_pad; cb += 32) {
                    float v[32];
                    if (touched) {
                        tmem_ld_32cols(tmem + ((uint32_t)(warp * 32) << 16) +
                                           (uint32_t)(g * prm.p_pad + cb),
                                       v);
                    } else {
#pragma unroll
                        for (int j = 0; j < 32; ++j) v[j] = 0.0f;
                    }
                    if (row < prm.n) {
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            if (cb + j < prm.p) dst[(size_t)(cb + j) * prm.n] = v[j];
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(acc_empty);
        }
    }
    __syncwarp();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == kStreamProducer && lane == 0) {
        mbar_wait(mma_done, 0u, err, 37, true);
        if (abort_flag) {
            const int issued = issued_count;
            for (int i = max(0, issued - stages); i < issued; ++i) {
                mbar_wait(full_bar(i % stages), (uint32_t)((i / stages) & 1), err, 38, true);
            }
        }
    }
    __syncthreads();
    if (warp == kStreamProducer) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512)
                     : "memory");
    }
}

}  // namespace tc

// FP32 storage of a TF32 tensor-core operand (values pre-rounded to TF32).
struct tf32_t {
    float v;
};

// ---------------------------------------------------------------------------
// Delta conversion: out[i * ldp + l] = lp(scale * H[i, l]) for l != i, 0 on the
// diagonal and in the padding columns.  H column-major (ld = n).  32x32 tiles
// through shared memory so that both the read and the write are coalesced.
// ---------------------------------------------------------------------------
template <typename LP>
__device__ __forceinline__ LP to_lp(float v);
template <>
__device__ __forceinline__ __half to_lp<__half>(float v)
{
    return __float2half_rn(v);
}
template <>
__device__ __forceinline__ __nv_bfloat16 to_lp<__nv_bfloat16>(float v)
{
    return __float2bfloat16_rn(v);
}
template <>
__device__ __forceinline__ float to_lp<float>(float v)
{
    return v;
}
template <>
__device__ __forceinline__ tf32_t to_lp<tf32_t>(float v)
{
    // TF32 operand: round to nearest into the 10-bit mantissa kept by the
    // tensor core (cvt.rna.tf32.f32 returns the rounded value in fp32 bits).
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
    tf32_t t;
    t.v = __uint_as_float(r);
    return t;
}

// Delta (row-major, diagonal zeroed, scaled) in LP; with hi/lo also the
// double-FP32 split of the full H in the same pass over H.
template <typename LP>
__global__ void convert_delta_kernel(const double *__restrict__ H, int n, int ldp, double scale,
                                     LP *__restrict__ out, float *__restrict__ hi,
                                     float *__restrict__ lo)
{
    __shared__ float tile[32][33];
    const int l0 = blockIdx.x * 32;  // column block of H (= K index)
    const int i0 = blockIdx.y * 32;  // row block of H
    const int tx = threadIdx.x;      // 0..31
    for (int ty = threadIdx.y; ty < 32; ty += blockDim.y) {
        const int i = i0 + tx;
        const int l = l0 + ty;
        float v = 0.0f;
        if (i < n && l < n) {
            const size_t o = (size_t)i + (size_t)l * n;
            const double h = H[o];
            if (i != l) v = (float)(scale * h);
            if (hi != nullptr) {
                const float hh = __double2float_rn(h);
                hi[o] = hh;
                lo[o] = __double2float_rn(h - (double)hh);
            }
        }
        tile[ty][tx] = v;  // tile[l - l0][i - i0]
    }
    __syncthreads();
    for (int ty = threadIdx.y; ty < 32; ty += blockDim.y) {
        const int i = i0 + ty;
        const int l = l0 + tx;
        if (i < n && l < ldp) {
            out[(size_t)i * ldp + l] = to_lp<LP>(tile[tx][ty]);
        }
    }
}

// The same conversion for a symmetric H without the transpose: row i of
// Delta is column i of H, so the pass streams H column by column, writes
// Delta rows and (with hi/lo) the split in H's own layout.  One CTA covers
// 2048 entries of one column; each thread two adjacent entries per step
// (double2 loads when vec: n even and H 16-byte aligned).
constexpr int kSymChunk = kLowpColsumChunk;
template <typename LP>
struct alignas(2 * sizeof(LP)) LpPair {  // two adjacent Delta entries, one store
    LP x, y;
};
// One entry: (hi, lo) from the integer-pipe split, and the Delta value
// RN_float(2^s2 h) = 2^s2 hi when both are normal floats (s2 is the exponent
// of the power-of-two scale).
__device__ __forceinline__ float sym_entry(double h, int s2, double scale, float &hi, float &lo)
{
    uint32_t hb, lb;
    if (split_double_bits((unsigned long long)__double_as_longlong(h), &hb, &lb)) {
        hi = __uint_as_float(hb);
        lo = __uint_as_float(lb);
        const int ex = (int)((hb >> 23) & 0xFFu) + s2;
        if (ex >= 1 && ex <= 254) {
            return __uint_as_float(hb + ((uint32_t)s2 << 23));
        }
    } else {
        hi = __double2float_rn(h);
        lo = __double2float_rn(h - (double)hi);
    }
    return (float)(scale * h);
}

// (S, C) += (So, Co) for double-float pairs
__device__ __forceinline__ void df_pair_add(float &S, float &C, float So, float Co)
{
    const float t = __fadd_rn(S, So);
    const float bp = __fsub_rn(t, S);
    const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(t, bp)), __fsub_rn(So, bp));
    S = t;
    C = __fadd_rn(__fadd_rn(C, Co), err);
}

template <typename LP>
__global__ void __launch_bounds__(256)
    convert_delta_sym_kernel(const double *__restrict__ H, int n, int ldp, double scale, int s2,
                             bool vec, LP *__restrict__ out, float *__restrict__ hi,
                             float *__restrict__ lo, double *__restrict__ colpart)
{
    const int c = blockIdx.x;  // column of H = row of Delta
    const size_t col = (size_t)c * n;
    LP *orow = out + (size_t)c * ldp;
    float S = 0.0f, C = 0.0f;  // this thread's share of the column sum of |H|
#pragma unroll
    for (int u = 0; u < kSymChunk / 512; ++u) {
        const int l = blockIdx.y * kSymChunk + u * 512 + 2 * threadIdx.x;  // even
        if (l >= ldp) break;  // ldp is a multiple of 64: l + 1 < ldp as well
        double h0 = 0.0, h1 = 0.0;
        if (vec && l + 1 < n) {
            const double2 v = *reinterpret_cast<const double2 *>(H + col + l);
            h0 = v.x;
            h1 = v.y;
        } else {
            if (l < n) h0 = H[col + l];
            if (l + 1 < n) h1 = H[col + l + 1];
        }
        float a0, a1, b0, b1;
        float v0 = sym_entry(h0, s2, scale, a0, b0);
        float v1 = sym_entry(h1, s2, scale, a1, b1);
        if (!(l < n && l != c)) v0 = 0.0f;
        if (!(l + 1 < n && l + 1 != c)) v1 = 0.0f;
        if (colpart != nullptr) {
            df_abs_add(S, C, a0, b0);  // entries beyond n are zero
            df_abs_add(S, C, a1, b1);
        }
        *reinterpret_cast<LpPair<LP> *>(orow + l) = LpPair<LP>{to_lp<LP>(v0), to_lp<LP>(v1)};
        if (hi != nullptr) {
            if (vec && l + 1 < n) {
                *reinterpret_cast<float2 *>(hi + col + l) = make_float2(a0, a1);
                *reinterpret_cast<float2 *>(lo + col + l) = make_float2(b0, b1);
            } else {
                if (l < n) {
                    hi[col + l] = a0;
                    lo[col + l] = b0;
                }
                if (l + 1 < n) {
                    hi[col + l + 1] = a1;
                    lo[col + l + 1] = b1;
                }
            }
        }
    }
    if (colpart != nullptr) {
        // fixed-order reduction: lanes, then the 8 warps
        for (int off = 16; off > 0; off >>= 1) {
            df_pair_add(S, C, __shfl_xor_sync(0xffffffffu, S, off),
                        __shfl_xor_sync(0xffffffffu, C, off));
        }
        __shared__ float red[2][8];
        const int w = threadIdx.x >> 5;
        if ((threadIdx.x & 31) == 0) {
            red[0][w] = S;
            red[1][w] = C;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            float St = red[0][0], Ct = red[1][0];
            for (int q = 1; q < 8; ++q) df_pair_add(St, Ct, red[0][q], red[1][q]);
            colpart[(size_t)blockIdx.y * n + c] = (double)St + (double)Ct;
        }
    }
}

// Fused setup of a symmetric H: one CTA per column c (= row c of Delta).
// Pass 0 reads the column (writing the FP64 device copy when the source is
// host memory) and finds its largest off-diagonal |h| (integer max of the bit
// patterns); the row's FP16 scale is the largest power of two 2^s2 with
// 2^s2 max <= 16384 (BF16/TF32: 1).  Pass 1 re-reads the column from device
// memory (L2-resident by then: the source over the host link is read once)
// and writes row c of Delta and the double-FP32 split of column c, and forms
// the exact double-float column sum.  The CTA's thread 0 then stores 2^-s2, the
// diagonal entry, the column sum (atomic max: hnorm), its maximum and whether
// d_{c+1} < d_c.  No FP64 arithmetic per entry (the conversions run on the
// integer pipe), so the pass streams at memory (or host link) speed.
template <typename LP>
__global__ void __launch_bounds__(256)
    fused_setup_kernel(const double *__restrict__ src, int n, int ldp, int fp16_scale,
                       double *__restrict__ copy, LP *__restrict__ delta, float *__restrict__ hi,
                       float *__restrict__ lo, float *__restrict__ inv_row,
                       double *__restrict__ diag, DenseStats *__restrict__ stats, int vec,
                       __half *__restrict__ oz, int *__restrict__ oz_rowexp, int c0)
{
    __shared__ unsigned long long wmax[8];
    __shared__ float wS[8], wC[8];
    __shared__ int s2_sh;
    const int c = c0 + blockIdx.x;
    const int tid = threadIdx.x;
    const double *scol = src + (size_t)c * n;
    double *ccol = copy != nullptr ? copy + (size_t)c * n : nullptr;
    unsigned long long m = 0;
    if (vec) {  // n even, src (and copy) 16-byte aligned
        const double2 *s2v = reinterpret_cast<const double2 *>(scol);
        for (int q = tid; q < n / 2; q += 256) {
            const double2 v = s2v[q];
            if (ccol != nullptr) reinterpret_cast<double2 *>(ccol)[q] = v;
            const int l = 2 * q;
            const unsigned long long a0 =
                (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFULL;
            const unsigned long long a1 =
                (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFULL;
            if (l != c && a0 > m) m = a0;
            if (l + 1 != c && a1 > m) m = a1;
        }
    } else {
        for (int l = tid; l < n; l += 256) {
            const double v = scol[l];
            if (ccol != nullptr) ccol[l] = v;
            const unsigned long long a =
                (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFULL;
            if (l != c && a > m) m = a;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, m, off);
        if (o > m) m = o;
    }
    if ((tid & 31) == 0) wmax[tid >> 5] = m;
    __syncthreads();
    if (tid == 0) {
        unsigned long long mx = 0;
        for (int w = 0; w < 8; ++w) mx = wmax[w] > mx ? wmax[w] : mx;
        wmax[0] = mx;
        int s2 = 0;
        const double mv = __longlong_as_double((long long)mx);
        if (fp16_scale && mv > 0.0 && isfinite(mv)) {
            s2 = (int)floor(log2(16384.0 / mv));
            s2 = min(max(s2, -40), 40);
        }
        s2_sh = s2;
    }
    __syncthreads();
    const int s2 = s2_sh;
    const double scale = ldexp(1.0, s2);
    // exponent of row c's digit slices (symmetric H: column c is row c)
    const int oz_e = oz_exponent(wmax[0]);
    // the block's pass-0 writes of the copy are visible after the barrier;
    // pass 1 reads with ld.global.cg (coherent at L2), never through the
    // read-only path, since the copy is written by this kernel
    const double *rcol = ccol != nullptr ? ccol : scol;
    LP *orow = delta + (size_t)c * ldp;
    float S = 0.0f, C = 0.0f;
    for (int l = 2 * tid; l < ldp; l += 512) {  // ldp is a multiple of 64: l + 1 < ldp
        double h0 = 0.0, h1 = 0.0;
        if (vec && l + 1 < n) {
            const double2 v = __ldcg(reinterpret_cast<const double2 *>(rcol + l));
            h0 = v.x;
            h1 = v.y;
        } else {
            if (l < n) h0 = __ldcg(rcol + l);
            if (l + 1 < n) h1 = __ldcg(rcol + l + 1);
        }
        float a0, a1, b0, b1;
        float v0 = sym_entry(h0, s2, scale, a0, b0);
        float v1 = sym_entry(h1, s2, scale, a1, b1);
        if (!(l < n && l != c)) v0 = 0.0f;
        if (!(l + 1 < n && l + 1 != c)) v1 = 0.0f;
        *reinterpret_cast<LpPair<LP> *>(orow + l) = LpPair<LP>{to_lp<LP>(v0), to_lp<LP>(v1)};
        if (oz != nullptr) {
            oz_store_pair((l < n && l != c) ? h0 : 0.0, (l + 1 < n && l + 1 != c) ? h1 : 0.0,
                          oz_e, reinterpret_cast<__half2 *>(oz + (size_t)c * ldp + l),
                          (size_t)n * (size_t)ldp / 2);
        }
        df_abs_add(S, C, a0, b0);  // entries beyond n are zero
        df_abs_add(S, C, a1, b1);
        const size_t o = (size_t)c * n + l;
        if (vec && l + 1 < n) {
            if (hi != nullptr) {
                *reinterpret_cast<float2 *>(hi + o) = make_float2(a0, a1);
                *reinterpret_cast<float2 *>(lo + o) = make_float2(b0, b1);
            }
        } else {
            if (l < n) {
                if (hi != nullptr) {
                    hi[o] = a0;
                    lo[o] = b0;
                }
            }
            if (l + 1 < n) {
                if (hi != nullptr) {
                    hi[o + 1] = a1;
                    lo[o + 1] = b1;
                }
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        df_pair_add(S, C, __shfl_xor_sync(0xffffffffu, S, off),
                    __shfl_xor_sync(0xffffffffu, C, off));
    }
    if ((tid & 31) == 0) {
        wS[tid >> 5] = S;
        wC[tid >> 5] = C;
    }
    __syncthreads();
    if (tid == 0) {
        float St = wS[0], Ct = wC[0];
        for (int w = 1; w < 8; ++w) df_pair_add(St, Ct, wS[w], wC[w]);
        const double colsum = (double)St + (double)Ct;
        if (colsum > 0.0) {
            atomicMax(&stats->hnorm_bits, (unsigned long long)__double_as_longlong(colsum));
        }
        if (wmax[0] > 0) atomicMax(&stats->maxabs_bits, wmax[0]);
        const double dc = __ldcg(rcol + c);
        diag[c] = dc;
        if (c + 1 < n && src[(size_t)(c + 1) * ((size_t)n + 1)] < dc) {
            atomicAdd(&stats->descents, 1ULL);
        }
        inv_row[c] = (float)ldexp(1.0, -s2);
        if (oz_rowexp != nullptr) oz_rowexp[c] = oz_e;
    }
}

// Upper triangle of a symmetric H (column-major, ld = n) in pinned host
// memory -> device memory, columns [c0, c1): column j's rows 0..j, read as
// one contiguous run (16-byte loads, kCopyInFlight in flight per thread:
// host-memory reads wait about 11 us under load on GB300, and 211 GB/s
// over the host link needs ~2.4 MB in flight, i.e. one such CTA per SM,
// which leaves the rest of each SM to the setup pass of finished chunks).
// CTA b takes the columns c1 - 1 - b, c1 - 1 - b - G, ...: neighbouring
// columns are nearly the same length, so the CTAs stay balanced.
constexpr int kCopyInFlight = 8;
__global__ void __launch_bounds__(256)
upper_copy_kernel(const double *__restrict__ host, int n, int c0, int c1, double *__restrict__ dev,
                  int pairs_ok)
{
    if (!pairs_ok) {
        // odd n or an 8-byte aligned host copy: 8-byte loads
        for (int j = c1 - 1 - (int)blockIdx.x; j >= c0; j -= (int)gridDim.x) {
            const size_t off = (size_t)j * n;
            for (int q0 = threadIdx.x; q0 <= j; q0 += kCopyInFlight * blockDim.x) {
                double v[kCopyInFlight];
#pragma unroll
                for (int r = 0; r < kCopyInFlight; ++r) {
                    const int q = q0 + r * (int)blockDim.x;
                    if (q <= j) v[r] = host[off + q];
                }
#pragma unroll
                for (int r = 0; r < kCopyInFlight; ++r) {
                    const int q = q0 + r * (int)blockDim.x;
                    if (q <= j) dev[off + q] = v[r];
                }
            }
        }
        return;
    }
    for (int j = c1 - 1 - (int)blockIdx.x; j >= c0; j -= (int)gridDim.x) {
        const size_t off = (size_t)j * n;  // n even: 16-byte aligned
        const int pairs = (j + 1) / 2;     // rows 0 .. 2 pairs - 1
        const double2 *src = reinterpret_cast<const double2 *>(host + off);
        double2 *dst = reinterpret_cast<double2 *>(dev + off);
        for (int q0 = threadIdx.x; q0 < pairs; q0 += kCopyInFlight * blockDim.x) {
            double2 v[kCopyInFlight];
#pragma unroll
            for (int r = 0; r < kCopyInFlight; ++r) {
                const int q = q0 + r * (int)blockDim.x;
                if (q < pairs) v[r] = src[q];
            }
#pragma unroll
            for (int r = 0; r < kCopyInFlight; ++r) {
                const int q = q0 + r * (int)blockDim.x;
                if (q < pairs) dst[q] = v[r];
            }
        }
        if ((j & 1) == 0 && threadIdx.x == 0) dev[off + j] = host[off + j];  // the diagonal
    }
}

// Lower triangle of the columns [c0, c1) of the device copy from the upper
// triangle: entry (j, i), j > i, = entry (i, j) of column j.  32 x 32 tiles
// (ib = column block of i in the chunk, jb >= ib) through shared memory.
__global__ void __launch_bounds__(256)
mirror_lower_kernel(double *__restrict__ dev, int n, int ib0, int ib1)
{
    __shared__ double t[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int nb = (n + 31) / 32;
    // tiles (ib, jb) with ib0 <= ib < ib1, ib <= jb < nb, numbered row by
    // row (nb - ib tiles in row ib)
    for (long long q = blockIdx.x;; q += gridDim.x) {
        long long rem = q;
        int ib = ib0;
        while (ib < ib1 && rem >= nb - ib) {
            rem -= nb - ib;
            ++ib;
        }
        if (ib >= ib1) break;
        const int jb = ib + (int)rem;
        const int i0 = ib * 32, j0 = jb * 32;
        // read tile rows i0.., columns j0.. (upper part: i < j) of column j
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int j = j0 + ty + 8 * r, i = i0 + tx;
            t[ty + 8 * r][tx] = (j < n && i < j) ? dev[(size_t)j * n + i] : 0.0;
        }
        __syncthreads();
        // write column i (i0 + ii), rows j0 + tx (> i)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int ii = ty + 8 * r;
            const int i = i0 + ii, j = j0 + tx;
            if (j < n && i < j) dev[(size_t)i * n + j] = t[tx][ii];
        }
        __syncthreads();
    }
}

__device__ __forceinline__ float lp_to_float(__half v) { return __half2float(v); }
__device__ __forceinline__ float lp_to_float(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float lp_to_float(tf32_t v) { return v.v; }
__device__ __forceinline__ float lp_to_float(float v) { return v; }

// One common power-of-two scale for every row of a per-row scaled Delta (so
// that the stored matrix is symmetric again, for the symmetric product):
// the largest 1 / scale over the rows (one CTA), then each row multiplied by
// its own 1 / scale over that largest one (a power of two <= 1: exact unless
// an entry leaves FP16's normal range) and given the common 1 / scale.
__global__ void __launch_bounds__(256) max_inv_row_kernel(const float *__restrict__ inv_row, int n,
                                                          float *__restrict__ out)
{
    __shared__ float w[8];
    float m = 0.0f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, inv_row[i]);
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < 8; ++k) m = fmaxf(m, w[k]);
        out[0] = fmaxf(m, w[0]);
    }
}

template <typename LP>
__global__ void __launch_bounds__(256) common_row_scale_kernel(LP *__restrict__ delta, int ldp,
                                                               float *__restrict__ inv_row,
                                                               const float *__restrict__ gmax)
{
    const int row = blockIdx.x;
    const float g = gmax[0];
    const float f = inv_row[row] / g;  // power of two, <= 1
    if (f != 1.0f) {
        LP *r = delta + (size_t)row * ldp;
        for (int l = threadIdx.x; l < ldp; l += blockDim.x) {
            r[l] = to_lp<LP>(lp_to_float(r[l]) * f);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) inv_row[row] = g;
}

__global__ void max_abs_offdiag_kernel(const double *__restrict__ H, int n,
                                       unsigned long long *out)
{
    double m = 0.0;
    const size_t total = (size_t)n * n;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t i = e % (size_t)n;
        const size_t l = e / (size_t)n;
        if (i != l) {
            m = fmax(m, fabs(H[e]));
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, (unsigned long long)__double_as_longlong(m));
    }
}

// G_ij = 1 / (d_j - d_i) as FP32 (0 on the target position, NaN for a zero
// or non-finite gap); computed once per solve in FP64 then rounded.
__global__ void build_g32_kernel(const double *__restrict__ d, int n, int p, float *__restrict__ G)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n * p) return;
    const int i = (int)(e % (size_t)n);
    const int j = (int)(e / (size_t)n);
    float g = 0.0f;
    if (i != j) {
        const double gap = d[j] - d[i];
        g = (isfinite(gap) && gap != 0.0) ? (float)(1.0 / gap) : __int_as_float(0x7fc00000);
    }
    G[e] = g;
}

template <typename LP>
__global__ void lowp_identity_kernel(float *X32, LP *Xlp, int n, int p, int ldx)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n * p) return;
    const int i = (int)(e % (size_t)n);
    const int j = (int)(e / (size_t)n);
    const float v = i == j ? 1.0f : 0.0f;
    X32[e] = v;
    Xlp[(size_t)i + (size_t)j * ldx] = to_lp<LP>(v);
}

// History of the device-side stop (NormScratch): a stopped step copies the
// previous entry forward; a running step adds its block's sums.
__device__ __forceinline__ void hist_carry(double *hist, int step)
{
    if (blockIdx.x == 0 && threadIdx.x == 0 && step > 0) {
        hist[2 * step] = __ldcg(hist + 2 * (step - 1));
        hist[2 * step + 1] = __ldcg(hist + 2 * (step - 1) + 1);
    }
}

__device__ __forceinline__ void hist_add(double *hist, int step, double2 t)
{
    if (threadIdx.x == 0) {
        atomicAdd(hist + 2 * step, t.x);
        atomicAdd(hist + 2 * step + 1, t.y);
    }
}

// Low-precision IPT update (see file header); Delta has a zero diagonal so
// c_j = (Delta X)_jj is read straight from the product.
template <typename LP>
__global__ void lowp_update_kernel(const float *__restrict__ P, int S, int n, int p,
                                   float inv_scale, const float *__restrict__ inv_row,
                                   const float *__restrict__ G,
                                   const float *__restrict__ X, float *__restrict__ Xn,
                                   LP *__restrict__ Xlp, int ldx, int want_norms,
                                   double2 *partials, unsigned int *counter, double *norms,
                                   double *hist, int step, double stop_tol)
{
    pdl_wait();  // P and X come from the previous grids
    pdl_trigger();
    // grid-stride over the block (a few CTAs per SM)
    const size_t elems = (size_t)n * (size_t)p;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    if (hist_stopped(hist, step, stop_tol)) {
        // stopped: pass the block through to the next buffer pair
        for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < elems;
             idx += stride) {
            const float x = X[idx];
            Xn[idx] = x;
            Xlp[(idx % (size_t)n) + (idx / (size_t)n) * (size_t)ldx] = to_lp<LP>(x);
        }
        hist_carry(hist, step);
        return;
    }
    want_norms = want_norms || hist != nullptr;
    double dsq = 0.0, xsq = 0.0;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < elems; idx += stride) {
        const int row = (int)(idx % (size_t)n);
        const int col = (int)(idx / (size_t)n);
        const float x = X[idx];
        float out = 1.0f;
        if (row != col) {
            float y = 0.0f, c = 0.0f;
            for (int s = 0; s < S; ++s) {
                const size_t base = ((size_t)s * p + col) * (size_t)n;
                y += P[base + row];
                c += P[base + col];
            }
            const float ir = inv_row != nullptr ? inv_row[row] : inv_scale;
            const float ic = inv_row != nullptr ? inv_row[col] : inv_scale;
            out = (y * ir - x * (c * ic)) * G[idx];
        }
        Xn[idx] = out;
        Xlp[(size_t)row + (size_t)col * ldx] = to_lp<LP>(out);
        if (want_norms) {
            const double df = (double)out - (double)x;
            dsq = fma(df, df, dsq);
            xsq = fma((double)x, (double)x, xsq);
        }
    }
    if (hist != nullptr) {
        hist_add(hist, step, block_sum2(dsq, xsq));
    } else if (want_norms) {
        const double2 t = block_sum2(dsq, xsq);
        grid_finish_norms2(t, partials, counter, norms);
    }
}

// Four consecutive rows per thread (n % 4 == 0): the same update as
// lowp_update_kernel with 16-byte loads and stores and 32-bit index math;
// the update is latency-bound, so fewer and wider accesses shorten it.
template <typename LP>
struct alignas(4 * sizeof(LP)) LpQuad {
    LP a, b, c, d;
};

__device__ __forceinline__ float4 f4_add(float4 a, float4 b)
{
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

__device__ __forceinline__ float &f4_at(float4 &v, int i)
{
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// The sum over the product's partial slots of four rows (row0..row0+3) of
// column col, and of the diagonal entry (col, col), in slot order: the loads
// of up to kSlotsUnrolled slots are issued together (the update is bound by
// their latency, not by bandwidth), the adds keep the fixed order.
constexpr int kSlotsUnrolled = 8;

__device__ __forceinline__ void sum_slots4(const float *__restrict__ P, int S, int p, int n,
                                           int col, int row0, float4 &y, float &c)
{
    float4 v[kSlotsUnrolled];
    float d[kSlotsUnrolled];
#pragma unroll
    for (int s = 0; s < kSlotsUnrolled; ++s) {
        if (s < S) {
            const float *base = P + ((size_t)s * p + col) * (size_t)n;
            v[s] = *reinterpret_cast<const float4 *>(base + row0);
            d[s] = base[col];
        }
    }
#pragma unroll
    for (int s = 0; s < kSlotsUnrolled; ++s) {
        if (s < S) {
            y = f4_add(y, v[s]);
            c += d[s];
        }
    }
    for (int s = kSlotsUnrolled; s < S; ++s) {
        const float *base = P + ((size_t)s * p + col) * (size_t)n;
        y = f4_add(y, *reinterpret_cast<const float4 *>(base + row0));
        c += base[col];
    }
}

// Anderson mixing (lowp.h set_mixing): Xn receives the map's value f and
// Gout (non-null) g = f - x; Xlp may be null (the mixing kernel writes the
// operand).  mix_part: with n % 1024 == 0 and one item per thread, CTA b
// covers the 1024-row chunk b of one column; it stores that chunk's
// <g, g - Gprev> and ||g - Gprev||^2 in mix_part[b].  Null: not formed here.
template <typename LP>
__global__ void lowp_update4_kernel(const float *__restrict__ P, int S, int n, int p,
                                    float inv_scale, const float *__restrict__ inv_row,
                                    const float *__restrict__ G,
                                    const float *__restrict__ X, float *__restrict__ Xn,
                                    LP *__restrict__ Xlp, int ldx, int want_norms,
                                    double2 *partials, unsigned int *counter, double *norms,
                                    double *hist, int step, double stop_tol,
                                    const float *__restrict__ Gprev, float *__restrict__ Gout,
                                    double2 *__restrict__ mix_part)
{
    pdl_wait();  // P and X come from the previous grids
    pdl_trigger();
    const int nq = n >> 2;
    const int total = nq * p;
    const int stride = gridDim.x * blockDim.x;
    if (hist_stopped(hist, step, stop_tol)) {
        for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += stride) {
            const int col = q / nq;
            const int row0 = (q - col * nq) << 2;
            const size_t e = (size_t)col * n + row0;
            const float4 x = *reinterpret_cast<const float4 *>(X + e);
            *reinterpret_cast<float4 *>(Xn + e) = x;
            *reinterpret_cast<LpQuad<LP> *>(Xlp + (size_t)col * ldx + row0) =
                LpQuad<LP>{to_lp<LP>(x.x), to_lp<LP>(x.y), to_lp<LP>(x.z), to_lp<LP>(x.w)};
        }
        hist_carry(hist, step);
        return;
    }
    want_norms = want_norms || hist != nullptr;
    float dsq = 0.0f, xsq = 0.0f;
    double ma = 0.0, mb = 0.0;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += stride) {
        const int col = q / nq;
        const int row0 = (q - col * nq) << 2;
        const size_t e = (size_t)col * n + row0;
        float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
        float c = 0.0f;
        sum_slots4(P, S, p, n, col, row0, y, c);
        const float4 x = *reinterpret_cast<const float4 *>(X + e);
        const float4 g = *reinterpret_cast<const float4 *>(G + e);
        const float4 ir = inv_row != nullptr
                              ? *reinterpret_cast<const float4 *>(inv_row + row0)
                              : make_float4(inv_scale, inv_scale, inv_scale, inv_scale);
        const float ci = c * (inv_row != nullptr ? inv_row[col] : inv_scale);
        float4 o;
        o.x = (y.x * ir.x - x.x * ci) * g.x;
        o.y = (y.y * ir.y - x.y * ci) * g.y;
        o.z = (y.z * ir.z - x.z * ci) * g.z;
        o.w = (y.w * ir.w - x.w * ci) * g.w;
        if (col >= row0 && col < row0 + 4) f4_at(o, col - row0) = 1.0f;  // X_jj = 1
        *reinterpret_cast<float4 *>(Xn + e) = o;
        if (Xlp != nullptr) {
            *reinterpret_cast<LpQuad<LP> *>(Xlp + (size_t)col * ldx + row0) =
                LpQuad<LP>{to_lp<LP>(o.x), to_lp<LP>(o.y), to_lp<LP>(o.z), to_lp<LP>(o.w)};
        }
        if (Gout != nullptr) {
            *reinterpret_cast<float4 *>(Gout + e) =
                make_float4(o.x - x.x, o.y - x.y, o.z - x.z, o.w - x.w);
        }
        if (want_norms) {
            const float d0 = o.x - x.x, d1 = o.y - x.y, d2 = o.z - x.z, d3 = o.w - x.w;
            dsq += d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3;
            xsq += x.x * x.x + x.y * x.y + x.z * x.z + x.w * x.w;
        }
        if (mix_part != nullptr) {
            const float4 gp = *reinterpret_cast<const float4 *>(Gprev + e);
            const float g0 = o.x - x.x, g1 = o.y - x.y, g2 = o.z - x.z, g3 = o.w - x.w;
            const float e0 = g0 - gp.x, e1 = g1 - gp.y, e2 = g2 - gp.z, e3 = g3 - gp.w;
            ma += (double)g0 * e0 + (double)g1 * e1 + (double)g2 * e2 + (double)g3 * e3;
            mb += (double)e0 * e0 + (double)e1 * e1 + (double)e2 * e2 + (double)e3 * e3;
        }
    }
    if (mix_part != nullptr) {
        const double2 t = block_sum2(ma, mb);
        // only CTAs with items own a chunk (the grid has no others when the
        // host fuses the inner products, but an idle CTA must not write)
        if (threadIdx.x == 0 && (long long)blockIdx.x * blockDim.x < (long long)total) {
            mix_part[blockIdx.x] = t;
        }
    }
    if (hist != nullptr) {
        hist_add(hist, step, block_sum2((double)dsq, (double)xsq));
    } else if (want_norms) {
        grid_finish_norms2(block_sum2((double)dsq, (double)xsq), partials, counter, norms);
    }
}

__global__ void f32_to_f64_kernel(const float *__restrict__ in, size_t count, double *__restrict__ out)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count) out[e] = (double)in[e];
}

// ---------------------------------------------------------------------------
// Mixed refinement: low-precision correction solve (see lowp.h).
// ---------------------------------------------------------------------------
template <typename LP>
__global__ void refine_begin_kernel(const double *__restrict__ R0, const double *__restrict__ X,
                                    const double *__restrict__ c, const float *__restrict__ sigma_in,
                                    int use_sigma, int n, int p, int ldx, float *__restrict__ d32,
                                    LP *__restrict__ dlp, float *__restrict__ R32,
                                    float *__restrict__ X32, float *__restrict__ c32,
                                    float *__restrict__ sig, float *__restrict__ sig_inv)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < (size_t)p) {
        const float sg = use_sigma ? sigma_in[e] : 1.0f;
        sig[e] = sg;
        sig_inv[e] = 1.0f / sg;
        c32[e] = (float)c[e];
    }
    if (e >= (size_t)n * p) return;
    const int row = (int)(e % (size_t)n);
    const int col = (int)(e / (size_t)n);
    const float sg = use_sigma ? sigma_in[col] : 1.0f;
    const float r = (float)R0[e];
    d32[e] = r;
    R32[e] = r;
    X32[e] = (float)X[e];
    dlp[(size_t)row + (size_t)col * ldx] = to_lp<LP>(r * sg);
}

template <typename LP>
__global__ void refine_update_kernel(const float *__restrict__ P, int S, int n, int p,
                                     float inv_scale, const float *__restrict__ inv_row,
                                     const float *__restrict__ sig,
                                     const float *__restrict__ sig_inv, const float *__restrict__ G,
                                     const float *__restrict__ R32, const float *__restrict__ X32,
                                     const float *__restrict__ c32, const float *__restrict__ dcur,
                                     float *__restrict__ dnext, LP *__restrict__ dlp, int ldx,
                                     int want_norms, double2 *partials, unsigned int *counter,
                                     double *norms, double *hist, int step, double stop_tol)
{
    pdl_wait();  // P and X come from the previous grids
    pdl_trigger();
    const size_t elems = (size_t)n * (size_t)p;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    if (hist_stopped(hist, step, stop_tol)) {
        // stopped: pass the correction through to the next buffer pair
        for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < elems;
             idx += stride) {
            const float cur = dcur[idx];
            const int col = (int)(idx / (size_t)n);
            dnext[idx] = cur;
            dlp[(idx % (size_t)n) + (size_t)col * (size_t)ldx] = to_lp<LP>(cur * sig[col]);
        }
        hist_carry(hist, step);
        return;
    }
    want_norms = want_norms || hist != nullptr;
    double dsq = 0.0, xsq = 0.0;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < elems; idx += stride) {
        const int row = (int)(idx % (size_t)n);
        const int col = (int)(idx / (size_t)n);
        const float cur = dcur[idx];
        float out = 0.0f;
        if (row != col) {
            float y = 0.0f, b = 0.0f;
            for (int s = 0; s < S; ++s) {
                const size_t base = ((size_t)s * p + col) * (size_t)n;
                y += P[base + row];
                b += P[base + col];
            }
            const float ir = inv_row != nullptr ? inv_row[row] : inv_scale;
            const float ic = inv_row != nullptr ? inv_row[col] : inv_scale;
            y *= ir * sig_inv[col];
            b *= ic * sig_inv[col];
            out = R32[idx] + (y - X32[idx] * b - cur * (c32[col] + b)) * G[idx];
        }
        dnext[idx] = out;
        dlp[(size_t)row + (size_t)col * ldx] = to_lp<LP>(out * sig[col]);
        if (want_norms) {
            const double df = (double)out - (double)cur;
            dsq = fma(df, df, dsq);
            xsq = fma((double)cur, (double)cur, xsq);
        }
    }
    if (hist != nullptr) {
        hist_add(hist, step, block_sum2(dsq, xsq));
    } else if (want_norms) {
        const double2 t = block_sum2(dsq, xsq);
        grid_finish_norms2(t, partials, counter, norms);
    }
}

// refine_update_kernel with four consecutive rows per thread (n % 4 == 0).
template <typename LP>
__global__ void refine_update4_kernel(const float *__restrict__ P, int S, int n, int p,
                                      float inv_scale, const float *__restrict__ inv_row,
                                      const float *__restrict__ sig,
                                      const float *__restrict__ sig_inv,
                                      const float *__restrict__ G, const float *__restrict__ R32,
                                      const float *__restrict__ X32, const float *__restrict__ c32,
                                      const float *__restrict__ dcur, float *__restrict__ dnext,
                                      LP *__restrict__ dlp, int ldx, int want_norms,
                                      double2 *partials, unsigned int *counter, double *norms,
                                      double *hist, int step, double stop_tol,
                                      const float *__restrict__ Gprev, float *__restrict__ Gout,
                                      double2 *__restrict__ mix_part)
{
    pdl_wait();  // P and X come from the previous grids
    pdl_trigger();
    const int nq = n >> 2;
    const int total = nq * p;
    const int stride = gridDim.x * blockDim.x;
    if (hist_stopped(hist, step, stop_tol)) {
        for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += stride) {
            const int col = q / nq;
            const int row0 = (q - col * nq) << 2;
            const size_t e = (size_t)col * n + row0;
            const float4 cur = *reinterpret_cast<const float4 *>(dcur + e);
            const float sg = sig[col];
            *reinterpret_cast<float4 *>(dnext + e) = cur;
            *reinterpret_cast<LpQuad<LP> *>(dlp + (size_t)col * ldx + row0) =
                LpQuad<LP>{to_lp<LP>(cur.x * sg), to_lp<LP>(cur.y * sg), to_lp<LP>(cur.z * sg),
                           to_lp<LP>(cur.w * sg)};
        }
        hist_carry(hist, step);
        return;
    }
    want_norms = want_norms || hist != nullptr;
    float dsq = 0.0f, xsq = 0.0f;
    double ma = 0.0, mb = 0.0;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += stride) {
        const int col = q / nq;
        const int row0 = (q - col * nq) << 2;
        const size_t e = (size_t)col * n + row0;
        float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
        float b = 0.0f;
        sum_slots4(P, S, p, n, col, row0, y, b);
        const float4 ir = inv_row != nullptr
                              ? *reinterpret_cast<const float4 *>(inv_row + row0)
                              : make_float4(inv_scale, inv_scale, inv_scale, inv_scale);
        const float si = sig_inv[col];
        y = make_float4(y.x * (ir.x * si), y.y * (ir.y * si), y.z * (ir.z * si), y.w * (ir.w * si));
        b *= (inv_row != nullptr ? inv_row[col] : inv_scale) * si;
        const float cb = c32[col] + b;
        const float4 cur = *reinterpret_cast<const float4 *>(dcur + e);
        const float4 r = *reinterpret_cast<const float4 *>(R32 + e);
        const float4 x = *reinterpret_cast<const float4 *>(X32 + e);
        const float4 g = *reinterpret_cast<const float4 *>(G + e);
        float4 o;
        o.x = r.x + (y.x - x.x * b - cur.x * cb) * g.x;
        o.y = r.y + (y.y - x.y * b - cur.y * cb) * g.y;
        o.z = r.z + (y.z - x.z * b - cur.z * cb) * g.z;
        o.w = r.w + (y.w - x.w * b - cur.w * cb) * g.w;
        if (col >= row0 && col < row0 + 4) f4_at(o, col - row0) = 0.0f;  // X_jj stays 1
        *reinterpret_cast<float4 *>(dnext + e) = o;
        if (dlp != nullptr) {
            const float sg = sig[col];
            *reinterpret_cast<LpQuad<LP> *>(dlp + (size_t)col * ldx + row0) =
                LpQuad<LP>{to_lp<LP>(o.x * sg), to_lp<LP>(o.y * sg), to_lp<LP>(o.z * sg),
                           to_lp<LP>(o.w * sg)};
        }
        if (Gout != nullptr) {
            *reinterpret_cast<float4 *>(Gout + e) =
                make_float4(o.x - cur.x, o.y - cur.y, o.z - cur.z, o.w - cur.w);
        }
        if (want_norms) {
            const float d0 = o.x - cur.x, d1 = o.y - cur.y, d2 = o.z - cur.z, d3 = o.w - cur.w;
            dsq += d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3;
            xsq += cur.x * cur.x + cur.y * cur.y + cur.z * cur.z + cur.w * cur.w;
        }
        if (mix_part != nullptr) {
            const float4 gp = *reinterpret_cast<const float4 *>(Gprev + e);
            const float g0 = o.x - cur.x, g1 = o.y - cur.y, g2 = o.z - cur.z, g3 = o.w - cur.w;
            const float e0 = g0 - gp.x, e1 = g1 - gp.y, e2 = g2 - gp.z, e3 = g3 - gp.w;
            ma += (double)g0 * e0 + (double)g1 * e1 + (double)g2 * e2 + (double)g3 * e3;
            mb += (double)e0 * e0 + (double)e1 * e1 + (double)e2 * e2 + (double)e3 * e3;
        }
    }
    if (mix_part != nullptr) {
        const double2 t = block_sum2(ma, mb);
        // only CTAs with items own a chunk (the grid has no others when the
        // host fuses the inner products, but an idle CTA must not write)
        if (threadIdx.x == 0 && (long long)blockIdx.x * blockDim.x < (long long)total) {
            mix_part[blockIdx.x] = t;
        }
    }
    if (hist != nullptr) {
        hist_add(hist, step, block_sum2((double)dsq, (double)xsq));
    } else if (want_norms) {
        grid_finish_norms2(block_sum2((double)dsq, (double)xsq), partials, counter, norms);
    }
}

// Anderson mixing of depth one, column by column, of an n x p block
// (column-major, FP32).  The update kernel of a step writes the map's value
// f and g = f - x (x the step's iterate) into two-slot history rings; with
// theta = <g, g - g_prev> / ||g - g_prev||^2 (0 when g does not change, and
// on the first step), the next iterate is x+ = f - theta (f - f_prev),
// written with its low-precision operand copy (scaled by sig[col] when
// given).  Entries the map pins (X_jj = 1, delta_jj = 0) are pinned in f and
// f_prev alike, so they stay pinned.  The inner products come in partials per
// (column, chunk of kMixRows rows), from the update kernel itself or from
// anderson_dots_kernel; every CTA of a column adds its column's partials in
// chunk order (deterministic).  Mixing runs only when n % 4 == 0 (four rows
// per thread and item).
constexpr int kMixRows = 1024;

__global__ void __launch_bounds__(256)
anderson_dots_kernel(int n, const float *__restrict__ Gcur, const float *__restrict__ Gprev,
                     double2 *__restrict__ part)
{
    pdl_wait();  // Gcur comes from the update kernel
    pdl_trigger();
    const int col = blockIdx.x;
    const int r0 = blockIdx.y * kMixRows;
    const int r1 = min(n, r0 + kMixRows);
    const size_t off = (size_t)col * n;
    double a = 0.0, b = 0.0;
    // four consecutive rows per item (n % 4 == 0: 16-byte aligned columns)
    for (int i = r0 + 4 * (int)threadIdx.x; i < r1; i += 4 * (int)blockDim.x) {
        const float4 g = *reinterpret_cast<const float4 *>(Gcur + off + i);
        const float4 gp = *reinterpret_cast<const float4 *>(Gprev + off + i);
        const float d0 = g.x - gp.x, d1 = g.y - gp.y, d2 = g.z - gp.z, d3 = g.w - gp.w;
        a += (double)g.x * d0 + (double)g.y * d1 + (double)g.z * d2 + (double)g.w * d3;
        b += (double)d0 * d0 + (double)d1 * d1 + (double)d2 * d2 + (double)d3 * d3;
    }
    const double2 ab = block_sum2(a, b);
    if (threadIdx.x == 0) part[(size_t)col * gridDim.y + blockIdx.y] = ab;
}

template <typename LP>
__global__ void __launch_bounds__(256)
anderson_mix_kernel(int n, const float *__restrict__ F, const float *__restrict__ Fprev,
                    float *__restrict__ Xout, LP *__restrict__ Xlp, int ldx,
                    const float *__restrict__ sig, const double2 *__restrict__ part, int first)
{
    pdl_wait();  // F and the partials come from the previous grids
    pdl_trigger();
    const int col = blockIdx.x;
    const int r0 = blockIdx.y * kMixRows;
    const int r1 = min(n, r0 + kMixRows);
    const size_t off = (size_t)col * n;
    float theta = 0.0f;
    if (!first) {
        double a = 0.0, b = 0.0;
        for (int r = 0; r < (int)gridDim.y; ++r) {
            const double2 t = part[(size_t)col * gridDim.y + r];
            a += t.x;
            b += t.y;
        }
        theta = b > 0.0 && isfinite(a) && isfinite(b) ? (float)(a / b) : 0.0f;
    }
    const float sg = sig != nullptr ? sig[col] : 1.0f;
    // four consecutive rows per item (n % 4 == 0: 16-byte aligned columns)
    for (int i = r0 + 4 * (int)threadIdx.x; i < r1; i += 4 * (int)blockDim.x) {
        const float4 f = *reinterpret_cast<const float4 *>(F + off + i);
        float4 xn = f;
        // the first step reads no history (the ring holds no values yet)
        if (!first) {
            const float4 fp = *reinterpret_cast<const float4 *>(Fprev + off + i);
            xn = make_float4(fmaf(-theta, f.x - fp.x, f.x), fmaf(-theta, f.y - fp.y, f.y),
                             fmaf(-theta, f.z - fp.z, f.z), fmaf(-theta, f.w - fp.w, f.w));
        }
        *reinterpret_cast<float4 *>(Xout + off + i) = xn;
        *reinterpret_cast<LpQuad<LP> *>(Xlp + (size_t)col * ldx + i) =
            LpQuad<LP>{to_lp<LP>(xn.x * sg), to_lp<LP>(xn.y * sg), to_lp<LP>(xn.z * sg),
                       to_lp<LP>(xn.w * sg)};
    }
}

__global__ void refine_apply_kernel(double *__restrict__ X, const float *__restrict__ d,
                                    size_t count)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count) X[e] += (double)d[e];
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace {


int pick_splits(int row_blocks, int chunks, int sms)
{
    int best = 1;
    double best_eff = 0.0;
    for (int s = 1; s <= 16 && s * 4 <= chunks; ++s) {
        const int ctas = row_blocks * s;
        const int waves = (ctas + sms - 1) / sms;
        const double eff = (double)ctas / (double)(waves * sms);
        if (eff > best_eff + 0.02) {
            best_eff = eff;
            best = s;
        }
    }
    return best;
}

template <typename LP>
struct LowpTypes;
template <>
struct LowpTypes<__half> {
    static constexpr CUtensorMapDataType dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    static constexpr int kind = kLowpF16;
};
template <>
struct LowpTypes<__nv_bfloat16> {
    static constexpr CUtensorMapDataType dt = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    static constexpr int kind = kLowpBF16;
};
template <>
struct LowpTypes<tf32_t> {
    static constexpr CUtensorMapDataType dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    static constexpr int kind = kLowpTF32;
};

}  // namespace

template <typename LP>
struct LowpDense final : LowpDenseOperator {
    static constexpr int esize = (int)sizeof(LP);
    static constexpr int kchunk = 128 / esize;

    int init(const double *dH, int n_, cudaStream_t s_, LowpDenseSetup *setup = nullptr)
    {
        LowpDenseSetup none;
        LowpDenseSetup &su = setup != nullptr ? *setup : none;
        const bool symmetric = su.symmetric;
        symmetric_delta = symmetric;
        float *split_hi = symmetric ? su.split_hi : nullptr;
        float *split_lo = symmetric ? su.split_lo : nullptr;
        if (split_hi == nullptr || split_lo == nullptr) split_hi = split_lo = nullptr;
        n = n_;
        s = s_;
        sms = 148;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        ldp = ((n + 63) / 64) * 64;
        IPTGB_CHECK(delta.alloc((size_t)n * ldp, s));
        if (su.fused_src != nullptr && symmetric && n <= kFusedSetupMaxN && su.diag != nullptr &&
            su.stats != nullptr) {
            IPTGB_CHECK(inv_rows.alloc((size_t)n, s));
            auto kfn = fused_setup_kernel<LP>;
            const int vec = (n % 2 == 0) &&
                            ((reinterpret_cast<uintptr_t>(su.fused_src) & 15) == 0) &&
                            ((reinterpret_cast<uintptr_t>(split_hi) & 7) == 0) &&
                            ((reinterpret_cast<uintptr_t>(split_lo) & 7) == 0) &&
                            ((reinterpret_cast<uintptr_t>(su.fused_copy) & 15) == 0);
            if (su.upper_host != nullptr && su.fused_copy != nullptr) {
                IPTGB_CHECK(upper_pipeline(su, split_hi, split_lo));
            } else {
                kfn<<<n, 256, 0, s>>>(su.fused_src, n, ldp,
                                         LowpTypes<LP>::kind == kLowpF16 ? 1 : 0, su.fused_copy,
                                         delta.ptr, split_hi, split_lo, inv_rows.ptr, su.diag,
                                         su.stats, vec, su.oz, su.oz_rowexp, 0);
                IPTGB_LAUNCH();
            }
            scale = 1.0;  // per-row scales in inv_rows
            per_row_scales = true;
            su.fused_done = true;
            su.split_done = split_hi != nullptr;
            su.oz_done = su.oz != nullptr && su.oz_rowexp != nullptr;
            IPTGB_CHECK(make_map(&mapA, LowpTypes<LP>::dt, esize, delta.ptr, ldp, n, tc::kBM));
            IPTGB_CHECK(err.alloc(1, s));
            IPTGB_CUDA(cudaMemsetAsync(err.ptr, 0, sizeof(int), s));
            set_l2_keep(dev);
            return IPT_CUDA_SUCCESS;
        }
        double maxabs = su.maxabs;
        if (!(maxabs >= 0.0)) {
            DeviceBuffer<unsigned long long> mx;
            IPTGB_CHECK(mx.alloc(1, s));
            IPTGB_CUDA(cudaMemsetAsync(mx.ptr, 0, sizeof(unsigned long long), s));
            max_abs_offdiag_kernel<<<std::min(4 * sms, blocks_for((size_t)n * n)), kThreads, 0,
                                     s>>>(dH, n, mx.ptr);
            IPTGB_LAUNCH();
            unsigned long long bits = 0;
            IPTGB_CUDA(cudaMemcpyAsync(&bits, mx.ptr, sizeof(bits), cudaMemcpyDeviceToHost, s));
            IPTGB_CUDA(cudaStreamSynchronize(s));
            memcpy(&maxabs, &bits, sizeof(maxabs));
        }
        scale = 1.0;
        int s2 = 0;
        if (LowpTypes<LP>::kind == kLowpF16 && maxabs > 0.0 && isfinite(maxabs)) {
            // largest power of two with maxabs * scale <= 16384 (FP16 max 65504)
            s2 = (int)floor(log2(16384.0 / maxabs));
            s2 = std::min(std::max(s2, -40), 40);
            scale = ldexp(1.0, s2);
        }
        if (symmetric) {
            // vec also needs hi/lo 8-byte aligned at even offsets (pool allocations are)
            const bool vec = (n % 2 == 0) && ((reinterpret_cast<uintptr_t>(dH) & 15) == 0) &&
                             ((reinterpret_cast<uintptr_t>(split_hi) & 7) == 0) &&
                             ((reinterpret_cast<uintptr_t>(split_lo) & 7) == 0);
            dim3 grid(n, (ldp + kSymChunk - 1) / kSymChunk);
            convert_delta_sym_kernel<LP><<<grid, 256, 0, s>>>(dH, n, ldp, scale, s2, vec,
                                                              delta.ptr, split_hi, split_lo,
                                                              su.colsum_part);
            su.split_done = split_hi != nullptr;
            su.colsum_chunks = su.colsum_part != nullptr ? (int)grid.y : 0;
        } else {
            dim3 grid((ldp + 31) / 32, (n + 31) / 32);
            convert_delta_kernel<LP><<<grid, dim3(32, 8), 0, s>>>(dH, n, ldp, scale, delta.ptr,
                                                                  nullptr, nullptr);
        }
        IPTGB_LAUNCH();
        IPTGB_CHECK(make_map(&mapA, LowpTypes<LP>::dt, esize, delta.ptr, ldp, n, tc::kBM));
        set_l2_keep(dev);
        IPTGB_CHECK(err.alloc(1, s));
        IPTGB_CUDA(cudaMemsetAsync(err.ptr, 0, sizeof(int), s));
        return IPT_CUDA_SUCCESS;
    }

    // Setup from the upper triangle of H in pinned host memory: column
    // chunks in decreasing order cross the host link on stream s (a chunk's
    // columns are then complete: their lower parts are the transposes of
    // tiles of higher columns), and the setup of each chunk runs on a second
    // stream behind its transfer.  Only n (n + 1) / 2 entries cross the link.
    int upper_pipeline(LowpDenseSetup &su, float *split_hi, float *split_lo)
    {
        const int nb = (n + 31) / 32;
        const int chunk_blocks = std::max(1, std::min(nb, 16));  // 512 columns
        // the setup stream gets the highest priority: its CTAs take SM slots
        // as they free up, ahead of later work on s
        int prio_lo = 0, prio_hi = 0;
        cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
        cudaStream_t s2 = nullptr;
        IPTGB_CUDA(cudaStreamCreateWithPriority(&s2, cudaStreamNonBlocking, prio_hi));
        std::vector<cudaEvent_t> evs;
        int st = IPT_CUDA_SUCCESS;
        auto fail = [&](int code) {
            st = code;
        };
        cudaEvent_t done = nullptr;
        if (cudaEventCreateWithFlags(&done, cudaEventDisableTiming) != cudaSuccess) {
            cudaStreamDestroy(s2);
            return IPT_CUDA_CUDA_ERROR;
        }
        const int vec = (n % 2 == 0) &&
                        ((reinterpret_cast<uintptr_t>(su.fused_copy) & 15) == 0) &&
                        ((reinterpret_cast<uintptr_t>(split_hi) & 7) == 0) &&
                        ((reinterpret_cast<uintptr_t>(split_lo) & 7) == 0);
        const int pairs_ok = (n % 2 == 0) &&
                             ((reinterpret_cast<uintptr_t>(su.upper_host) & 15) == 0) &&
                             ((reinterpret_cast<uintptr_t>(su.fused_copy) & 15) == 0);
        // s2 starts after everything queued on s so far (allocations, zeroed stats)
        if (cudaEventRecord(done, s) != cudaSuccess || cudaStreamWaitEvent(s2, done, 0) != cudaSuccess) {
            fail(IPT_CUDA_CUDA_ERROR);
        }
        for (int jb1 = nb; jb1 > 0 && st == IPT_CUDA_SUCCESS; jb1 -= chunk_blocks) {
            const int jb0 = std::max(0, jb1 - chunk_blocks);
            const int c0 = jb0 * 32, c1 = std::min(n, jb1 * 32);
            upper_copy_kernel<<<std::max(1, sms), 256, 0, s>>>(su.upper_host, n, c0, c1,
                                                              su.fused_copy, pairs_ok);
            if (cudaGetLastError() != cudaSuccess) {
                fail(IPT_CUDA_CUDA_ERROR);
                break;
            }
            count_launch();
            cudaEvent_t ev = nullptr;
            if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
                fail(IPT_CUDA_CUDA_ERROR);
                break;
            }
            evs.push_back(ev);
            if (cudaEventRecord(ev, s) != cudaSuccess || cudaStreamWaitEvent(s2, ev, 0) != cudaSuccess) {
                fail(IPT_CUDA_CUDA_ERROR);
                break;
            }
            trace_mark(jb1 == nb ? "upper:first_chunk_moved" : (jb0 == 0 ? "upper:last_chunk_moved" : "upper:chunk_moved"), s);
            mirror_lower_kernel<<<2 * std::max(1, sms), 256, 0, s2>>>(su.fused_copy, n, jb0, jb1);
            if (cudaGetLastError() != cudaSuccess) {
                fail(IPT_CUDA_CUDA_ERROR);
                break;
            }
            count_launch();
            fused_setup_kernel<LP><<<c1 - c0, 256, 0, s2>>>(
                su.fused_copy, n, ldp, LowpTypes<LP>::kind == kLowpF16 ? 1 : 0, nullptr, delta.ptr,
                split_hi, split_lo, inv_rows.ptr, su.diag, su.stats, vec, su.oz, su.oz_rowexp, c0);
            if (cudaGetLastError() != cudaSuccess) {
                fail(IPT_CUDA_CUDA_ERROR);
                break;
            }
            count_launch();
        }
        trace_mark("upper:setups_done", s2);
        // s continues after the last setup
        if (cudaEventRecord(done, s2) != cudaSuccess || cudaStreamWaitEvent(s, done, 0) != cudaSuccess) {
            fail(IPT_CUDA_CUDA_ERROR);
        }
        for (cudaEvent_t ev : evs) cudaEventDestroy(ev);
        cudaEventDestroy(done);
        cudaStreamDestroy(s2);
        return st;
    }

    // Delta is streamed once per product; when it is larger than about
    // half of L2, that share of it is marked evict_last so that it stays
    // resident across the products (the rest evict_first).  Measured at
    // n = 8192 (FP16 Delta 134 MB): keeping 40-55% of Delta gives the
    // fastest solve; more than 60% thrashes again.
    void set_l2_keep(int dev)
    {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
        const double bytes = (double)n * (double)ldp * esize;
        const double keep_bytes = 0.45 * (double)l2;
        a_keep = bytes > keep_bytes && l2 > 0 ? (float)(keep_bytes / bytes) : 0.0f;
        // tuning knob: IPT_GB300_L2_KEEP_PCT overrides the fraction (0 = no hint)
        const int pct = env_int("IPT_GB300_L2_KEEP_PCT", -1);
        if (pct >= 0) a_keep = std::min(pct, 100) / 100.0f;
    }

    int set_width(int p_) override
    {
        p = p_;
        p_pad = ((p + 15) / 16) * 16;
        if (p_pad > 256) {
            return IPT_CUDA_INVALID_ARGUMENT;
        }
        tmem_cols = 32;
        while (tmem_cols < p_pad) tmem_cols <<= 1;
        const int row_blocks = (n + tc::kBM - 1) / tc::kBM;
        chunks_total = ldp / kchunk;
        const size_t stage_bytes0 = (size_t)(tc::kBM + p_pad) * tc::kRowBytes;
        // Two CTAs per SM with a 4-stage pipeline when it fits in shared
        // memory (measured faster than one 8-stage CTA per SM), and enough
        // K splits to fill one wave of CTA slots.
        const bool two_per_sm = 4 * stage_bytes0 + 2048 <= 113u * 1024u;
        const int slots = sms * (two_per_sm ? 2 : 1);
        splits = std::max(1, std::min(slots / std::max(1, row_blocks), chunks_total / 4));
        if (splits < 1) splits = pick_splits(row_blocks, chunks_total, sms);
        // tuning knob: IPT_GB300_TC_SPLITS overrides the split-K factor
        const int forced = env_int("IPT_GB300_TC_SPLITS", 0);
        if (forced > 0) {
            splits = std::min(forced, chunks_total);
        }
        const int forced_stages = env_int("IPT_GB300_TC_STAGES", 0);
        const int afmt = LowpTypes<LP>::kind == kLowpF16 ? 0 : (LowpTypes<LP>::kind == kLowpBF16 ? 1 : 2);
        idesc = (1u << 4) | ((uint32_t)afmt << 7) | ((uint32_t)afmt << 10) |
                ((uint32_t)(p_pad >> 3) << 17) | ((uint32_t)(tc::kBM >> 4) << 24);
        // persistent stream-K schedule with two CTAs per SM (tuning knob
        // IPT_GB300_TC_STREAMK: 1 = one CTA per SM with a deeper ring, 0 =
        // the split-K grid below).  Measured per product (FP16, k = 32):
        // n = 8192 22.1 us (one CTA per SM 28.0, split-K 23.3); n = 16384
        // 91-93 us for all three, 0.85-0.87 of the measured HBM bandwidth.
        // symmetric form (FP16 / BF16, p_pad <= 64): half of Delta's bytes,
        // twice the MMAs per byte.  Off by default: measured at n = 8192,
        // k = 32 it took 27 us per product against 21 us for stream-K (one
        // super-tile per SM leaves the MMA issue, the TMA ring and the
        // epilogue in series) and its 17 partial slots per row slow the
        // update.  Tuning knob IPT_GB300_TC_SYM: 1 = from n = 6144, 2 = always.
        const int sym_knob = env_int("IPT_GB300_TC_SYM", 0);
        sym = false;
        if (LowpTypes<LP>::kind != kLowpTF32 && p_pad <= 64 && symmetric_delta &&
            (sym_knob >= 2 || (sym_knob == 1 && n >= 6144))) {
            return set_width_sym(row_blocks);
        }
        const int sk = env_int("IPT_GB300_TC_STREAMK", 2);
        streamk = sk > 0;
        if (streamk) return set_width_streamk(row_blocks, forced_stages, std::min(sk, 2));
        chunks_per_split = (chunks_total + splits - 1) / splits;
        splits = (chunks_total + chunks_per_split - 1) / chunks_per_split;
        const size_t stage_bytes = (size_t)(tc::kBM + p_pad) * tc::kRowBytes;
        stages = (int)std::min<size_t>(8, (200u * 1024u) / stage_bytes);
        if (two_per_sm) {
            stages = 4;
        }
        if (forced_stages >= 2) {
            stages = std::min(stages, forced_stages);
        }
        if (stages < 2) return IPT_CUDA_INVALID_ARGUMENT;
        smem_bytes = 1024 + stages * stage_bytes + (2 * stages + 1) * 8 + 16;
        IPTGB_CHECK(P.alloc((size_t)splits * p * n, s));
        IPTGB_CHECK(alloc_blocks());
        auto kfn = tc::tc_partial_kernel<LowpTypes<LP>::kind>;
        IPTGB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem_bytes));
        cur = 0;
        return IPT_CUDA_SUCCESS;
    }

    // Symmetric product: super-tiles of 4 x 4 upper tiles, one per CTA at a
    // time; nS + 1 partial slots per row block, every one written each
    // product.  Delta's upper half is marked evict_last when it fits in L2.
    int set_width_sym(int row_blocks)
    {
        sprm_sym = tc::SymParams{};
        sprm_sym.n = n;
        sprm_sym.p = p;
        sprm_sym.p_pad = p_pad;
        sprm_sym.nb = row_blocks;
        sprm_sym.nS = (row_blocks + tc::kSymG - 1) / tc::kSymG;
        sprm_sym.items = sprm_sym.nS * (sprm_sym.nS + 1) / 2;
        sprm_sym.idesc = idesc;
        const size_t bbytes = (size_t)2 * tc::kSymG * 2 * p_pad * tc::kRowBytes;
        const size_t budget = 220u * 1024u;
        if (bbytes + 2 * tc::kSymTileBytes > budget) return IPT_CUDA_INVALID_ARGUMENT;
        stages = (int)std::min<size_t>(6, (budget - bbytes) / tc::kSymTileBytes);
        sprm_sym.stages = stages;
        smem_bytes = 1024 + (size_t)stages * tc::kSymTileBytes + bbytes + (2 * stages + 5) * 8 + 16;
        grid_g = std::min(sprm_sym.items, sms);
        splits = sprm_sym.nS + 1;
        IPTGB_CHECK(P.alloc((size_t)splits * p * n, s));
        IPTGB_CHECK(alloc_blocks());
        auto kfn = tc::tc_sym_kernel<LowpTypes<LP>::kind>;
        IPTGB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem_bytes));
        // the upper half of Delta: all of it evict_last when it fits in 70 %
        // of L2, else the share that does
        int dev = 0, l2 = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
        const double half = 0.5 * (double)n * (double)ldp * esize;
        a_keep_sym = l2 > 0 ? (float)std::min(1.0, 0.7 * l2 / half) : 0.0f;
        const int pct = env_int("IPT_GB300_L2_KEEP_PCT", -1);
        if (pct >= 0) a_keep_sym = std::min(pct, 100) / 100.0f;
        if (per_row_scales) {
            // the fused setup scaled each row on its own: one common scale
            DeviceBuffer<float> gmax;
            IPTGB_CHECK(gmax.alloc(1, s));
            max_inv_row_kernel<<<1, 256, 0, s>>>(inv_rows.ptr, n, gmax.ptr);
            IPTGB_LAUNCH();
            common_row_scale_kernel<LP><<<n, 256, 0, s>>>(delta.ptr, ldp, inv_rows.ptr, gmax.ptr);
            IPTGB_LAUNCH();
            per_row_scales = false;
        }
        sym = true;
        streamk = false;
        cur = 0;
        return IPT_CUDA_SUCCESS;
    }

    // One CTA per SM, each walking an equal contiguous share of the (tile,
    // K chunk) items with a TMA ring as deep as shared memory allows; the
    // partial slots of a tile are the CTAs its items span (at most
    // `splits`), the unused ones zeroed here once.
    int set_width_streamk(int row_blocks, int forced_stages, int per_sm)
    {
        const size_t stage_bytes = (size_t)(tc::kBM + p_pad) * tc::kRowBytes;
        stages = (int)std::min<size_t>(12, (per_sm == 2 ? 108u : 216u) * 1024u / stage_bytes);
        if (forced_stages >= 2) stages = std::min(stages, forced_stages);
        if (stages < 2) return IPT_CUDA_INVALID_ARGUMENT;
        sprm = tc::StreamParams{};
        sprm.n = n;
        sprm.p = p;
        sprm.p_pad = p_pad;
        sprm.stages = stages;
        sprm.acc_cols = tmem_cols;
        sprm.acc_bufs = 2 * tmem_cols <= 512 ? 2 : 1;
        sprm.tmem_cols = sprm.acc_bufs * tmem_cols;
        sprm.chunks = chunks_total;
        sprm.kchunk = (int)kchunk;
        sprm.items = (long long)row_blocks * chunks_total;
        sprm.idesc = idesc;
        grid_g = (int)std::min<long long>((long long)sms * per_sm, sprm.items);
        // tuning knob IPT_GB300_TC_ALTERNATE=0: every product walks forwards
        alternate = env_int("IPT_GB300_TC_ALTERNATE", 1) != 0;
        products = 0;
        splits = 1;
        for (int t = 0; t < row_blocks; ++t) {
            const long long f = tc::owner_of((long long)t * chunks_total, sprm.items, grid_g);
            const long long l =
                tc::owner_of((long long)t * chunks_total + chunks_total - 1, sprm.items, grid_g);
            splits = std::max(splits, (int)(l - f + 1));
        }
        smem_bytes = 1024 + stages * stage_bytes + (2 * stages + 5) * 8 + 16;
        IPTGB_CHECK(P.alloc((size_t)splits * p * n, s));
        IPTGB_CUDA(cudaMemsetAsync(P.ptr, 0, (size_t)splits * p * n * sizeof(float), s));
        IPTGB_CHECK(alloc_blocks());
        auto kfn = tc::tc_stream_kernel<LowpTypes<LP>::kind>;
        IPTGB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem_bytes));
        cur = 0;
        return IPT_CUDA_SUCCESS;
    }

    int alloc_blocks()
    {
        for (int b = 0; b < 2; ++b) {
            IPTGB_CHECK(Xlp[b].alloc((size_t)ldp * p_pad, s));
            IPTGB_CUDA(cudaMemsetAsync(Xlp[b].ptr, 0, (size_t)ldp * p_pad * sizeof(LP), s));
            IPTGB_CHECK(make_map(&mapB[b], LowpTypes<LP>::dt, esize, Xlp[b].ptr, ldp, p_pad, p_pad));
            IPTGB_CHECK(X32[b].alloc((size_t)n * p, s));
        }
        IPTGB_CHECK(G.alloc((size_t)n * p, s));
        return IPT_CUDA_SUCCESS;
    }

    int reset_identity(const double *d) override
    {
        build_g32_kernel<<<blocks_for((size_t)n * p), kThreads, 0, s>>>(d, n, p, G.ptr);
        IPTGB_LAUNCH();
        lowp_identity_kernel<LP><<<blocks_for((size_t)n * p), kThreads, 0, s>>>(
            X32[0].ptr, Xlp[0].ptr, n, p, ldp);
        IPTGB_LAUNCH();
        cur = 0;
        mix_first = true;
        kf = 0;
        return IPT_CUDA_SUCCESS;
    }

    int product() override { return product_until(nullptr, 0, 0.0); }

    // update grid: grid-stride over the block with a few CTAs per SM (four
    // rows per thread when n % 4 == 0); tuning knob IPT_GB300_UPDATE_CTAS_PER_SM
    int update_grid() const
    {
        const size_t items = n % 4 == 0 ? (size_t)n * p / 4 : (size_t)n * p;
        const int per_sm = env_int("IPT_GB300_UPDATE_CTAS_PER_SM", 4);
        const int all = blocks_for(items);
        return per_sm > 0 ? std::min(all, per_sm * sms) : all;
    }

    // hist/step/tol: the device-side stop of the running iteration (or null)
    int product_until(const double *hist, int step, double tol)
    {
        KernelTimerScope timer(kProfLowpProduct, s);
        if (sym) {
            return launch_pdl(tc::tc_sym_kernel<LowpTypes<LP>::kind>, dim3(grid_g),
                              dim3(tc::kStreamThreads), smem_bytes, s, mapA, mapB[cur], sprm_sym,
                              P.ptr, err.ptr, a_keep_sym, hist, step, tol, spin);
        }
        if (streamk) {
            const int reverse = alternate ? (int)(products++ & 1) : 0;
            return launch_pdl(tc::tc_stream_kernel<LowpTypes<LP>::kind>, dim3(grid_g),
                              dim3(tc::kStreamThreads), smem_bytes, s, mapA, mapB[cur], sprm,
                              P.ptr, err.ptr, a_keep, hist, step, tol, spin, reverse);
        }
        const int row_blocks = (n + tc::kBM - 1) / tc::kBM;
        dim3 grid(row_blocks, splits);
        return launch_pdl(tc::tc_partial_kernel<LowpTypes<LP>::kind>, grid, dim3(tc::kThreads),
                          smem_bytes, s, mapA, mapB[cur], n, p, p_pad, stages, tmem_cols,
                          chunks_total, chunks_per_split, (int)kchunk, idesc, P.ptr, err.ptr,
                          a_keep, hist, step, tol, spin);
    }

    int step(int want_norms, NormScratch *ns) override
    {
        const bool hm = ns->hist != nullptr && ns->step < ns->hist_cap;
        double *hist = hm ? ns->hist : nullptr;
        const int hstep = ns->step;
        IPTGB_CHECK(product_until(hist, hstep, ns->stop_tol));
        const int grid = update_grid();
        if (want_norms && grid > ns->capacity) return IPT_CUDA_INVALID_ARGUMENT;
        const int nxt = cur ^ 1;
        const bool mixed = mixing && hist == nullptr && n % 4 == 0;
        const bool fused = mixed && fused_dots(grid);
        if (mixed) IPTGB_CHECK(mix_buffers());
        {
            KernelTimerScope timer(kProfLowpUpdate, s);
            if (n % 4 == 0) {
                IPTGB_CHECK(launch_pdl(lowp_update4_kernel<LP>, dim3(grid), dim3(kThreads), 0, s,
                                       (const float *)P.ptr, splits, n, p, (float)(1.0 / scale),
                                       (const float *)inv_rows.ptr, (const float *)G.ptr,
                                       (const float *)X32[cur].ptr,
                                       mixed ? Fring[kf].ptr : X32[nxt].ptr,
                                       mixed ? (LP *)nullptr : Xlp[nxt].ptr, ldp, want_norms,
                                       ns->partials, ns->counter, ns->norms, hist, hstep,
                                       ns->stop_tol, (const float *)Gring[kf ^ 1].ptr,
                                       mixed ? Gring[kf].ptr : nullptr,
                                       fused ? mix_part.ptr : nullptr));
            } else {
                IPTGB_CHECK(launch_pdl(lowp_update_kernel<LP>, dim3(grid), dim3(kThreads), 0, s,
                                       (const float *)P.ptr, splits, n, p, (float)(1.0 / scale),
                                       (const float *)inv_rows.ptr, (const float *)G.ptr,
                                       (const float *)X32[cur].ptr, X32[nxt].ptr, Xlp[nxt].ptr,
                                       ldp, want_norms, ns->partials, ns->counter, ns->norms,
                                       hist, hstep, ns->stop_tol));
            }
        }
        if (mixed) IPTGB_CHECK(mix(nxt, nullptr, fused));
        if (hm) ++ns->step;
        cur = nxt;
        return IPT_CUDA_SUCCESS;
    }

    // The update kernel forms the mixing's partial inner products itself when
    // each of its threads takes one four-row item and every CTA one 1024-row
    // chunk of a column (n % 1024 == 0), after the first mixed step.
    bool fused_dots(int grid) const
    {
        return !mix_first && n % kMixRows == 0 &&
               (size_t)grid * kThreads >= (size_t)n * p / 4 && kThreads * 4 == kMixRows;
    }

    int mix_buffers()
    {
        const size_t elems = (size_t)n * p;
        const int chunks = (n + kMixRows - 1) / kMixRows;
        for (int r = 0; r < 2; ++r) {
            if (Fring[r].count < elems) {
                IPTGB_CHECK(Fring[r].alloc(elems, s));
                IPTGB_CHECK(Gring[r].alloc(elems, s));
            }
        }
        if (mix_part.count < (size_t)p * chunks) IPTGB_CHECK(mix_part.alloc((size_t)p * chunks, s));
        return IPT_CUDA_SUCCESS;
    }

    // Anderson mixing of this step's map value (in X32[nxt]) with the last
    // one's (lowp.h set_mixing); `fused`: the update kernel formed the
    // partial inner products
    int mix(int nxt, const float *sig, bool fused)
    {
        const int chunks = (n + kMixRows - 1) / kMixRows;
        KernelTimerScope timer(kProfLowpUpdate, s);
        const dim3 grid(p, chunks);
        if (!mix_first && !fused) {
            IPTGB_CHECK(launch_pdl(anderson_dots_kernel, grid, dim3(256), 0, s, n,
                                   (const float *)Gring[kf].ptr, (const float *)Gring[kf ^ 1].ptr,
                                   mix_part.ptr));
        }
        IPTGB_CHECK(launch_pdl(anderson_mix_kernel<LP>, grid, dim3(256), 0, s, n,
                               (const float *)Fring[kf].ptr, (const float *)Fring[kf ^ 1].ptr,
                               X32[nxt].ptr, Xlp[nxt].ptr, ldp, sig,
                               (const double2 *)mix_part.ptr, mix_first ? 1 : 0));
        mix_first = false;
        kf ^= 1;
        return IPT_CUDA_SUCCESS;
    }
    void set_mixing(bool on) override { mixing = on; }

    int read_error(int *host_err) override
    {
        IPTGB_CUDA(cudaMemcpyAsync(host_err, err.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
        return IPT_CUDA_SUCCESS;
    }

    int export_fp64(double *X) override
    {
        f32_to_f64_kernel<<<blocks_for((size_t)n * p), kThreads, 0, s>>>(X32[cur].ptr,
                                                                         (size_t)n * p, X);
        IPTGB_LAUNCH();
        return IPT_CUDA_SUCCESS;
    }

    int export_fp64_prev(double *X) override
    {
        f32_to_f64_kernel<<<blocks_for((size_t)n * p), kThreads, 0, s>>>(X32[cur ^ 1].ptr,
                                                                         (size_t)n * p, X);
        IPTGB_LAUNCH();
        return IPT_CUDA_SUCCESS;
    }

    const float *partials() const override { return P.ptr; }
    int num_splits() const override { return splits; }
    double streamed_bytes() const override { return (double)n * (double)ldp * esize; }

    int refine_begin(const double *R0, const double *X, const double *c,
                     const float *sigma) override
    {
        const size_t elems = (size_t)n * p;
        if (R32.count < elems) {
            IPTGB_CHECK(R32.alloc(elems, s));
            IPTGB_CHECK(Xref32.alloc(elems, s));
            IPTGB_CHECK(small.alloc(4 * (size_t)p, s));
        }
        refine_begin_kernel<LP><<<blocks_for(elems), kThreads, 0, s>>>(
            R0, X, c, sigma, 1, n, p, ldp, X32[0].ptr, Xlp[0].ptr, R32.ptr, Xref32.ptr,
            small.ptr, small.ptr + p, small.ptr + 2 * p);
        IPTGB_LAUNCH();
        cur = 0;
        mix_first = true;
        kf = 0;
        return IPT_CUDA_SUCCESS;
    }

    int refine_step(int want_norms, NormScratch *ns) override
    {
        const bool hm = ns->hist != nullptr && ns->step < ns->hist_cap;
        double *hist = hm ? ns->hist : nullptr;
        const int hstep = ns->step;
        IPTGB_CHECK(product_until(hist, hstep, ns->stop_tol));
        const int grid = update_grid();
        if (want_norms && grid > ns->capacity) return IPT_CUDA_INVALID_ARGUMENT;
        const int nxt = cur ^ 1;
        const bool mixed = mixing && hist == nullptr && n % 4 == 0;
        const bool fused = mixed && fused_dots(grid);
        if (mixed) IPTGB_CHECK(mix_buffers());
        {
            KernelTimerScope timer(kProfLowpUpdate, s);
            if (n % 4 == 0) {
                IPTGB_CHECK(launch_pdl(refine_update4_kernel<LP>, dim3(grid), dim3(kThreads), 0, s,
                                       (const float *)P.ptr, splits, n, p, (float)(1.0 / scale),
                                       (const float *)inv_rows.ptr,
                                       (const float *)(small.ptr + p),
                                       (const float *)(small.ptr + 2 * p), (const float *)G.ptr,
                                       (const float *)R32.ptr, (const float *)Xref32.ptr,
                                       (const float *)small.ptr, (const float *)X32[cur].ptr,
                                       mixed ? Fring[kf].ptr : X32[nxt].ptr,
                                       mixed ? (LP *)nullptr : Xlp[nxt].ptr, ldp, want_norms,
                                       ns->partials, ns->counter, ns->norms, hist, hstep,
                                       ns->stop_tol, (const float *)Gring[kf ^ 1].ptr,
                                       mixed ? Gring[kf].ptr : nullptr,
                                       fused ? mix_part.ptr : nullptr));
            } else {
                IPTGB_CHECK(launch_pdl(refine_update_kernel<LP>, dim3(grid), dim3(kThreads), 0, s,
                                       (const float *)P.ptr, splits, n, p, (float)(1.0 / scale),
                                       (const float *)inv_rows.ptr,
                                       (const float *)(small.ptr + p),
                                       (const float *)(small.ptr + 2 * p), (const float *)G.ptr,
                                       (const float *)R32.ptr, (const float *)Xref32.ptr,
                                       (const float *)small.ptr, (const float *)X32[cur].ptr,
                                       X32[nxt].ptr, Xlp[nxt].ptr, ldp, want_norms, ns->partials,
                                       ns->counter, ns->norms, hist, hstep, ns->stop_tol));
            }
        }
        if (mixed) IPTGB_CHECK(mix(nxt, small.ptr + p, fused));
        if (hm) ++ns->step;
        cur = nxt;
        return IPT_CUDA_SUCCESS;
    }

    int refine_apply(double *X) override
    {
        refine_apply_kernel<<<blocks_for((size_t)n * p), kThreads, 0, s>>>(X, X32[cur].ptr,
                                                                          (size_t)n * p);
        IPTGB_LAUNCH();
        return IPT_CUDA_SUCCESS;
    }

    DeviceBuffer<float> R32, Xref32, small;  // small: c32 | sigma | 1/sigma
    DeviceBuffer<float> Fring[2], Gring[2];  // Anderson mixing history (f, g)
    DeviceBuffer<double2> mix_part;          // its partial inner products
    bool mixing = false, mix_first = true;
    int kf = 0;                              // ring slot of this step

    int sms = 148;
    int n = 0;
    int ldp = 0, p = 0, p_pad = 0, tmem_cols = 32, chunks_total = 0, chunks_per_split = 0;
    int splits = 1, stages = 2, cur = 0;
    size_t smem_bytes = 0;
    uint32_t idesc = 0;
    bool sym = false;
    bool symmetric_delta = false;  // H symmetric: Delta == Delta^T up to row scales
    bool per_row_scales = false;   // rows of the stored Delta carry their own scales
    tc::SymParams sprm_sym{};
    float a_keep_sym = 0.0f;
    bool streamk = false;
    bool alternate = true;  // every other product walks its items backwards
    long long products = 0;
    int grid_g = 0;
    tc::StreamParams sprm{};
    double scale = 1.0;
    float a_keep = 0.0f;  // fraction of Delta kept in L2 (evict_last) across products
    // polls of a pipeline wait before the kernel gives up (tuning and test
    // knob IPT_GB300_SPIN_LIMIT; the drain before TMEM is released always
    // uses the full bound)
    long long spin = env_int("IPT_GB300_SPIN_LIMIT", 0) > 0 ? env_int("IPT_GB300_SPIN_LIMIT", 0)
                                                             : tc::kSpinLimit;
    // per-row 1/scale of Delta (row i scaled by its own power of two) when the
    // fused setup pass built Delta; empty: one scale for the whole matrix
    DeviceBuffer<float> inv_rows;
    cudaStream_t s = nullptr;
    DeviceBuffer<LP> delta;
    DeviceBuffer<LP> Xlp[2];
    DeviceBuffer<float> X32[2];
    DeviceBuffer<float> G, P;
    DeviceBuffer<int> err;
    CUtensorMap mapA, mapB[2];
};

// FP32 SIMT operator (no tensor cores): Delta kept column-major in FP32 and
// multiplied with the FP32 split-K kernel; the update shares the kernel
// above with exact FP32 operand copies.
__global__ void convert_delta_f32_colmajor_kernel(const double *__restrict__ H, int n,
                                                  float *__restrict__ out)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n * n) return;
    const size_t i = e % (size_t)n;
    const size_t l = e / (size_t)n;
    out[e] = i == l ? 0.0f : (float)H[e];
}

struct LowpDenseSimtF32 final : LowpDenseOperator {
    int init(const double *dH, int n_, cudaStream_t s_)
    {
        n = n_;
        s = s_;
        sms = 148;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        IPTGB_CHECK(delta.alloc((size_t)n * n, s));
        convert_delta_f32_colmajor_kernel<<<blocks_for((size_t)n * n), kThreads, 0, s>>>(dH, n,
                                                                                      delta.ptr);
        IPTGB_LAUNCH();
        IPTGB_CHECK(err.alloc(1, s));
        IPTGB_CUDA(cudaMemsetAsync(err.ptr, 0, sizeof(int), s));
        return IPT_CUDA_SUCCESS;
    }
    int set_width(int p_) override
    {
        p = p_;
        splits = dense64_split_for(n, p, sms);
        IPTGB_CHECK(P.alloc((size_t)splits * p * n, s));
        for (int b = 0; b < 2; ++b) {
            IPTGB_CHECK(X32[b].alloc((size_t)n * p, s));
        }
        IPTGB_CHECK(G.alloc((size_t)n * p, s));
        cur = 0;
        return IPT_CUDA_SUCCESS;
    }
    int reset_identity(const double *d) override
    {
        build_g32_kernel<<<blocks_for((size_t)n * p), kThreads, 0, s>>>(d, n, p, G.ptr);
        IPTGB_LAUNCH();
        lowp_identity_kernel<float><<<blocks_for((size_t)n * p), kThreads, 0, s>>>(
            X32[0].ptr, X32[0].ptr, n, p, n);
        IPTGB_LAUNCH();
        cur = 0;
        return IPT_CUDA_SUCCESS;
    }
    int product() override
    {
        KernelTimerScope timer(kProfLowpProduct, s);
        return launch_dense32_partial(delta.ptr, n, n, X32[cur].ptr, n, p, P.ptr, splits, s);
    }
    int step(int want_norms, NormScratch *ns) override
    {
        const bool hm = ns->hist != nullptr && ns->step < ns->hist_cap;
        IPTGB_CHECK(product());
        const size_t elems = (size_t)n * p;
        const int grid = blocks_for(elems);
        if (want_norms && grid > ns->capacity) return IPT_CUDA_INVALID_ARGUMENT;
        const int nxt = cur ^ 1;
        KernelTimerScope timer(kProfLowpUpdate, s);
        lowp_update_kernel<float><<<grid, kThreads, 0, s>>>(
            P.ptr, splits, n, p, 1.0f, nullptr, G.ptr, X32[cur].ptr, X32[nxt].ptr, X32[nxt].ptr, n,
            want_norms, ns->partials, ns->counter, ns->norms, hm ? ns->hist : nullptr, ns->step,
            ns->stop_tol);
        IPTGB_LAUNCH();
        if (hm) ++ns->step;
        cur = nxt;
        return IPT_CUDA_SUCCESS;
    }
    int read_error(int *host_err) override
    {
        IPTGB_CUDA(cudaMemcpyAsync(host_err, err.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
        return IPT_CUDA_SUCCESS;
    }
    int export_fp64(double *X) override
    {
        f32_to_f64_kernel<<<blocks_for((size_t)n * p), kThreads, 0, s>>>(X32[cur].ptr,
                                                                         (size_t)n * p, X);
        IPTGB_LAUNCH();
        return IPT_CUDA_SUCCESS;
    }
    int export_fp64_prev(double *X) override
    {
        f32_to_f64_kernel<<<blocks_for((size_t)n * p), kThreads, 0, s>>>(X32[cur ^ 1].ptr,
                                                                         (size_t)n * p, X);
        IPTGB_LAUNCH();
        return IPT_CUDA_SUCCESS;
    }
    const float *partials() const override { return P.ptr; }
    int num_splits() const override { return splits; }

    int refine_begin(const double *R0, const double *X, const double *c,
                     const float *sigma) override
    {
        const size_t elems = (size_t)n * p;
        if (R32.count < elems) {
            IPTGB_CHECK(R32.alloc(elems, s));
            IPTGB_CHECK(Xref32.alloc(elems, s));
            IPTGB_CHECK(small.alloc(4 * (size_t)p, s));
        }
        // FP32 operands need no column scaling
        refine_begin_kernel<float><<<blocks_for(elems), kThreads, 0, s>>>(
            R0, X, c, sigma, 0, n, p, n, X32[0].ptr, X32[0].ptr, R32.ptr, Xref32.ptr, small.ptr,
            small.ptr + p, small.ptr + 2 * p);
        IPTGB_LAUNCH();
        cur = 0;
        return IPT_CUDA_SUCCESS;
    }

    int refine_step(int want_norms, NormScratch *ns) override
    {
        const bool hm = ns->hist != nullptr && ns->step < ns->hist_cap;
        IPTGB_CHECK(product());
        const size_t elems = (size_t)n * p;
        const int grid = blocks_for(elems);
        if (want_norms && grid > ns->capacity) return IPT_CUDA_INVALID_ARGUMENT;
        const int nxt = cur ^ 1;
        KernelTimerScope timer(kProfLowpUpdate, s);
        refine_update_kernel<float><<<grid, kThreads, 0, s>>>(
            P.ptr, splits, n, p, 1.0f, nullptr, small.ptr + p, small.ptr + 2 * p, G.ptr, R32.ptr,
            Xref32.ptr, small.ptr, X32[cur].ptr, X32[nxt].ptr, X32[nxt].ptr, n, want_norms,
            ns->partials, ns->counter, ns->norms, hm ? ns->hist : nullptr, ns->step,
            ns->stop_tol);
        IPTGB_LAUNCH();
        if (hm) ++ns->step;
        cur = nxt;
        return IPT_CUDA_SUCCESS;
    }

    int refine_apply(double *X) override
    {
        refine_apply_kernel<<<blocks_for((size_t)n * p), kThreads, 0, s>>>(X, X32[cur].ptr,
                                                                          (size_t)n * p);
        IPTGB_LAUNCH();
        return IPT_CUDA_SUCCESS;
    }

    DeviceBuffer<float> R32, Xref32, small;

    int n = 0, p = 0, sms = 148, splits = 1, cur = 0;
    cudaStream_t s = nullptr;
    DeviceBuffer<float> delta, G, P;
    DeviceBuffer<float> X32[2];
    DeviceBuffer<int> err;
};

LowpDenseOperator *make_lowp_dense_operator(const double *dH, int n, int kind, cudaStream_t s,
                                            int *status, LowpDenseSetup *setup)
{
    if (setup != nullptr) {
        setup->split_done = false;
        setup->colsum_chunks = 0;
    }
    int dev = 0, major = 0, minor = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (kind != kLowpF32 && (major != 10 || encode_fn() == nullptr)) {
        fprintf(stderr, "ipt_gb300: tensor-core IPT stage needs an sm_103 (GB300) device\n");
        *status = IPT_CUDA_CUDA_ERROR;
        return nullptr;
    }
    std::unique_ptr<LowpDenseOperator> op;
    int st = IPT_CUDA_INVALID_ARGUMENT;
    if (kind == kLowpF16) {
        auto *o = new LowpDense<__half>();
        op.reset(o);
        st = o->init(dH, n, s, setup);
    } else if (kind == kLowpBF16) {
        auto *o = new LowpDense<__nv_bfloat16>();
        op.reset(o);
        st = o->init(dH, n, s, setup);
    } else if (kind == kLowpTF32) {
        auto *o = new LowpDense<tf32_t>();
        op.reset(o);
        st = o->init(dH, n, s, setup);
    } else if (kind == kLowpF32) {
        auto *o = new LowpDenseSimtF32();
        op.reset(o);
        st = o->init(dH, n, s);
    }
    *status = st;
    if (st != IPT_CUDA_SUCCESS) {
        return nullptr;
    }
    return op.release();
}

// ---------------------------------------------------------------------------
// The IPT stage of the block solver on the low-precision operator.
// ---------------------------------------------------------------------------
struct LowpStage final : IptStage {
    std::unique_ptr<LowpDenseOperator> owned;
    LowpDenseOperator *op = nullptr;
    const double *d = nullptr;
    int n = 0;
    cudaStream_t s = nullptr;
    int run(int p, int maxiter, double tol, int check_every, double *X, int *iterations,
            double *fpres_out, long long *matvecs) override
    {
        IPTGB_CHECK(op->set_width(p));
        IPTGB_CHECK(op->reset_identity(d));
        trace_mark("ipt:start", s);
        return run_lowp_ipt(*op, n, p, maxiter, tol, check_every, X, iterations, fpres_out,
                            matvecs, s, true);
    }
};

IptStage *make_lowp_dense_stage(const double *dH, int n, const double *d, int precision,
                                cudaStream_t stream, int *status)
{
    const int kind = precision == IPT_BLOCK_FP16 ? kLowpF16
                     : precision == IPT_BLOCK_BF16 ? kLowpBF16
                                                   : kLowpTF32;
    LowpDenseOperator *op = make_lowp_dense_operator(dH, n, kind, stream, status);
    if (op == nullptr) {
        return nullptr;
    }
    auto *st = new LowpStage();
    st->owned.reset(op);
    st->op = op;
    st->d = d;
    st->n = n;
    st->s = stream;
    return st;
}

IptStage *make_lowp_stage_on(LowpDenseOperator *op, const double *d, int n, cudaStream_t stream)
{
    auto *st = new LowpStage();
    st->op = op;
    st->d = d;
    st->n = n;
    st->s = stream;
    return st;
}

bool lowp_device_stop(const LowpDenseOperator &op)
{
    const int ds = env_int("IPT_GB300_DEVICE_STOP", -1);
    if (ds >= 0) return ds != 0;
    int dev = 0, l2 = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
    // measured at n = 8192 FP16 (Delta 1.07 x L2): break-even, so off there
    return l2 > 0 && op.streamed_bytes() > 2.0 * (double)l2;
}

// Shared IPT loop on a low-precision operator: reads the fixed-point residual
// every `check_every` iterations; with `guard`, stops once the residual stops
// decreasing and rolls back a non-finite step.  The final block is exported
// to X (FP64, n x p).
int run_lowp_ipt(LowpDenseOperator &op, int n, int p, int maxiter, double tol, int check_every,
                 double *X, int *iterations, double *fpres_out, long long *matvecs,
                 cudaStream_t s, bool guard)
{
    SolveScratch scratch;
    IPTGB_CHECK(scratch.init((size_t)n * p, s));
    // every step adds its norms to the device history; the step after the
    // one that meets tol passes the block through, so the host reads the
    // history only every check_every steps
    const bool device_stop = lowp_device_stop(op);
    if (device_stop) IPTGB_CHECK(scratch.arm_history(std::max(1, maxiter), tol, s));
    int launched = 0, done = 0;
    double fpres = NAN;
    double best = INFINITY;
    int worse = 0;
    int status = IPT_CUDA_SUCCESS;
    bool rollback = false;
    int host_err = 0;
    for (int it = 0; it < maxiter; ++it) {
        const int want = ((it + 1) % check_every == 0) || it + 1 == maxiter;
        status = op.step(device_stop ? 0 : want, &scratch.ns);
        if (status != IPT_CUDA_SUCCESS) break;
        launched = it + 1;
        done = launched;
        if (want) {
            trace_mark("ipt:check", s);
            int stopped_at = -1;
            double r = NAN;
            int rs = IPT_CUDA_SUCCESS;
            if (device_stop) {
                rs = scratch.read_history(launched, &stopped_at, &r, s);
            } else if (cudaMemcpyAsync(scratch.host_norms, scratch.ns.norms, 2 * sizeof(double),
                                       cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                       cudaStreamSynchronize(s) != cudaSuccess) {
                rs = IPT_CUDA_CUDA_ERROR;
            } else {
                r = scratch.host_norms[0] / scratch.host_norms[1];
                if (r <= tol) stopped_at = launched - 1;
            }
            if (op.read_error(&host_err) != IPT_CUDA_SUCCESS || rs != IPT_CUDA_SUCCESS) {
                status = IPT_CUDA_CUDA_ERROR;
                break;
            }
            if (host_err != 0) {
                fprintf(stderr, "ipt_gb300: tensor-core product timed out (code %d)\n", host_err);
                status = IPT_CUDA_CUDA_ERROR;
                break;
            }
            if (stopped_at >= 0) {
                done = stopped_at + 1;
                fpres = r;
                break;
            }
            if (!isfinite(r)) {
                rollback = guard;
                if (!guard) {
                    status = IPT_CUDA_INVALID_ARGUMENT;
                }
                break;
            }
            fpres = r;
            if (guard) {
                if (r < best) {
                    best = r;
                    worse = 0;
                } else if (++worse >= 3) {
                    break;
                }
            }
        }
    }
    scratch.release(s);
    if (status != IPT_CUDA_SUCCESS) return status;
    if (rollback) {
        IPTGB_CHECK(op.export_fp64_prev(X));
    } else {
        IPTGB_CHECK(op.export_fp64(X));
    }
    *iterations = done;
    *fpres_out = fpres;
    *matvecs = (long long)done * p;
    return IPT_CUDA_SUCCESS;
}

}  // namespace iptgb
