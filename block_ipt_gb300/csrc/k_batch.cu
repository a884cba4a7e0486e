// k_batch.cu - batched dense block IPT: hundreds of independent symmetric
// instances of uneven n and k solved by one persistent kernel, replayed as a
// captured CUDA graph, with launch shapes picked by an autotuner.
//
// Per instance (the reference's plain dense IPT, IPT_C_GPU/src/ipt_cuda.cu:
// 1644-1703, targets = the first k diagonal positions, X_jj = 1):
//   Y = H X,  lambda_j = Y_jj,  r_ij = Y_ij - lambda_j X_ij,
//   X'_ij = X_ij + r_ij / (d_j - d_i)  (i != j),  X'_jj = 1,
// which is the reference's update (Delta X - X diag(Delta X)) o G written
// through the eigen-residual.  Each sweep therefore certifies the current
// block for free: the instance stops when every scaled residual
// ||r_j|| / (max(1, ||H||_inf) max(1, ||x_j||)) is at most residual_tol, and
// the certified block (not the next iterate) is returned with its Rayleigh
// quotients x_j^T H x_j / x_j^T x_j (from the same product; second order in
// the vector error, where (HX)_jj is first order).  ||H||_inf comes from the
// row sums of the first product.
//
// Mixed precision: the sweeps first run the product in FP32 (X staged in
// FP32, FP32 accumulation) until the fixed-point residual ||X' - X||_F /
// ||X||_F reaches lowp_tol, then switch to FP64-accurate sweeps, which
// certify and refine the block (the reference's mixed scheme: low-precision
// IPT, then FP64 IPT; IPT_C_GPU/src/mixed_precision/
// ipt_mixed_precision_cuda.cu:1153-1225).  The first FP32 sweep reads H in
// FP64 and writes its FP32 rounding to the plan's scratch, so the later FP32
// sweeps stream 4 bytes per entry.  The FP64-accurate sweeps run on the FP64
// pipe or, by default after FP32 sweeps, in double-float arithmetic on the
// FP32 pipe: every H entry split into an exact (hi, lo) float pair on the
// integer pipe, X staged as (hi, lo) pairs, each term accumulated by an exact
// two-product and two-sum (12 FP32 operations, about 2^-48 relative), so that
// a sweep costs about a fifth of its FP64-pipe time on GB300, whose FP64 pipe
// retires 1/64 of the FP32 rate.
//
// Scheduling: CTAs take instances from a device counter in descending order
// of cost n^2 k (longest first).  The kernel is launched in thread-block
// clusters; the most expensive instances (the leading n_team entries of the
// order, each above a fraction of the average load of one CTA) are solved by
// a whole cluster, each CTA owning a contiguous range of rows: after the
// product the cluster meets at a hardware barrier (the diagonal Y_jj that
// every row's update needs lies in the first CTA's rows), after the update
// each CTA publishes its per-column sums in shared memory and, past a second
// barrier, every CTA adds the cluster's sums in rank order from distributed
// shared memory, so all of them take the same (bitwise identical) decisions.
// Once the counter passes the team instances, every CTA takes the remaining
// instances on its own.  Without the split, one CTA of ~2 FP64 FMAs per clock
// holds an n = 2048, k = 16 instance for ~100 ms and sets the makespan.
//
// Within a CTA, a thread owns one row and all k columns of Y, k padded to a
// multiple of 4 (KP); columns of H stream in L-row chunks (coalesced,
// column-major, several loads per thread in flight), with the matching X
// chunk staged in shared memory.  Per-column sums are per-warp partials added
// in warp order, so every result is deterministic.  No host synchronisation
// inside the batch, so the whole solve is one graph launch.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <type_traits>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"
#include "dfloat.cuh"
#include "reduce.cuh"

#define IPT_API extern "C" __attribute__((visibility("default")))

namespace cg = cooperative_groups;

namespace iptgb {
namespace batch {

constexpr int kKMax = 16;
constexpr int kMaxWarps = 16;  // 512 threads
// per-sweep sums: r^2, x^2 and x.y per column, then |X' - X|^2, |X|^2 and the
// largest absolute row sum (a maximum)
constexpr int kDx = 3 * kKMax;
constexpr int kXx = kDx + 1;
constexpr int kHinf = kDx + 2;
constexpr int kRed = kDx + 3;

struct Inst {
    const double *H;
    double *vectors;  // output n x k column-major
    double *values;   // output k
    // FP64 scratch: two X blocks (n x KP, row-major, columns k..KP-1 zero),
    // Y and G_ij = 1/(d_j - d_i) (n x k each), and, for double-float sweeps,
    // the exact (hi, lo) float split of the two X blocks (n x KP each)
    double *xa;
    double *xb;
    double *y;
    double *g;
    float2 *xsa;
    float2 *xsb;
    // FP32 scratch of mixed plans: two X blocks (n x KP), Y and G (n x k), and
    // the FP32 rounding of H (n x n, written by the first FP32 sweep)
    float *xa32;
    float *xb32;
    float *y32;
    float *g32;
    float *h32;
    int n;
    int k;
};

struct Out {
    int iterations;       // all sweeps
    int fp64_iterations;  // certifying sweeps
    int converged;
    int status;           // 0 ok, 1 non-finite / zero gap
    double max_scaled_residual;
    unsigned long long t_start;
    unsigned long long t_end;
};

struct Params {
    const Inst *inst;
    const int *order;
    int count;
    int team;    // cluster size of the launch (1: no clusters)
    int n_team;  // the first n_team entries of `order` are solved by a whole cluster
    int *counter;
    Out *out;
    int mixed;
    int certify_df;  // FP64-accurate sweeps in double-float (FP32 pipe)
    double tol;
    int maxiter;
    int lowp_maxiter;
    double lowp_tol;
};

// arithmetic of one sweep's product
enum Kind {
    kF64 = 0,       // FP64 FMAs on H, FP64 X and Y
    kF32First = 1,  // FP32 FMAs, H rounded on load and written to h32, FP32 X and Y
    kF32 = 2,       // FP32 FMAs on h32, FP32 X and Y
    kDF = 3         // double-float terms on the exact (hi, lo) split of H and X, FP64 Y
};

template <int L>
struct Shared {
    double xs[2][L * kKMax];      // staged X chunks (double, float or float2 entries)
    double red[kMaxWarps][kRed];  // per-warp partial sums
    double part[2][kRed];         // this CTA's sums of the last two sweeps (read by the cluster)
    double tot[kRed];
    double lam[kKMax];
    float lamf[kKMax];  // lam of an FP32 sweep
    int cur;
};

// The CTA's Shared<L>, in dynamic shared memory.
extern __shared__ __align__(16) double g_batch_smem[];
template <int L>
__device__ __forceinline__ Shared<L> &smem()
{
    return *reinterpret_cast<Shared<L> *>(g_batch_smem);
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ double warp_sum_d(double x)
{
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    return x;
}

__device__ __forceinline__ double warp_max_d(double x)
{
    for (int off = 16; off > 0; off >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, off));
    return x;
}

// Bytes of one staged X entry of a sweep: FP64 X, FP32 X, or an X (hi, lo) pair.
template <int KIND>
struct EntryBytes {
    static constexpr int value = KIND == kF32 || KIND == kF32First ? 4 : 8;
};

// Rows [l0, l0 + lc) of a KP-padded X block (row-major, 16-byte aligned) into
// shared memory by 16-byte asynchronous copies through L2 (X rows of other
// CTAs of a cluster were written on other SMs), committed as one group.
template <int KIND, int KP>
__device__ __forceinline__ void stage_async(double *xs, const void *X, int l0, int lc)
{
    constexpr int kRowBytes = KP * EntryBytes<KIND>::value;  // a multiple of 16
    const char *src = static_cast<const char *>(X) + (size_t)l0 * kRowBytes;
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(xs);
    const int bytes = lc * kRowBytes;
    for (int o = 16 * (int)threadIdx.x; o < bytes; o += 16 * (int)blockDim.x) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + (uint32_t)o),
                     "l"(src + o)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ void stage_wait()
{
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// One column l of H (held in h: double for kF64/kF32First/kDF, float for kF32)
// times the staged X row xrow, into the row's accumulators.
template <int KIND, int KP>
__device__ __forceinline__ void term(double h, float hf, float hl, const double *xrow,
                                     double *a64, float *a32, float *e32)
{
    if (KIND == kF64) {
        const double2 *xr = reinterpret_cast<const double2 *>(xrow);
#pragma unroll
        for (int q = 0; q < KP / 2; ++q) {
            const double2 x = xr[q];
            a64[2 * q] = fma(h, x.x, a64[2 * q]);
            a64[2 * q + 1] = fma(h, x.y, a64[2 * q + 1]);
        }
    } else if (KIND == kDF) {
        const float4 *xr = reinterpret_cast<const float4 *>(xrow);
#pragma unroll
        for (int q = 0; q < KP / 2; ++q) {
            const float4 x = xr[q];
            df_acc(a32[2 * q], e32[2 * q], hf, hl, x.x, x.y);
            df_acc(a32[2 * q + 1], e32[2 * q + 1], hf, hl, x.z, x.w);
        }
    } else {
        const float4 *xr = reinterpret_cast<const float4 *>(xrow);
#pragma unroll
        for (int q = 0; q < KP / 4; ++q) {
            const float4 x = xr[q];
            a32[4 * q] = fmaf(hf, x.x, a32[4 * q]);
            a32[4 * q + 1] = fmaf(hf, x.y, a32[4 * q + 1]);
            a32[4 * q + 2] = fmaf(hf, x.z, a32[4 * q + 2]);
            a32[4 * q + 3] = fmaf(hf, x.w, a32[4 * q + 3]);
        }
    }
}

// One entry h = H[i, l] (FP64) of a sweep that reads H: the row sum of the
// first sweep, the FP32 copy of the first FP32 sweep, the exact split of a
// double-float sweep; then its term.
template <int KIND, int KP>
__device__ __forceinline__ void entry_term(const Inst &I, size_t off, double h, bool rowsum,
                                           double &rs, const double *xrow, double *a64,
                                           float *a32, float *e32)
{
    if (rowsum) rs += fabs(h);
    if (KIND == kF64) {
        term<KIND, KP>(h, 0.0f, 0.0f, xrow, a64, a32, e32);
    } else if (KIND == kDF) {
        const dfloat d = df_from_double(h);
        term<KIND, KP>(h, d.hi, d.lo, xrow, a64, a32, e32);
    } else {
        const float hf = __double2float_rn(h);
        I.h32[off] = hf;
        term<KIND, KP>(h, hf, 0.0f, xrow, a64, a32, e32);
    }
}

// Rows [r0, r1) of Y = H X in KIND's arithmetic.  With `rowsum`, also returns
// the largest absolute row sum of those rows.  X chunks of L rows are copied
// into two shared-memory buffers asynchronously, one chunk ahead of use, so
// each chunk costs one barrier and no exposed L2 latency.
template <int KIND, int KP, int L>
__device__ __forceinline__ double product(const Inst &I, const void *X, void *Yv, int r0, int r1,
                                          bool rowsum)
{
    Shared<L> &sm = smem<L>();
    // loads in flight per thread: FP32 entries are half the bytes
    constexpr int U = KIND == kF32 ? 16 : 8;
    // entries of one staged X row, in doubles
    constexpr int XD = KIND == kF64 || KIND == kDF ? KP : KP / 2;
    const int n = I.n, k = I.k;
    double hinf = 0.0;
    for (int rb = r0; rb < r1; rb += blockDim.x) {
        const int i = rb + threadIdx.x;
        const bool row = i < r1;
        double a64[KIND == kF64 ? KP : 1];
        float a32[KIND == kF64 ? 1 : KP];
        float e32[KIND == kDF ? KP : 1];
#pragma unroll
        for (int j = 0; j < (KIND == kF64 ? KP : 1); ++j) a64[j] = 0.0;
#pragma unroll
        for (int j = 0; j < (KIND == kF64 ? 1 : KP); ++j) a32[j] = 0.0f;
#pragma unroll
        for (int j = 0; j < (KIND == kDF ? KP : 1); ++j) e32[j] = 0.0f;
        double rs = 0.0;
        __syncthreads();  // both buffers free (previous row block or sweep done)
        stage_async<KIND, KP>(sm.xs[0], X, 0, min(L, n));
        int buf = 0;
        for (int l0 = 0; l0 < n; l0 += L) {
            const int lc = min(L, n - l0);
            stage_wait();
            __syncthreads();  // chunk l0 staged; everyone done with the other buffer
            if (l0 + L < n) stage_async<KIND, KP>(sm.xs[buf ^ 1], X, l0 + L, min(L, n - l0 - L));
            if (row) {
                const double *xs = sm.xs[buf];
                const size_t base = (size_t)l0 * n + i;
                int l = 0;
                for (; l + U <= lc; l += U) {
                    double hd[KIND == kF32 ? 1 : U];
                    float hv[KIND == kF32 ? U : 1];
                    if (KIND == kF32) {
                        // written by this thread in the first FP32 sweep: plain loads
                        const float *p = I.h32 + base + (size_t)l * n;
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            hv[u] = *p;
                            p += n;
                        }
                    } else {
                        const double *p = I.H + base + (size_t)l * n;
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            hd[u] = __ldg(p);
                            p += n;
                        }
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const double *xrow = xs + (l + u) * XD;
                        if (KIND == kF32) {
                            term<KIND, KP>(0.0, hv[u], 0.0f, xrow, a64, a32, e32);
                        } else {
                            entry_term<KIND, KP>(I, base + (size_t)(l + u) * n, hd[u], rowsum,
                                                 rs, xrow, a64, a32, e32);
                        }
                    }
                }
                for (; l < lc; ++l) {
                    const double *xrow = xs + l * XD;
                    const size_t off = base + (size_t)l * n;
                    if (KIND == kF32) {
                        term<KIND, KP>(0.0, I.h32[off], 0.0f, xrow, a64, a32, e32);
                    } else {
                        entry_term<KIND, KP>(I, off, __ldg(I.H + off), rowsum, rs, xrow, a64,
                                             a32, e32);
                    }
                }
            }
            buf ^= 1;
        }
        if (row) {
#pragma unroll
            for (int j = 0; j < KP; ++j) {
                if (j < k) {
                    if (KIND == kF64) {
                        static_cast<double *>(Yv)[(size_t)i * k + j] = a64[j];
                    } else if (KIND == kDF) {
                        static_cast<double *>(Yv)[(size_t)i * k + j] =
                            (double)a32[j] + (double)e32[j];
                    } else {
                        static_cast<float *>(Yv)[(size_t)i * k + j] = a32[j];
                    }
                }
            }
            hinf = fmax(hinf, rs);
        }
    }
    return hinf;
}

template <int KIND, int L>
__device__ __forceinline__ double product_kp(const Inst &I, const void *X, void *Y, int r0,
                                             int r1, bool rowsum)
{
    switch ((I.k + 3) >> 2) {
    case 1: return product<KIND, 4, L>(I, X, Y, r0, r1, rowsum);
    case 2: return product<KIND, 8, L>(I, X, Y, r0, r1, rowsum);
    case 3: return product<KIND, 12, L>(I, X, Y, r0, r1, rowsum);
    default: return product<KIND, 16, L>(I, X, Y, r0, r1, rowsum);
    }
}

// Solve instance order[q]: alone (TEAM false, rows [0, n)) or as CTA `rank`
// of a cluster of `team` CTAs (rows in contiguous ranges of a multiple of 32).
template <int L, bool TEAM>
__device__ void solve(const Params &p, int q, int rank, int team)
{
    Shared<L> &sm = smem<L>();
    const int id = p.order[q];
    const Inst I = p.inst[id];
    const int n = I.n, k = I.k;
    const int KP = (k + 3) & ~3;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    int r0 = 0, r1 = n;
    if (TEAM) {
        const int rows = ((n + team - 1) / team + 31) & ~31;
        r0 = min(n, rank * rows);
        r1 = min(n, r0 + rows);
    }
    auto team_sync = [&]() {
        if (TEAM) {
            cg::this_cluster().sync();
        } else {
            __syncthreads();
        }
    };
    Out o{};
    if (tid == 0 && rank == 0) o.t_start = global_ns();
    // own rows: X = the first k unit vectors (both buffers padded with zeros),
    // G_ij = 1/(d_j - d_i) (the reference's factor, IPT_C_GPU/src/ipt_cuda.cu:
    // 1369-1443), and their FP32 / split copies
    for (size_t e = (size_t)r0 * KP + tid; e < (size_t)r1 * KP; e += blockDim.x) {
        const int i = (int)(e / KP);
        const int j = (int)(e - (size_t)i * KP);
        const double x = i == j && j < k ? 1.0 : 0.0;
        I.xa[e] = x;
        I.xb[e] = 0.0;
        if (p.certify_df) {
            I.xsa[e] = make_float2((float)x, 0.0f);
            I.xsb[e] = make_float2(0.0f, 0.0f);
        }
        if (p.mixed) {
            I.xa32[e] = (float)x;
            I.xb32[e] = 0.0f;
        }
        if (j < k) {
            const size_t eg = (size_t)i * k + j;
            const double g =
                i == j ? 0.0 : 1.0 / (I.H[(size_t)j * n + j] - I.H[(size_t)i * n + i]);
            I.g[eg] = g;
            if (p.mixed) I.g32[eg] = (float)g;
        }
    }
    team_sync();
    double *X = I.xa, *Xn = I.xb;
    float2 *Xs = I.xsa, *Xsn = I.xsb;
    float *X32 = I.xa32, *Xn32 = I.xb32;
    bool fp64 = !p.mixed;
    bool h32_ready = false;
    double hinf = -1.0;
    int it = 0, it64 = 0;
    bool done = false;
    int status = 0;
    double maxres = INFINITY;
    const int limit = p.maxiter + (p.mixed ? p.lowp_maxiter : 0);
    for (; it < limit && !done; ++it) {
        if (lane == 0) {
            for (int c = 0; c < kRed; ++c) sm.red[warp][c] = 0.0;
        }
        const bool first = hinf < 0.0;
        double hs;
        if (fp64 && p.certify_df) {
            hs = product_kp<kDF, L>(I, Xs, I.y, r0, r1, first);
        } else if (fp64) {
            hs = product_kp<kF64, L>(I, X, I.y, r0, r1, first);
        } else if (h32_ready) {
            hs = product_kp<kF32, L>(I, X32, I.y32, r0, r1, first);
        } else {
            hs = product_kp<kF32First, L>(I, X32, I.y32, r0, r1, first);
            h32_ready = true;
        }
        if (first) {
            hs = warp_max_d(hs);
            if (lane == 0) sm.red[warp][kHinf] = hs;
        }
        team_sync();  // Y rows of every CTA written
        if (tid < k) {
            if (fp64) {
                sm.lam[tid] = __ldcg(I.y + (size_t)tid * k + tid);
            } else {
                sm.lamf[tid] = __ldcg(I.y32 + (size_t)tid * k + tid);
            }
        }
        __syncthreads();
        // residuals r = Y - X diag(lambda), update X' = X + r o G, norms
        if (!fp64) {
            // FP32 sweep: FP32 arithmetic, only the fixed-point residual
            float fdx = 0.0f, fx = 0.0f;
            for (int rb = r0; rb < r1; rb += blockDim.x) {
                const int i = rb + tid;
                if (i >= r1) continue;
                for (int j = 0; j < k; ++j) {
                    const size_t e = (size_t)i * k + j, ex = (size_t)i * KP + j;
                    const float x = X32[ex];
                    if (i != j) {
                        const float r = fmaf(-sm.lamf[j], x, I.y32[e]);
                        const float dx = r * I.g32[e];
                        Xn32[ex] = x + dx;
                        fdx = fmaf(dx, dx, fdx);
                    } else {
                        Xn32[ex] = 1.0f;
                    }
                    fx = fmaf(x, x, fx);
                }
            }
            const double sdx = warp_sum_d((double)fdx);
            const double sx = warp_sum_d((double)fx);
            if (lane == 0) {
                sm.red[warp][kDx] += sdx;
                sm.red[warp][kXx] += sx;
            }
        } else {
            for (int rb = r0; rb < r1; rb += blockDim.x) {
                const int i = rb + tid;
                const bool row = i < r1;
                for (int j = 0; j < k; ++j) {
                    double rr = 0.0, xx = 0.0, xy = 0.0;
                    if (row) {
                        const size_t e = (size_t)i * k + j, ex = (size_t)i * KP + j;
                        const double x = X[ex];
                        const double yv = I.y[e];
                        const double r = fma(-sm.lam[j], x, yv);
                        xy = x * yv;
                        const double xn = i != j ? fma(r, I.g[e], x) : 1.0;
                        Xn[ex] = xn;
                        if (p.certify_df) {
                            const dfloat d = df_from_double(xn);
                            Xsn[ex] = make_float2(d.hi, d.lo);
                        }
                        if (i != j) rr = r * r;
                        xx = x * x;
                    }
                    rr = warp_sum_d(rr);
                    xx = warp_sum_d(xx);
                    xy = warp_sum_d(xy);
                    if (lane == 0) {
                        sm.red[warp][j] += rr;
                        sm.red[warp][kKMax + j] += xx;
                        sm.red[warp][2 * kKMax + j] += xy;
                    }
                }
            }
        }
        __syncthreads();
        const int par = it & 1;
        if (tid < kRed) {
            double s = 0.0;
            for (int w = 0; w < nwarps; ++w) {
                s = tid == kHinf ? fmax(s, sm.red[w][tid]) : s + sm.red[w][tid];
            }
            sm.part[par][tid] = s;
        }
        if (TEAM) {
            cg::cluster_group cl = cg::this_cluster();
            cl.sync();  // every CTA's sums published
            if (tid < kRed) {
                double s = 0.0;
                for (int r = 0; r < team; ++r) {
                    const double v = *cl.map_shared_rank(&sm.part[par][tid], r);
                    s = tid == kHinf ? fmax(s, v) : s + v;
                }
                sm.tot[tid] = s;
            }
        } else if (tid < kRed) {
            sm.tot[tid] = sm.part[par][tid];
        }
        __syncthreads();
        if (first) hinf = sm.tot[kHinf];
        if (fp64) {
            ++it64;
            double mx = 0.0;
            bool finite = true;
            for (int j = 0; j < k; ++j) {
                const double sc = sqrt(sm.tot[j]) /
                                  (fmax(1.0, hinf) * fmax(1.0, sqrt(sm.tot[kKMax + j])));
                if (!isfinite(sc)) finite = false;
                mx = fmax(mx, sc);
            }
            maxres = finite ? mx : INFINITY;
            if (!finite) {
                status = 1;
                done = true;
            } else if (mx <= p.tol) {
                done = true;  // X (not Xn) is the certified block
            }
            if (!done) {
                double *t = X;
                X = Xn;
                Xn = t;
                float2 *ts = Xs;
                Xs = Xsn;
                Xsn = ts;
                if (it64 >= p.maxiter) {
                    ++it;
                    break;
                }
            }
        } else {
            const double fp = sqrt(sm.tot[kDx]) / sqrt(fmax(sm.tot[kXx], 1e-300));
            const bool diverged = !isfinite(fp);
            if (diverged || fp <= p.lowp_tol || it + 1 >= p.lowp_maxiter) {
                // FP64-accurate sweeps from here: the FP32 iterate as the FP64
                // block (own rows), or, if the FP32 sweeps diverged, the unit
                // vectors
                for (size_t e = (size_t)r0 * KP + tid; e < (size_t)r1 * KP; e += blockDim.x) {
                    const int i = (int)(e / KP);
                    const int j = (int)(e - (size_t)i * KP);
                    const double x = diverged ? (i == j && j < k ? 1.0 : 0.0) : (double)Xn32[e];
                    X[e] = x;
                    if (p.certify_df) {
                        const dfloat d = df_from_double(x);
                        Xs[e] = make_float2(d.hi, d.lo);
                    }
                }
                team_sync();  // every row before the next product stages X
                fp64 = true;
            } else {
                float *t = X32;
                X32 = Xn32;
                Xn32 = t;
            }
        }
    }
    __syncthreads();
    // outputs: the certified block (own rows), column-major, and its Ritz values
    for (size_t e = (size_t)r0 * k + tid; e < (size_t)r1 * k; e += blockDim.x) {
        const int i = (int)(e / k);
        const int j = (int)(e - (size_t)i * k);
        I.vectors[(size_t)j * n + i] = X[(size_t)i * KP + j];
    }
    if (rank == 0) {
        // Rayleigh quotients of the returned block (the sums hold its last sweep)
        if (tid < k) I.values[tid] = sm.tot[2 * kKMax + tid] / sm.tot[kKMax + tid];
        if (tid == 0) {
            o.iterations = it;
            o.fp64_iterations = it64;
            o.converged = done && status == 0 ? 1 : 0;
            o.status = status;
            o.max_scaled_residual = maxres;
            o.t_end = global_ns();
            p.out[id] = o;
        }
    }
}

template <int L>
__global__ void __launch_bounds__(512, 1)
batch_ipt_kernel(Params p)
{
    Shared<L> &sm = smem<L>();
    const int tid = threadIdx.x;
    int rank = 0;
    if (p.team > 1) rank = (int)cg::this_cluster().block_rank();
    bool team_mode = p.team > 1 && p.n_team > 0;
    for (;;) {
        __syncthreads();
        int q;
        if (team_mode) {
            cg::cluster_group cl = cg::this_cluster();
            if (rank == 0 && tid == 0) sm.cur = atomicAdd(p.counter, 1);
            cl.sync();
            q = *cl.map_shared_rank(&sm.cur, 0);
            cl.sync();  // every CTA has read the index before rank 0 moves on
            if (q >= p.count) return;
            if (q < p.n_team) {
                solve<L, true>(p, q, rank, p.team);
                continue;
            }
            // past the team instances: rank 0 solves this one alone, the
            // others fetch their own from now on
            team_mode = false;
            if (rank != 0) continue;
        } else {
            if (tid == 0) sm.cur = atomicAdd(p.counter, 1);
            __syncthreads();
            q = sm.cur;
            if (q >= p.count) return;
        }
        solve<L, false>(p, q, 0, 1);
    }
}

}  // namespace batch

// ---------------------------------------------------------------------------
// Plan: device instance table, scratch pool, autotuned launch shape, graph.
// ---------------------------------------------------------------------------
// Scratch of one instance, rounded so that the next instance's blocks stay
// 16-byte aligned: doubles (two KP-padded X blocks, their double-float
// splits, Y and G) and, for mixed plans, floats (two KP-padded X blocks, Y,
// G and the FP32 copy of H).
inline size_t batch_doubles(int n, int k)
{
    const size_t kp = (size_t)((k + 3) & ~3);
    return 4 * (size_t)n * kp + ((2 * (size_t)n * k + 1) & ~(size_t)1);
}

inline size_t batch_floats(int n, int k)
{
    const size_t kp = (size_t)((k + 3) & ~3);
    return 2 * (size_t)n * kp + (((2 * (size_t)n * k + (size_t)n * n) + 3) & ~(size_t)3);
}

struct BatchPlan {
    int count = 0;
    std::vector<batch::Inst> host_inst;
    std::vector<double> cost;  // n^2 k of order[q]
    std::vector<int> order_n;  // n of order[q]
    batch::Inst *inst = nullptr;
    int *order = nullptr;
    int *counter = nullptr;
    batch::Out *out = nullptr;
    double *pool = nullptr;
    float *pool32 = nullptr;
    int mixed = 0;
    int certify_df = 0;
    double tol = 1e-8;
    int maxiter = 100;
    int lowp_maxiter = 200;
    double lowp_tol = 1e-6;
    int threads = 512;
    int chunk = 128;
    // instances above team_pct % of the average load of one CTA go to a
    // whole cluster (0: every instance on one CTA)
    int team_pct = 25;
    int cluster = 1;  // cluster size of the launch
    int n_team = 0;
    int ctas = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;

    // grid, cluster size and team instances for the current threads/chunk/team_pct
    int configure()
    {
        int dev = 0, sms = 0, per_sm = 0;
        IPTGB_CUDA(cudaGetDevice(&dev));
        IPTGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (chunk == 64) {
            IPTGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per_sm, batch::batch_ipt_kernel<64>, threads, sizeof(batch::Shared<64>)));
        } else {
            IPTGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per_sm, batch::batch_ipt_kernel<128>, threads, sizeof(batch::Shared<128>)));
        }
        const int full = std::max(1, sms * std::max(1, per_sm));
        cluster = 1;
        ctas = std::min(count, full);
        n_team = 0;
        if (team_pct <= 0) return IPT_CUDA_SUCCESS;
        // the largest cluster size that keeps nearly every CTA slot of the
        // device busy (clusters are placed within one GPC)
        const int forced = env_int("IPT_GB300_BATCH_CLUSTER", 0);
        const int sizes[3] = {8, 4, 2};
        for (int c : sizes) {
            if (forced > 0 && c != forced) continue;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)(full / c * c));
            cfg.blockDim = dim3((unsigned)threads);
            cfg.dynamicSmemBytes = chunk == 64 ? sizeof(batch::Shared<64>)
                                               : sizeof(batch::Shared<128>);
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = (unsigned)c;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int clusters = 0;
            cudaError_t e;
            if (chunk == 64) {
                e = cudaOccupancyMaxActiveClusters(&clusters, batch::batch_ipt_kernel<64>, &cfg);
            } else {
                e = cudaOccupancyMaxActiveClusters(&clusters, batch::batch_ipt_kernel<128>, &cfg);
            }
            if (e != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            if (clusters * c >= (forced > 0 ? 1 : (9 * full) / 10)) {
                cluster = c;
                ctas = clusters * c;
                break;
            }
        }
        if (cluster == 1) return IPT_CUDA_SUCCESS;
        double total = 0.0;
        for (double c : cost) total += c;
        const double thr = (double)team_pct / 100.0 * total / ctas;
        while (n_team < count && cost[(size_t)n_team] > thr &&
               order_n[(size_t)n_team] >= 32 * cluster) {
            ++n_team;
        }
        if (n_team == 0) {
            cluster = 1;
            ctas = std::min(count, full);
        }
        return IPT_CUDA_SUCCESS;
    }

    int launch(cudaStream_t s)
    {
        batch::Params p{inst,   order, count,      cluster, n_team,  counter,      out,
                        mixed,  certify_df, tol,   maxiter, lowp_maxiter, lowp_tol};
        IPTGB_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), s));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)ctas);
        cfg.blockDim = dim3((unsigned)threads);
        cfg.dynamicSmemBytes = chunk == 64 ? sizeof(batch::Shared<64>) : sizeof(batch::Shared<128>);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)cluster;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = cluster > 1 ? 1 : 0;
        if (chunk == 64) {
            IPTGB_CUDA(cudaLaunchKernelEx(&cfg, batch::batch_ipt_kernel<64>, p));
        } else {
            IPTGB_CUDA(cudaLaunchKernelEx(&cfg, batch::batch_ipt_kernel<128>, p));
        }
        IPTGB_LAUNCH();
        return IPT_CUDA_SUCCESS;
    }
    void drop_graph()
    {
        if (exec != nullptr) cudaGraphExecDestroy(exec);
        if (graph != nullptr) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
    int capture(cudaStream_t s)
    {
        drop_graph();
        cudaStream_t cs = nullptr;
        IPTGB_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        int st = IPT_CUDA_SUCCESS;
        if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            st = IPT_CUDA_CUDA_ERROR;
        } else {
            st = launch(cs);
            if (cudaStreamEndCapture(cs, &graph) != cudaSuccess) st = IPT_CUDA_CUDA_ERROR;
        }
        if (st == IPT_CUDA_SUCCESS && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
            st = IPT_CUDA_CUDA_ERROR;
        }
        cudaStreamDestroy(cs);
        (void)s;
        return st;
    }
    ~BatchPlan()
    {
        drop_graph();
        cudaFree(inst);
        cudaFree(order);
        cudaFree(counter);
        cudaFree(out);
        cudaFree(pool);
        cudaFree(pool32);
    }
};

}  // namespace iptgb

using namespace iptgb;

#include "../../include/ipt_block.h"

IPT_API void ipt_block_batch_default_options(IPTBatchOptions *o)
{
    if (o == nullptr) return;
    o->precision = IPT_BLOCK_FP64;
    o->residual_tol = 1e-8;
    o->maxiter = 100;
    o->lowp_maxiter = 200;
    o->lowp_tol = 1e-6;
    o->threads = 0;
    o->chunk = 0;
    o->certify_precision = -1;
}

IPT_API int ipt_block_batch_plan_create(const IPTBatchInstance *instances, int count,
                                        const IPTBatchOptions *options, void **plan_out)
{
    if (plan_out == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    *plan_out = nullptr;
    if (instances == nullptr || count <= 0) return IPT_CUDA_INVALID_ARGUMENT;
    IPTBatchOptions opt;
    ipt_block_batch_default_options(&opt);
    if (options != nullptr) opt = *options;
    if ((opt.precision != IPT_BLOCK_FP64 && opt.precision != IPT_BLOCK_FP32) ||
        !(opt.residual_tol > 0.0) || opt.maxiter <= 0 || opt.lowp_maxiter < 0 ||
        (opt.threads != 0 && opt.threads != 128 && opt.threads != 256 && opt.threads != 512) ||
        (opt.chunk != 0 && opt.chunk != 64 && opt.chunk != 128) ||
        (opt.certify_precision != -1 && opt.certify_precision != IPT_BLOCK_FP64 &&
         opt.certify_precision != IPT_BLOCK_DF64)) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    const bool mixed = opt.precision == IPT_BLOCK_FP32;
    size_t pool = 0, pool32 = 0;
    for (int b = 0; b < count; ++b) {
        const IPTBatchInstance &x = instances[b];
        if (x.H == nullptr || x.vectors == nullptr || x.values == nullptr || x.n <= 0 ||
            x.k <= 0 || x.k > batch::kKMax || x.k > x.n) {
            return IPT_CUDA_INVALID_ARGUMENT;
        }
        pool += batch_doubles(x.n, x.k);
        if (mixed) pool32 += batch_floats(x.n, x.k);
    }
    auto *P = new BatchPlan();
    P->count = count;
    P->mixed = mixed ? 1 : 0;
    P->certify_df = opt.certify_precision == IPT_BLOCK_DF64 ||
                    (opt.certify_precision == -1 && P->mixed);
    P->tol = opt.residual_tol;
    P->maxiter = opt.maxiter;
    P->lowp_maxiter = opt.lowp_maxiter;
    P->lowp_tol = opt.lowp_tol;
    P->threads = opt.threads != 0 ? opt.threads : 256;
    P->chunk = opt.chunk != 0 ? opt.chunk : 128;
    P->team_pct = std::max(0, env_int("IPT_GB300_BATCH_TEAM_PCT", 25));
    int st = IPT_CUDA_SUCCESS;
    if (cudaMalloc((void **)&P->pool, pool * sizeof(double)) != cudaSuccess ||
        (pool32 > 0 && cudaMalloc((void **)&P->pool32, pool32 * sizeof(float)) != cudaSuccess) ||
        cudaMalloc((void **)&P->inst, count * sizeof(batch::Inst)) != cudaSuccess ||
        cudaMalloc((void **)&P->order, count * sizeof(int)) != cudaSuccess ||
        cudaMalloc((void **)&P->counter, sizeof(int)) != cudaSuccess ||
        cudaMalloc((void **)&P->out, count * sizeof(batch::Out)) != cudaSuccess) {
        st = IPT_CUDA_ALLOCATION_FAILED;
    }
    if (st == IPT_CUDA_SUCCESS) {
        P->host_inst.resize(count);
        size_t off = 0, off32 = 0;
        for (int b = 0; b < count; ++b) {
            const IPTBatchInstance &x = instances[b];
            batch::Inst &I = P->host_inst[b];
            I.H = x.H;
            I.vectors = x.vectors;
            I.values = x.values;
            I.n = x.n;
            I.k = x.k;
            // KP-padded X blocks first: every block starts 16-byte aligned
            const size_t nkp = (size_t)x.n * (size_t)((x.k + 3) & ~3);
            const size_t nk = (size_t)x.n * x.k;
            I.xa = P->pool + off;
            I.xb = I.xa + nkp;
            I.xsa = reinterpret_cast<float2 *>(I.xb + nkp);
            I.xsb = I.xsa + nkp;
            I.y = reinterpret_cast<double *>(I.xsb + nkp);
            I.g = I.y + nk;
            off += batch_doubles(x.n, x.k);
            I.xa32 = I.xb32 = I.y32 = I.g32 = I.h32 = nullptr;
            if (mixed) {
                I.xa32 = P->pool32 + off32;
                I.xb32 = I.xa32 + nkp;
                I.y32 = I.xb32 + nkp;
                I.g32 = I.y32 + nk;
                I.h32 = I.g32 + nk;
                off32 += batch_floats(x.n, x.k);
            }
        }
        // longest (n^2 k) first
        std::vector<int> order(count);
        std::iota(order.begin(), order.end(), 0);
        auto cost_of = [&](int b) {
            return (double)instances[b].n * instances[b].n * instances[b].k;
        };
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return cost_of(a) > cost_of(b); });
        P->cost.resize(count);
        P->order_n.resize(count);
        for (int q = 0; q < count; ++q) {
            P->cost[(size_t)q] = cost_of(order[(size_t)q]);
            P->order_n[(size_t)q] = instances[order[(size_t)q]].n;
        }
        if (cudaMemcpy(P->inst, P->host_inst.data(), count * sizeof(batch::Inst),
                       cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(P->order, order.data(), count * sizeof(int), cudaMemcpyHostToDevice) !=
                cudaSuccess) {
            st = IPT_CUDA_CUDA_ERROR;
        }
    }
    if (st == IPT_CUDA_SUCCESS) st = P->configure();
    if (st == IPT_CUDA_SUCCESS) st = P->capture(nullptr);
    if (st != IPT_CUDA_SUCCESS) {
        delete P;
        return st;
    }
    *plan_out = P;
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_block_batch_plan_run(void *plan, void *stream)
{
    if (plan == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    auto *P = static_cast<BatchPlan *>(plan);
    if (P->exec == nullptr) return IPT_CUDA_CUDA_ERROR;
    IPTGB_CUDA(cudaGraphLaunch(P->exec, (cudaStream_t)stream));
    count_launch();
    return IPT_CUDA_SUCCESS;
}

// Times every launch shape (threads x chunk x team threshold) on the real
// batch, one warm-up launch first, and re-captures the fastest.
IPT_API int ipt_block_batch_plan_autotune(void *plan, void *stream, int *threads_out,
                                          int *chunk_out, double *best_ms_out)
{
    if (plan == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    auto *P = static_cast<BatchPlan *>(plan);
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t e0, e1;
    IPTGB_CUDA(cudaEventCreate(&e0));
    IPTGB_CUDA(cudaEventCreate(&e1));
    const int cand_threads[3] = {128, 256, 512};
    const int cand_chunk[2] = {64, 128};
    const int cand_team[3] = {0, 25, 100};
    double best = INFINITY;
    int bt = P->threads, bc = P->chunk, bp = P->team_pct;
    int st = P->launch(s);  // warm-up
    for (int ti = 0; ti < 3 && st == IPT_CUDA_SUCCESS; ++ti) {
        for (int ci = 0; ci < 2 && st == IPT_CUDA_SUCCESS; ++ci) {
            for (int pi = 0; pi < 3 && st == IPT_CUDA_SUCCESS; ++pi) {
                P->threads = cand_threads[ti];
                P->chunk = cand_chunk[ci];
                P->team_pct = cand_team[pi];
                st = P->configure();
                float ms = 0.f;
                if (st == IPT_CUDA_SUCCESS) {
                    cudaEventRecord(e0, s);
                    st = P->launch(s);
                    cudaEventRecord(e1, s);
                    if (cudaEventSynchronize(e1) != cudaSuccess ||
                        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
                        st = IPT_CUDA_CUDA_ERROR;
                    }
                }
                if (st == IPT_CUDA_SUCCESS && ms < best) {
                    best = ms;
                    bt = P->threads;
                    bc = P->chunk;
                    bp = P->team_pct;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    P->threads = bt;
    P->chunk = bc;
    P->team_pct = bp;
    if (st == IPT_CUDA_SUCCESS) st = P->configure();
    if (st == IPT_CUDA_SUCCESS) st = P->capture(s);
    if (threads_out) *threads_out = bt;
    if (chunk_out) *chunk_out = bc;
    if (best_ms_out) *best_ms_out = best;
    return st;
}

IPT_API int ipt_block_batch_plan_reports(void *plan, IPTBatchReport *reports)
{
    if (plan == nullptr || reports == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    auto *P = static_cast<BatchPlan *>(plan);
    std::vector<batch::Out> h(P->count);
    IPTGB_CUDA(cudaMemcpy(h.data(), P->out, P->count * sizeof(batch::Out),
                          cudaMemcpyDeviceToHost));
    unsigned long long t0 = ~0ULL;
    for (const auto &o : h) t0 = std::min(t0, o.t_start);
    for (int b = 0; b < P->count; ++b) {
        reports[b].converged = h[b].converged;
        reports[b].status = h[b].status;
        reports[b].iterations = h[b].iterations;
        reports[b].fp64_iterations = h[b].fp64_iterations;
        reports[b].max_scaled_residual = h[b].max_scaled_residual;
        reports[b].latency_ms = (double)(h[b].t_end - h[b].t_start) * 1e-6;
        reports[b].completion_ms = (double)(h[b].t_end - t0) * 1e-6;
    }
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_block_batch_plan_shape(void *plan, int *threads, int *chunk, int *cluster,
                                      int *ctas, int *team_instances)
{
    if (plan == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    const auto *P = static_cast<const BatchPlan *>(plan);
    if (threads) *threads = P->threads;
    if (chunk) *chunk = P->chunk;
    if (cluster) *cluster = P->cluster;
    if (ctas) *ctas = P->ctas;
    if (team_instances) *team_instances = P->n_team;
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_block_batch_plan_destroy(void *plan)
{
    delete static_cast<BatchPlan *>(plan);
    return IPT_CUDA_SUCCESS;
}
