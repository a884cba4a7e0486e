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
    double *xa;       // scratch, row-major n x k
    double *xb;
    double *y;
    float *h32;       // scratch n x n (mixed plans): FP32 rounding of H
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
    kF64 = 0,       // FP64 FMAs on H
    kF32First = 1,  // FP32 FMAs, H rounded on load and written to h32
    kF32 = 2,       // FP32 FMAs on h32
    kDF = 3         // double-float terms on the exact (hi, lo) split of H
};

template <int L>
struct Shared {
    double xs[L * kKMax];         // staged X chunk (double, float or float2 entries)
    double red[kMaxWarps][kRed];  // per-warp partial sums
    double part[2][kRed];         // this CTA's sums of the last two sweeps (read by the cluster)
    double tot[kRed];
    double lam[kKMax];
    int cur;
};

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

// X chunk rows [l0, l0 + lc) into shared memory as KIND's operand type, KP
// entries per row (zero past k).  X rows of other CTAs of a cluster were
// written on other SMs: read through L2.
template <int KIND, int KP, int L>
__device__ __forceinline__ void stage_x(Shared<L> &sm, const double *__restrict__ X, int l0,
                                        int lc, int k)
{
    for (int e = threadIdx.x; e < lc * KP; e += blockDim.x) {
        const int l = e / KP;
        const int j = e - l * KP;
        const double v = j < k ? __ldcg(X + (size_t)(l0 + l) * k + j) : 0.0;
        if (KIND == kF64) {
            sm.xs[e] = v;
        } else if (KIND == kDF) {
            const dfloat d = df_from_double(v);
            reinterpret_cast<float2 *>(sm.xs)[e] = make_float2(d.hi, d.lo);
        } else {
            reinterpret_cast<float *>(sm.xs)[e] = __double2float_rn(v);
        }
    }
}

// One column l of H (held in h: double for kF64/kF32First/kDF, float for
// kF32) times the staged X row xr, into the row's accumulators.
template <int KIND, int KP>
__device__ __forceinline__ void term(double h, float hf, const double *xrow, double *a64,
                                     float *a32, float *e32)
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
        const dfloat d = df_from_double(h);
        const float4 *xr = reinterpret_cast<const float4 *>(xrow);
#pragma unroll
        for (int q = 0; q < KP / 2; ++q) {
            const float4 x = xr[q];
            df_acc(a32[2 * q], e32[2 * q], d.hi, d.lo, x.x, x.y);
            df_acc(a32[2 * q + 1], e32[2 * q + 1], d.hi, d.lo, x.z, x.w);
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

// Rows [r0, r1) of Y = H X in KIND's arithmetic.  With `rowsum`, also returns
// the largest absolute row sum of those rows (from the FP64 entries).
template <int KIND, int KP, int L>
__device__ double product(const Inst &I, const double *__restrict__ X, Shared<L> &sm, int r0,
                          int r1, bool rowsum)
{
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
        for (int l0 = 0; l0 < n; l0 += L) {
            const int lc = min(L, n - l0);
            __syncthreads();
            stage_x<KIND, KP, L>(sm, X, l0, lc, k);
            __syncthreads();
            if (!row) continue;
            const size_t base = (size_t)l0 * n + i;
            int l = 0;
            for (; l + U <= lc; l += U) {
                double hd[KIND == kF32 ? 1 : U];
                float hf[KIND == kF32 ? U : 1];
                if (KIND == kF32) {
                    // written by this thread in the first FP32 sweep: plain loads
                    const float *p = I.h32 + base + (size_t)l * n;
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        hf[u] = *p;
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
                    const double *xrow = sm.xs + (l + u) * XD;
                    if (KIND == kF32) {
                        term<KIND, KP>(0.0, hf[u], xrow, a64, a32, e32);
                    } else {
                        if (rowsum) rs += fabs(hd[u]);
                        float h32 = 0.0f;
                        if (KIND == kF32First) {
                            h32 = __double2float_rn(hd[u]);
                            I.h32[base + (size_t)(l + u) * n] = h32;
                        }
                        term<KIND, KP>(hd[u], h32, xrow, a64, a32, e32);
                    }
                }
            }
            for (; l < lc; ++l) {
                const double *xrow = sm.xs + l * XD;
                const size_t off = base + (size_t)l * n;
                if (KIND == kF32) {
                    term<KIND, KP>(0.0, I.h32[off], xrow, a64, a32, e32);
                } else {
                    const double h = __ldg(I.H + off);
                    if (rowsum) rs += fabs(h);
                    float h32 = 0.0f;
                    if (KIND == kF32First) {
                        h32 = __double2float_rn(h);
                        I.h32[off] = h32;
                    }
                    term<KIND, KP>(h, h32, xrow, a64, a32, e32);
                }
            }
        }
        if (row) {
            double *yr = I.y + (size_t)i * k;
#pragma unroll
            for (int j = 0; j < KP; ++j) {
                if (j < k) {
                    if (KIND == kF64) {
                        yr[j] = a64[j];
                    } else if (KIND == kDF) {
                        yr[j] = (double)a32[j] + (double)e32[j];
                    } else {
                        yr[j] = (double)a32[j];
                    }
                }
            }
            hinf = fmax(hinf, rs);
        }
    }
    return hinf;
}

template <int KIND, int L>
__device__ __forceinline__ double product_kp(const Inst &I, const double *X, Shared<L> &sm, int r0,
                                             int r1, bool rowsum)
{
    switch ((I.k + 3) >> 2) {
    case 1: return product<KIND, 4, L>(I, X, sm, r0, r1, rowsum);
    case 2: return product<KIND, 8, L>(I, X, sm, r0, r1, rowsum);
    case 3: return product<KIND, 12, L>(I, X, sm, r0, r1, rowsum);
    default: return product<KIND, 16, L>(I, X, sm, r0, r1, rowsum);
    }
}

template <int L>
__device__ __forceinline__ double product_any(int kind, const Inst &I, const double *X,
                                              Shared<L> &sm, int r0, int r1, bool rowsum)
{
    switch (kind) {
    case kF64: return product_kp<kF64, L>(I, X, sm, r0, r1, rowsum);
    case kF32First: return product_kp<kF32First, L>(I, X, sm, r0, r1, rowsum);
    case kF32: return product_kp<kF32, L>(I, X, sm, r0, r1, rowsum);
    default: return product_kp<kDF, L>(I, X, sm, r0, r1, rowsum);
    }
}

// Solve instance order[q]: alone (TEAM false, rows [0, n)) or as CTA `rank`
// of a cluster of `team` CTAs (rows in contiguous ranges of a multiple of 32).
template <int L, bool TEAM>
__device__ void solve(const Params &p, int q, Shared<L> &sm, int rank, int team)
{
    const int id = p.order[q];
    const Inst I = p.inst[id];
    const int n = I.n, k = I.k;
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
    // X = the first k unit vectors (own rows)
    for (size_t e = (size_t)r0 * k + tid; e < (size_t)r1 * k; e += blockDim.x) {
        const int i = (int)(e / k);
        const int j = (int)(e - (size_t)i * k);
        I.xa[e] = i == j ? 1.0 : 0.0;
    }
    team_sync();
    double *X = I.xa;
    double *Xn = I.xb;
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
        const int kind = fp64 ? (p.certify_df ? kDF : kF64) : (h32_ready ? kF32 : kF32First);
        const bool first = hinf < 0.0;
        double hs = product_any<L>(kind, I, X, sm, r0, r1, first);
        if (kind == kF32First) h32_ready = true;
        if (first) {
            hs = warp_max_d(hs);
            if (lane == 0) sm.red[warp][kHinf] = hs;
        }
        team_sync();  // Y rows of every CTA written
        if (tid < k) sm.lam[tid] = __ldcg(I.y + (size_t)tid * k + tid);
        __syncthreads();
        // residuals r = Y - X diag(lambda), update X' = X + r / (d_j - d_i), norms
        double fp_dx = 0.0, fp_x = 0.0;
        for (int rb = r0; rb < r1; rb += blockDim.x) {
            const int i = rb + tid;
            const bool row = i < r1;
            const double di = row ? I.H[(size_t)i * n + i] : 0.0;
            for (int j = 0; j < k; ++j) {
                double rr = 0.0, xx = 0.0, xy = 0.0;
                if (row) {
                    const size_t e = (size_t)i * k + j;
                    const double x = X[e];
                    const double yv = I.y[e];
                    const double r = yv - sm.lam[j] * x;
                    xy = x * yv;
                    if (i != j) {
                        const double dx = r / (I.H[(size_t)j * n + j] - di);
                        Xn[e] = x + dx;
                        fp_dx += dx * dx;
                        rr = r * r;
                    } else {
                        Xn[e] = 1.0;
                    }
                    xx = x * x;
                    fp_x += xx;
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
        fp_dx = warp_sum_d(fp_dx);
        fp_x = warp_sum_d(fp_x);
        if (lane == 0) {
            sm.red[warp][kDx] += fp_dx;
            sm.red[warp][kXx] += fp_x;
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
        } else {
            const double fp = sqrt(sm.tot[kDx]) / sqrt(fmax(sm.tot[kXx], 1e-300));
            if (!isfinite(fp)) {
                // the low-precision sweeps diverged: certify from the unit vectors
                for (size_t e = (size_t)r0 * k + tid; e < (size_t)r1 * k; e += blockDim.x) {
                    const int i = (int)(e / k);
                    Xn[e] = i == (int)(e - (size_t)i * k) ? 1.0 : 0.0;
                }
                if (TEAM) team_sync();  // every CTA's rows reset before the next product
                fp64 = true;
            } else if (fp <= p.lowp_tol || it + 1 >= p.lowp_maxiter) {
                fp64 = true;
            }
        }
        if (!done) {
            double *t = X;
            X = Xn;
            Xn = t;
            if (fp64 && it64 >= p.maxiter) {
                ++it;
                break;
            }
        }
    }
    __syncthreads();
    // outputs: the certified block (own rows), column-major, and its Ritz values
    for (size_t e = (size_t)r0 * k + tid; e < (size_t)r1 * k; e += blockDim.x) {
        const int i = (int)(e / k);
        const int j = (int)(e - (size_t)i * k);
        I.vectors[(size_t)j * n + i] = X[e];
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
__global__ void __launch_bounds__(512)
batch_ipt_kernel(Params p)
{
    __shared__ __align__(16) Shared<L> sm;
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
                solve<L, true>(p, q, sm, rank, p.team);
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
        solve<L, false>(p, q, sm, 0, 1);
    }
}

}  // namespace batch

// ---------------------------------------------------------------------------
// Plan: device instance table, scratch pool, autotuned launch shape, graph.
// ---------------------------------------------------------------------------
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
                &per_sm, batch::batch_ipt_kernel<64>, threads, 0));
        } else {
            IPTGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per_sm, batch::batch_ipt_kernel<128>, threads, 0));
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
        pool += 3 * (size_t)x.n * x.k;
        // FP32 copy of H for the FP32 sweeps, 16-byte aligned per instance
        if (mixed) pool32 += ((size_t)x.n * x.n + 3) & ~(size_t)3;
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
            const size_t nk = (size_t)x.n * x.k;
            I.xa = P->pool + off;
            I.xb = I.xa + nk;
            I.y = I.xb + nk;
            off += 3 * nk;
            I.h32 = nullptr;
            if (mixed) {
                I.h32 = P->pool32 + off32;
                off32 += ((size_t)x.n * x.n + 3) & ~(size_t)3;
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
