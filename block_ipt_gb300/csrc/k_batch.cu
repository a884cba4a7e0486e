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
// Mixed precision: the sweeps first run the product in FP32 (H converted on
// load, X staged in FP32, FP32 accumulation) until the fixed-point residual
// ||X' - X||_F / ||X||_F reaches lowp_tol, then switch to FP64-accurate
// sweeps, which certify and refine the block (the reference's mixed scheme:
// low-precision IPT, then FP64 IPT; IPT_C_GPU/src/mixed_precision/
// ipt_mixed_precision_cuda.cu:1153-1225).  Those run on the FP64 pipe or, by
// default after FP32 sweeps, in double-float arithmetic on the FP32 pipe:
// every H entry split once into an exact (hi, lo) float pair on the integer
// pipe, X staged as (hi, lo) pairs, each term accumulated by an exact
// two-product and two-sum (12 FP32 operations, about 2^-48 relative), so
// that a sweep costs about a fifth of its FP64-pipe time on GB300, whose
// FP64 pipe retires 1/64 of the FP32 rate.
//
// Scheduling: one CTA per instance at a time; CTAs take instances from a
// device counter in descending order of cost n^2 k (longest first), so the
// batch ends when the largest instances end.  Within a CTA, a thread owns
// one row and all k <= 16 columns of Y; columns of H stream in L-row chunks
// (coalesced, column-major), with the matching X chunk staged in shared
// memory.  No host synchronisation inside the batch, so the whole solve is
// one graph launch.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "dfloat.cuh"
#include "reduce.cuh"

#define IPT_API extern "C" __attribute__((visibility("default")))

namespace iptgb {
namespace batch {

constexpr int kKMax = 16;

struct Inst {
    const double *H;
    double *vectors;  // output n x k column-major
    double *values;   // output k
    double *xa;       // scratch, row-major n x k
    double *xb;
    double *y;
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
    int *counter;
    Out *out;
    int mixed;
    int certify_df;  // FP64-accurate sweeps in double-float (FP32 pipe)
    double tol;
    int maxiter;
    int lowp_maxiter;
    double lowp_tol;
};

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Y = H X for one instance (rows strided over the block), T the arithmetic
// type.  With `rowsum`, also returns the largest absolute row sum of H.
template <typename T, int L>
__device__ double product(const Inst &I, const double *__restrict__ X, T *xs, bool rowsum)
{
    const int n = I.n, k = I.k;
    const int tid = threadIdx.x;
    double hinf = 0.0;
    for (int rb = 0; rb < n; rb += blockDim.x) {
        const int i = rb + tid;
        T acc[kKMax];
#pragma unroll
        for (int j = 0; j < kKMax; ++j) acc[j] = T(0);
        double rs = 0.0;
        for (int l0 = 0; l0 < n; l0 += L) {
            const int lc = min(L, n - l0);
            __syncthreads();
            for (int e = tid; e < L * kKMax; e += blockDim.x) {
                const int l = e / kKMax;
                const int j = e - l * kKMax;
                xs[e] = (l < lc && j < k) ? (T)X[(size_t)(l0 + l) * k + j] : T(0);
            }
            __syncthreads();
            if (i < n) {
                const double *hc = I.H + (size_t)l0 * n + i;
                for (int l = 0; l < lc; ++l) {
                    const double hd = hc[(size_t)l * n];
                    if (rowsum) rs += fabs(hd);
                    const T h = (T)hd;
                    const T *xr = xs + l * kKMax;
#pragma unroll
                    for (int j = 0; j < kKMax; ++j) acc[j] = fma(h, xr[j], acc[j]);
                }
            }
        }
        if (i < n) {
#pragma unroll
            for (int j = 0; j < kKMax; ++j) {
                if (j < k) I.y[(size_t)i * k + j] = (double)acc[j];
            }
            hinf = fmax(hinf, rs);
        }
    }
    return hinf;
}

// Y = H X in double-float arithmetic (see the file header); with `rowsum`,
// also the largest absolute row sum of H.
template <int L>
__device__ double product_df(const Inst &I, const double *__restrict__ X, float2 *xs, bool rowsum)
{
    const int n = I.n, k = I.k;
    const int tid = threadIdx.x;
    double hinf = 0.0;
    for (int rb = 0; rb < n; rb += blockDim.x) {
        const int i = rb + tid;
        float S[kKMax], e[kKMax];
#pragma unroll
        for (int j = 0; j < kKMax; ++j) {
            S[j] = 0.0f;
            e[j] = 0.0f;
        }
        double rs = 0.0;
        for (int l0 = 0; l0 < n; l0 += L) {
            const int lc = min(L, n - l0);
            __syncthreads();
            for (int q = tid; q < L * kKMax; q += blockDim.x) {
                const int l = q / kKMax;
                const int j = q - l * kKMax;
                float2 v = make_float2(0.0f, 0.0f);
                if (l < lc && j < k) {
                    const dfloat d = df_from_double(X[(size_t)(l0 + l) * k + j]);
                    v = make_float2(d.hi, d.lo);
                }
                xs[q] = v;
            }
            __syncthreads();
            if (i < n) {
                const double *hc = I.H + (size_t)l0 * n + i;
                for (int l = 0; l < lc; ++l) {
                    const double hd = hc[(size_t)l * n];
                    if (rowsum) rs += fabs(hd);
                    const dfloat h = df_from_double(hd);
                    const float2 *xr = xs + l * kKMax;
#pragma unroll
                    for (int j = 0; j < kKMax; ++j) df_acc(S[j], e[j], h.hi, h.lo, xr[j].x, xr[j].y);
                }
            }
        }
        if (i < n) {
#pragma unroll
            for (int j = 0; j < kKMax; ++j) {
                if (j < k) I.y[(size_t)i * k + j] = (double)S[j] + (double)e[j];
            }
            hinf = fmax(hinf, rs);
        }
    }
    return hinf;
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

template <int L>
__global__ void __launch_bounds__(512)
batch_ipt_kernel(Params p)
{
    __shared__ __align__(16) double xs64[L * kKMax];
    // per-column sums of r^2, x^2, x.y, then |X' - X|^2, |X|^2, max row sum
    __shared__ double sums[3 * kKMax + 3];
    __shared__ double lam[kKMax];
    __shared__ int cur;
    float *xs32 = reinterpret_cast<float *>(xs64);
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    for (;;) {
        __syncthreads();
        if (tid == 0) cur = atomicAdd(p.counter, 1);
        __syncthreads();
        const int q = cur;
        if (q >= p.count) return;
        const int id = p.order[q];
        const Inst I = p.inst[id];
        const int n = I.n, k = I.k;
        Out o{};
        if (tid == 0) o.t_start = global_ns();
        // X = the first k unit vectors
        for (size_t e = tid; e < (size_t)n * k; e += blockDim.x) {
            const int i = (int)(e / k);
            const int j = (int)(e - (size_t)i * k);
            I.xa[e] = i == j ? 1.0 : 0.0;
        }
        double *X = I.xa;
        double *Xn = I.xb;
        bool fp64 = !p.mixed;
        double hinf = -1.0;
        int it = 0, it64 = 0;
        bool done = false;
        int status = 0;
        double maxres = INFINITY;
        const int limit = p.maxiter + (p.mixed ? p.lowp_maxiter : 0);
        for (; it < limit && !done; ++it) {
            __syncthreads();
            if (tid < 3 * kKMax + 3) sums[tid] = 0.0;
            double hs;
            if (fp64 && p.certify_df) {
                hs = product_df<L>(I, X, reinterpret_cast<float2 *>(xs64), hinf < 0.0);
            } else if (fp64) {
                hs = product<double, L>(I, X, xs64, hinf < 0.0);
            } else {
                hs = product<float, L>(I, X, xs32, hinf < 0.0);
            }
            if (hinf < 0.0) {
                hs = warp_max_d(hs);
                // non-negative doubles order like their bit patterns
                if (lane == 0) {
                    atomicMax((unsigned long long *)&sums[3 * kKMax + 2],
                              (unsigned long long)__double_as_longlong(hs));
                }
            }
            __syncthreads();
            if (hinf < 0.0) hinf = sums[3 * kKMax + 2];
            if (tid < k) lam[tid] = I.y[(size_t)tid * k + tid];
            __syncthreads();
            // residuals r = Y - X diag(lambda), update X' = X + r / (d_j - d_i), norms
            double fp_dx = 0.0, fp_x = 0.0;
            for (int rb = 0; rb < n; rb += blockDim.x) {
                const int i = rb + tid;
                const bool row = i < n;
                const double di = row ? I.H[(size_t)i * n + i] : 0.0;
                for (int j = 0; j < k; ++j) {
                    double rr = 0.0, xx = 0.0, xy = 0.0;
                    if (row) {
                        const size_t e = (size_t)i * k + j;
                        const double x = X[e];
                        const double yv = I.y[e];
                        const double r = yv - lam[j] * x;
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
                        atomicAdd(&sums[j], rr);
                        atomicAdd(&sums[kKMax + j], xx);
                        atomicAdd(&sums[2 * kKMax + j], xy);
                    }
                }
            }
            fp_dx = warp_sum_d(fp_dx);
            fp_x = warp_sum_d(fp_x);
            if (lane == 0) {
                atomicAdd(&sums[3 * kKMax], fp_dx);
                atomicAdd(&sums[3 * kKMax + 1], fp_x);
            }
            __syncthreads();
            if (fp64) {
                ++it64;
                double mx = 0.0;
                bool finite = true;
                for (int j = 0; j < k; ++j) {
                    const double sc = sqrt(sums[j]) /
                                      (fmax(1.0, hinf) * fmax(1.0, sqrt(sums[kKMax + j])));
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
                const double fp = sqrt(sums[3 * kKMax]) / sqrt(fmax(sums[3 * kKMax + 1], 1e-300));
                if (!isfinite(fp)) {
                    // the low-precision sweeps diverged: certify from the unit vectors
                    for (size_t e = tid; e < (size_t)n * k; e += blockDim.x) {
                        const int i = (int)(e / k);
                        Xn[e] = i == (int)(e - (size_t)i * k) ? 1.0 : 0.0;
                    }
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
        // outputs: the certified block, column-major, and its Ritz values
        for (size_t e = tid; e < (size_t)n * k; e += blockDim.x) {
            const int j = (int)(e / n);
            const int i = (int)(e - (size_t)j * n);
            I.vectors[e] = X[(size_t)i * k + j];
        }
        // Rayleigh quotients of the returned block (sums hold its last sweep)
        if (tid < k) I.values[tid] = sums[2 * kKMax + tid] / sums[kKMax + tid];
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

}  // namespace batch

// ---------------------------------------------------------------------------
// Plan: device instance table, scratch pool, autotuned launch shape, graph.
// ---------------------------------------------------------------------------
struct BatchPlan {
    int count = 0;
    std::vector<batch::Inst> host_inst;
    batch::Inst *inst = nullptr;
    int *order = nullptr;
    int *counter = nullptr;
    batch::Out *out = nullptr;
    double *pool = nullptr;
    int mixed = 0;
    int certify_df = 0;
    double tol = 1e-8;
    int maxiter = 100;
    int lowp_maxiter = 200;
    double lowp_tol = 1e-6;
    int threads = 512;
    int chunk = 128;
    int ctas = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;

    int launch(cudaStream_t s)
    {
        batch::Params p{inst, order, count, counter, out, mixed, certify_df, tol, maxiter,
                        lowp_maxiter, lowp_tol};
        IPTGB_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), s));
        if (chunk == 64) {
            batch::batch_ipt_kernel<64><<<ctas, threads, 0, s>>>(p);
        } else {
            batch::batch_ipt_kernel<128><<<ctas, threads, 0, s>>>(p);
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
    }
};

int batch_ctas(int threads)
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch::batch_ipt_kernel<128>, threads,
                                                  0);
    return std::max(1, sms * std::max(1, per_sm));
}

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
    size_t pool = 0;
    for (int b = 0; b < count; ++b) {
        const IPTBatchInstance &x = instances[b];
        if (x.H == nullptr || x.vectors == nullptr || x.values == nullptr || x.n <= 0 ||
            x.k <= 0 || x.k > batch::kKMax || x.k > x.n) {
            return IPT_CUDA_INVALID_ARGUMENT;
        }
        pool += 3 * (size_t)x.n * x.k;
    }
    auto *P = new BatchPlan();
    P->count = count;
    P->mixed = opt.precision == IPT_BLOCK_FP32 ? 1 : 0;
    P->certify_df = opt.certify_precision == IPT_BLOCK_DF64 ||
                    (opt.certify_precision == -1 && P->mixed);
    P->tol = opt.residual_tol;
    P->maxiter = opt.maxiter;
    P->lowp_maxiter = opt.lowp_maxiter;
    P->lowp_tol = opt.lowp_tol;
    P->threads = opt.threads != 0 ? opt.threads : 512;
    P->chunk = opt.chunk != 0 ? opt.chunk : 128;
    int st = IPT_CUDA_SUCCESS;
    if (cudaMalloc((void **)&P->pool, pool * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void **)&P->inst, count * sizeof(batch::Inst)) != cudaSuccess ||
        cudaMalloc((void **)&P->order, count * sizeof(int)) != cudaSuccess ||
        cudaMalloc((void **)&P->counter, sizeof(int)) != cudaSuccess ||
        cudaMalloc((void **)&P->out, count * sizeof(batch::Out)) != cudaSuccess) {
        st = IPT_CUDA_ALLOCATION_FAILED;
    }
    if (st == IPT_CUDA_SUCCESS) {
        P->host_inst.resize(count);
        size_t off = 0;
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
        }
        // longest (n^2 k) first
        std::vector<int> order(count);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            const double ca = (double)instances[a].n * instances[a].n * instances[a].k;
            const double cb = (double)instances[b].n * instances[b].n * instances[b].k;
            return ca > cb;
        });
        if (cudaMemcpy(P->inst, P->host_inst.data(), count * sizeof(batch::Inst),
                       cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(P->order, order.data(), count * sizeof(int), cudaMemcpyHostToDevice) !=
                cudaSuccess) {
            st = IPT_CUDA_CUDA_ERROR;
        }
    }
    if (st == IPT_CUDA_SUCCESS) {
        P->ctas = std::min(count, batch_ctas(P->threads));
        st = P->capture(nullptr);
    }
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
    double best = INFINITY;
    int bt = P->threads, bc = P->chunk;
    int st = IPT_CUDA_SUCCESS;
    for (int ti = 0; ti < 3 && st == IPT_CUDA_SUCCESS; ++ti) {
        for (int ci = 0; ci < 2 && st == IPT_CUDA_SUCCESS; ++ci) {
            P->threads = cand_threads[ti];
            P->chunk = cand_chunk[ci];
            P->ctas = std::min(P->count, batch_ctas(P->threads));
            st = P->launch(s);  // warm-up of this shape
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
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    P->threads = bt;
    P->chunk = bc;
    P->ctas = std::min(P->count, batch_ctas(P->threads));
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

IPT_API int ipt_block_batch_plan_destroy(void *plan)
{
    delete static_cast<BatchPlan *>(plan);
    return IPT_CUDA_SUCCESS;
}
