// block_api.cu - FP64 operators/stages and the exported block-solver API
// (include/ipt_block.h), plus the reference's IPT_BLOCK_CLUSTER sparse path.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "block_solver.h"
#include "cluster.h"
#include "common.cuh"
#include "fpconv.cuh"
#include "ipt_plain.h"
#include "lowp.h"
#include "oz_product.h"
#include "prep.h"
#include "reduce.cuh"

#define IPT_API extern "C" __attribute__((visibility("default")))

namespace iptgb {

// ---------------------------------------------------------------------------
// FP64 accurate products
// ---------------------------------------------------------------------------
struct DenseApply final : Fp64Apply {
    const double *H = nullptr;
    // optional split-operand product on the tensor cores (k_oz.cu), the
    // default of the mixed solve
    OzProduct *oz = nullptr;
    // optional double-FP32 copy of H: products in double-float arithmetic on
    // the FP32 pipe (k_df64.cu) instead of FP64 FMAs
    const float *Hh = nullptr;
    const float *Hl = nullptr;
    int n = 0;
    int sms = 148;
    cudaStream_t s = nullptr;
    DeviceBuffer<double> P;
    DeviceBuffer<float> Xs;
    int apply(const double *V, int c, double *AV) override
    {
        if (oz != nullptr) {
            KernelTimerScope timer(kProfFp64Product, s);
            return oz->apply(V, n, c, AV, n);
        }
        const int S = Hh != nullptr ? df64_split_for(n, c, sms) : dense64_split_for(n, c, sms);
        const size_t need = (size_t)S * (size_t)n * (size_t)c;
        if (P.count < need) {
            IPTGB_CHECK(P.alloc(need, s));
        }
        {
            KernelTimerScope timer(kProfFp64Product, s);
            if (Hh != nullptr) {
                const size_t nc = (size_t)n * c;
                if (Xs.count < 2 * nc) IPTGB_CHECK(Xs.alloc(2 * nc, s));
                IPTGB_CHECK(launch_df_split(V, nc, Xs.ptr, Xs.ptr + nc, s));
                IPTGB_CHECK(launch_df64_partial(Hh, Hl, n, n, Xs.ptr, Xs.ptr + nc, n, c, P.ptr, S,
                                                s));
            } else {
                IPTGB_CHECK(launch_dense64_partial(H, n, n, V, n, c, P.ptr, S, s));
            }
        }
        KernelTimerScope timer(kProfFp64Update, s);
        if (Hh != nullptr) return launch_df_sum_partials(P.ptr, S, (size_t)n * c, AV, s);
        return launch_sum_partials(P.ptr, S, (size_t)n * c, AV, s);
    }
};

struct CsrApply final : Fp64Apply {
    const int *row_ptr = nullptr;
    const int *col_ind = nullptr;
    const double *vals = nullptr;
    int n = 0;
    int nnz = 0;
    cudaStream_t s = nullptr;
    // double-float products (with the Davidson products' policy): the values
    // split into (hi, lo) floats at the first product
    bool df = false;
    DeviceBuffer<float> vsplit;
    int apply(const double *V, int c, double *AV) override
    {
        KernelTimerScope timer(kProfCsrProduct, s);
        if (df && nnz > 0) {
            if (vsplit.ptr == nullptr) {
                IPTGB_CHECK(vsplit.alloc(2 * (size_t)nnz, s));
                IPTGB_CHECK(launch_df_split(vals, (size_t)nnz, vsplit.ptr, vsplit.ptr + nnz, s));
            }
            return launch_csr_df_spmm(row_ptr, col_ind, vsplit.ptr, vsplit.ptr + nnz, n, V, c,
                                      AV, s);
        }
        return launch_csr64_spmm(row_ptr, col_ind, vals, n, V, c, AV, s);
    }
};

// ---------------------------------------------------------------------------
// FP64 IPT stage on a plain operator.  Stops at ipt_tol, at maxiter, or when
// the fixed-point residual stops decreasing (the block is then handed to
// Rayleigh-Ritz as it is; a non-finite step is rolled back).
// ---------------------------------------------------------------------------
struct Fp64Stage final : IptStage {
    std::unique_ptr<Fp64Operator> op;
    DenseFp64Operator *dense = nullptr;
    CsrFp64Operator *csr = nullptr;
    const double *d = nullptr;
    int n = 0;
    int sms = 148;
    cudaStream_t s = nullptr;
    DeviceBuffer<double> P, Y, Xb;

    int run(int p, int maxiter, double tol, int check_every, double *X, int *iterations,
            double *fpres_out, long long *matvecs) override
    {
        const size_t elems = (size_t)n * (size_t)p;
        if (dense != nullptr) {
            dense->k = p;
            dense->S = dense64_split_for(n, p, sms);
            IPTGB_CHECK(P.alloc((size_t)dense->S * elems, s));
            dense->P = P.ptr;
        } else {
            csr->k = p;
            IPTGB_CHECK(Y.alloc(elems, s));
            csr->Y = Y.ptr;
        }
        IPTGB_CHECK(Xb.alloc(elems, s));
        SolveScratch scratch;
        IPTGB_CHECK(scratch.init(elems, s));
        IPTGB_CHECK(launch_set_identity(X, n, p, s));
        double *x = X;
        double *y = Xb.ptr;
        double best = INFINITY;
        int worse = 0;
        int done = 0;
        double fpres = NAN;
        int status = IPT_CUDA_SUCCESS;
        for (int it = 0; it < maxiter; ++it) {
            // the first kFirstChecks steps are always checked, so a map that
            // diverges from the start stops after the same few steps whatever
            // check_every is (a diverged block would reach Rayleigh-Ritz as
            // non-finite columns, and the identity restart is a worse start)
            constexpr int kFirstChecks = 4;
            const int want = it < kFirstChecks || ((it + 1) % check_every == 0) ||
                             it + 1 == maxiter;
            status = op->step(x, y, d, want, &scratch.ns);
            if (status != IPT_CUDA_SUCCESS) break;
            done = it + 1;
            if (want) {
                if (cudaMemcpyAsync(scratch.host_norms, scratch.ns.norms, 2 * sizeof(double),
                                    cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                    cudaStreamSynchronize(s) != cudaSuccess) {
                    status = IPT_CUDA_CUDA_ERROR;
                    break;
                }
                const double r = scratch.host_norms[0] / scratch.host_norms[1];
                if (!isfinite(r)) {
                    break;  // keep x (the last finite block)
                }
                fpres = r;
                std::swap(x, y);
                if (r <= tol) break;
                if (r < best) {
                    best = r;
                    worse = 0;
                } else if (++worse >= 3) {
                    break;
                }
            } else {
                std::swap(x, y);
            }
        }
        scratch.release(s);
        if (status != IPT_CUDA_SUCCESS) return status;
        if (x != X) {
            IPTGB_CUDA(cudaMemcpyAsync(X, x, elems * sizeof(double), cudaMemcpyDeviceToDevice, s));
        }
        *iterations = done;
        *fpres_out = fpres;
        *matvecs = (long long)done * p;
        return IPT_CUDA_SUCCESS;
    }
};

IptStage *make_fp64_dense_stage(const double *dH, int n, const double *d, cudaStream_t stream)
{
    auto *st = new Fp64Stage();
    auto *op = new DenseFp64Operator();
    op->H = dH;
    op->ldh = n;
    op->n = n;
    op->stream = stream;
    st->op.reset(op);
    st->dense = op;
    st->d = d;
    st->n = n;
    st->sms = device_sm_count();
    st->s = stream;
    return st;
}

IptStage *make_fp64_csr_stage(const int *row_ptr, const int *col_ind, const double *vals, int n,
                              const double *d, cudaStream_t stream)
{
    auto *st = new Fp64Stage();
    auto *op = new CsrFp64Operator();
    op->row_ptr = row_ptr;
    op->col_ind = col_ind;
    op->vals = vals;
    op->n = n;
    op->stream = stream;
    st->op.reset(op);
    st->csr = op;
    st->d = d;
    st->n = n;
    st->sms = device_sm_count();
    st->s = stream;
    return st;
}

// ---------------------------------------------------------------------------
// Statistics of a dense symmetric H from one streaming pass: the diagonal,
// the largest row sum of |H| (hnorm; a column sum, H being symmetric, in
// double-float arithmetic on the FP32 pipe, about 1e-14 relative), the
// largest off-diagonal |H_il| (the low-precision copy's scale) and the number
// of descents d_{i+1} < d_i (zero: the diagonal is already ascending and no
// permutation is needed).  One warp per column reads the contiguous column;
// one 24-byte read brings the results to the host.
// ---------------------------------------------------------------------------
constexpr int kStatsWarps = 8;

// One entry of the statistics: |h| added to the double-float column sum
// (S, C) on the FP32 pipe (|h| = |hi| + sgn(hi) lo exactly, hi/lo from the
// integer-pipe split), |h| bits into the off-diagonal maximum (non-negative
// doubles order like their bit patterns).
__device__ __forceinline__ void stats_entry(double h, bool offdiag, float &S, float &C,
                                            unsigned long long &mbits)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(h);
    uint32_t hb, lb;
    float hi, lo;
    if (split_double_bits(b, &hb, &lb)) {
        hi = __uint_as_float(hb);
        lo = __uint_as_float(lb);
    } else {
        hi = __double2float_rn(h);
        lo = __double2float_rn(h - (double)hi);
    }
    const float a = fabsf(hi);
    const float bl = hi < 0.0f ? -lo : lo;
    const float t = __fadd_rn(S, a);
    const float bp = __fsub_rn(t, S);
    const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(t, bp)), __fsub_rn(a, bp));
    S = t;
    C = __fadd_rn(C, __fadd_rn(err, bl));
    const unsigned long long ab = b & 0x7FFFFFFFFFFFFFFFULL;
    if (offdiag && ab > mbits) mbits = ab;
}

// kSums false: no column sums (the low-precision operator's conversion pass
// forms them), only integer work per entry, so the pass runs at HBM speed.
template <bool kSums>
__global__ void __launch_bounds__(32 * kStatsWarps)
    dense_stats_kernel(const double *__restrict__ H, int n, bool vec, double *__restrict__ d,
                       DenseStats *__restrict__ stats)
{
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * kStatsWarps + (threadIdx.x >> 5);
    if (c >= n) return;  // whole warps leave together
    const double *col = H + (size_t)c * n;
    float S = 0.0f, C = 0.0f;
    unsigned long long mbits = 0;
    if (vec) {  // n even and H 16-byte aligned: every column starts 16-byte aligned
        const double2 *col2 = reinterpret_cast<const double2 *>(col);
        const int half = n / 2;
#pragma unroll 4
        for (int q = lane; q < half; q += 32) {
            const double2 v = col2[q];
            const int l = 2 * q;
            if (kSums) {
                stats_entry(v.x, l != c, S, C, mbits);
                stats_entry(v.y, l + 1 != c, S, C, mbits);
            } else {
                const unsigned long long a0 =
                    (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFULL;
                const unsigned long long a1 =
                    (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFULL;
                if (l != c && a0 > mbits) mbits = a0;
                if (l + 1 != c && a1 > mbits) mbits = a1;
            }
        }
    } else {
#pragma unroll 4
        for (int l = lane; l < n; l += 32) {
            if (kSums) {
                stats_entry(col[l], l != c, S, C, mbits);
            } else {
                const unsigned long long a =
                    (unsigned long long)__double_as_longlong(col[l]) & 0x7FFFFFFFFFFFFFFFULL;
                if (l != c && a > mbits) mbits = a;
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        const float So = __shfl_xor_sync(0xffffffffu, S, off);
        const float Co = __shfl_xor_sync(0xffffffffu, C, off);
        const float t = __fadd_rn(S, So);
        const float bp = __fsub_rn(t, S);
        const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(t, bp)), __fsub_rn(So, bp));
        S = t;
        C = __fadd_rn(__fadd_rn(C, Co), err);
        const unsigned long long mo = __shfl_xor_sync(0xffffffffu, mbits, off);
        if (mo > mbits) mbits = mo;
    }
    if (lane == 0) {
        const size_t dstride = (size_t)n + 1;
        const double dc = H[(size_t)c * dstride];
        d[c] = dc;
        if (c + 1 < n && H[(size_t)(c + 1) * dstride] < dc) {
            atomicAdd(&stats->descents, 1ULL);
        }
        const double sum = (double)S + (double)C;
        if (kSums && sum > 0.0) {
            atomicMax(&stats->hnorm_bits, (unsigned long long)__double_as_longlong(sum));
        }
        if (mbits > 0) atomicMax(&stats->maxabs_bits, mbits);
    }
}

// hnorm from the conversion pass's partial column sums [chunk][column]:
// chunks summed in a fixed order, the maximum over columns.
__global__ void colsum_finish_kernel(const double *__restrict__ part, int chunks, int n,
                                     unsigned long long *__restrict__ hnorm_bits)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double sum = 0.0;
    if (c < n) {
        for (int q = 0; q < chunks; ++q) sum += part[(size_t)q * n + c];
    }
    for (int off = 16; off > 0; off >>= 1) sum = fmax(sum, __shfl_xor_sync(0xffffffffu, sum, off));
    if ((threadIdx.x & 31) == 0 && sum > 0.0) {
        atomicMax(hnorm_bits, (unsigned long long)__double_as_longlong(sum));
    }
}

int dense_hnorm_from_colsums(const double *part, int chunks, int n, cudaStream_t s, double *hnorm)
{
    DeviceBuffer<unsigned long long> bits;
    IPTGB_CHECK(bits.alloc(1, s));
    IPTGB_CUDA(cudaMemsetAsync(bits.ptr, 0, sizeof(unsigned long long), s));
    colsum_finish_kernel<<<blocks_for(n), kThreads, 0, s>>>(part, chunks, n, bits.ptr);
    IPTGB_LAUNCH();
    unsigned long long h = 0;
    IPTGB_CUDA(cudaMemcpyAsync(&h, bits.ptr, sizeof(h), cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    memcpy(hnorm, &h, sizeof(double));
    return IPT_CUDA_SUCCESS;
}

// Diagonal and statistics of H on the stream; returns after the host has them.
// with_sums false leaves *hnorm at 0.
int dense_stats(const double *dH, int n, double *d, cudaStream_t s, double *hnorm,
                double *maxabs_off, unsigned long long *descents, bool with_sums = true)
{
    DeviceBuffer<DenseStats> st;
    IPTGB_CHECK(st.alloc(1, s));
    IPTGB_CUDA(cudaMemsetAsync(st.ptr, 0, sizeof(DenseStats), s));
    const bool vec = (n % 2 == 0) && ((reinterpret_cast<uintptr_t>(dH) & 15) == 0);
    const int grid = (n + kStatsWarps - 1) / kStatsWarps;
    if (with_sums) {
        dense_stats_kernel<true><<<grid, 32 * kStatsWarps, 0, s>>>(dH, n, vec, d, st.ptr);
    } else {
        dense_stats_kernel<false><<<grid, 32 * kStatsWarps, 0, s>>>(dH, n, vec, d, st.ptr);
    }
    IPTGB_LAUNCH();
    DenseStats h;
    IPTGB_CUDA(cudaMemcpyAsync(&h, st.ptr, sizeof(h), cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    memcpy(hnorm, &h.hnorm_bits, sizeof(double));
    memcpy(maxabs_off, &h.maxabs_bits, sizeof(double));
    *descents = h.descents;
    return IPT_CUDA_SUCCESS;
}

__global__ void csr_row_abs_sum_kernel(const int *row_ptr, const double *vals, int n, double *rs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
        s += fabs(vals[p]);
    }
    rs[i] = s;
}

// Dense symmetric permutation: out[i, j] = H[perm[i], perm[j]].
__global__ void dense_permute_kernel(const double *__restrict__ H, const int *__restrict__ perm,
                                     int n, double *__restrict__ out)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n * n) return;
    const int i = (int)(e % (size_t)n);
    const int j = (int)(e / (size_t)n);
    out[e] = H[(size_t)perm[i] + (size_t)perm[j] * n];
}

// out[perm[i], c] = in[i, c].
__global__ void unpermute_rows_kernel(const double *__restrict__ in, const int *__restrict__ perm,
                                      int n, int k, double *__restrict__ out)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n * k) return;
    const int i = (int)(e % (size_t)n);
    const int c = (int)(e / (size_t)n);
    out[(size_t)perm[i] + (size_t)c * n] = in[e];
}

namespace {

int max_of_device(const double *v, int n, cudaStream_t s, double *out)
{
    std::vector<double> h((size_t)n);
    IPTGB_CUDA(cudaMemcpyAsync(h.data(), v, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    double m = 0.0;
    for (double x : h) m = std::max(m, x);
    *out = m;
    return IPT_CUDA_SUCCESS;
}

bool options_valid(const IPTBlockOptions *o)
{
    return o->ipt_precision >= IPT_BLOCK_FP64 && o->ipt_precision <= IPT_BLOCK_TF32 &&
           o->ipt_maxiter >= 0 && o->davidson_maxsteps >= 0 &&
           (o->preconditioner == IPT_BLOCK_PRECOND_DIAGONAL ||
            (o->preconditioner == IPT_BLOCK_PRECOND_MLP && o->mlp_params != nullptr));
}

}  // namespace

// host_src (optional): a device-accessible pointer to H in pinned host
// memory; dH_in is then an uninitialised device buffer that the solve fills.
// The mixed solve's setup reads only the upper triangle of the host copy
// (H is symmetric), in column chunks that cross the host link while the
// setup pass of the chunks already there runs beside them.
int dense_block_device(const double *dH_in, int n, int k, const IPTBlockOptions *options,
                       double *d_vectors, double *d_values, IPTBlockReport *report,
                       const double *host_src = nullptr)
{
    IPTBlockOptions opt;
    if (options != nullptr) {
        opt = *options;
    } else {
        fill_default_options(&opt);
    }
    IPTBlockReport local;
    if (report == nullptr) report = &local;
    memset(report, 0, sizeof(*report));
    if (dH_in == nullptr || d_vectors == nullptr || d_values == nullptr || n <= 0 || k <= 0 ||
        k > n || !options_valid(&opt)) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)opt.stream;
    DeviceBuffer<double> d, Hp, Xtmp;
    DeviceBuffer<int> dperm;
    trace_mark("dense:start", s);
    IPTGB_CHECK(d.alloc((size_t)n, s));
    const bool lowp_mode = opt.ipt_precision != IPT_BLOCK_FP64;
    const int kind = opt.ipt_precision == IPT_BLOCK_FP16 ? kLowpF16
                     : opt.ipt_precision == IPT_BLOCK_BF16 ? kLowpBF16
                                                           : kLowpTF32;
    double hnorm = 0.0, maxabs_off = 0.0;
    unsigned long long descents = 0;
    // The mixed-precision solve forms its FP64-accurate products on the
    // tensor cores from digit slices of Delta (one split per solve, k_oz.cu);
    // tuning knob IPT_GB300_ACCURATE_PRODUCT = df selects double-FP32
    // arithmetic on the FP32 pipe instead, fp64 (or IPT_GB300_FP64_DFMA=1)
    // FP64 FMAs.  The plain FP64 path keeps FP64 FMAs throughout.
    const char *ap = getenv("IPT_GB300_ACCURATE_PRODUCT");
    const bool want_fp64 = env_flag("IPT_GB300_FP64_DFMA", 0) ||
                           (ap != nullptr && strcmp(ap, "fp64") == 0);
    const bool want_df = ap != nullptr && strcmp(ap, "df") == 0;
    const bool use_oz = lowp_mode && !want_fp64 && !want_df;
    DeviceBuffer<float> Hsplit;
    OzDelta ozd;
    OzProduct ozp;
    const size_t mat = (size_t)n * n;
    if (lowp_mode && want_df) {
        IPTGB_CHECK(Hsplit.alloc(2 * mat, s));
    }
    if (use_oz) {
        IPTGB_CHECK(ozd.init_storage(n, s));
    }
    std::unique_ptr<LowpDenseOperator> lowp;
    int st = IPT_CUDA_SUCCESS;
    // Mixed solve, n <= kFusedSetupMaxN: one fused pass builds Delta (row
    // scales of its own), the split, the diagonal and the statistics straight
    // from H (or from the host copy); an unsorted diagonal falls back to the
    // permuted path below.  Tuning knob IPT_GB300_FUSED_SETUP=0 disables it.
    bool fused = false, have_device_copy = host_src == nullptr;
    if (lowp_mode && n <= kFusedSetupMaxN && env_int("IPT_GB300_FUSED_SETUP", 1) != 0) {
        DeviceBuffer<DenseStats> stats;
        IPTGB_CHECK(stats.alloc(1, s));
        IPTGB_CUDA(cudaMemsetAsync(stats.ptr, 0, sizeof(DenseStats), s));
        LowpDenseSetup su;
        su.symmetric = true;
        su.split_hi = Hsplit.ptr;
        su.split_lo = Hsplit.ptr ? Hsplit.ptr + mat : nullptr;
        // from pinned host memory only the upper triangle crosses the host
        // link (H is symmetric); the pass mirrors it into the device copy
        // (an 8-byte aligned host copy; otherwise the pass reads all of H
        // from it)
        const bool upper = host_src != nullptr &&
                           (reinterpret_cast<uintptr_t>(host_src) & 7) == 0;
        su.fused_src = host_src != nullptr && !upper ? host_src : dH_in;
        su.fused_copy = host_src != nullptr ? const_cast<double *>(dH_in) : nullptr;
        su.upper_host = upper ? host_src : nullptr;
        su.diag = d.ptr;
        su.stats = stats.ptr;
        if (use_oz) {
            su.oz = ozd.A.ptr;
            su.oz_rowexp = ozd.rowexp.ptr;
        }
        lowp.reset(make_lowp_dense_operator(dH_in, n, kind, s, &st, &su));
        if (lowp == nullptr) {
            return st != IPT_CUDA_SUCCESS ? st : IPT_CUDA_INVALID_ARGUMENT;
        }
        if (su.fused_done) {
            have_device_copy = true;
            DenseStats h;
            IPTGB_CUDA(cudaMemcpyAsync(&h, stats.ptr, sizeof(h), cudaMemcpyDeviceToHost, s));
            IPTGB_CUDA(cudaStreamSynchronize(s));
            memcpy(&hnorm, &h.hnorm_bits, sizeof(double));
            memcpy(&maxabs_off, &h.maxabs_bits, sizeof(double));
            descents = h.descents;
            fused = descents == 0;
        }
        if (!fused) lowp.reset();
    }
    if (!have_device_copy) {
        IPTGB_CUDA(cudaMemcpyAsync(const_cast<double *>(dH_in), host_src, mat * sizeof(double),
                                   cudaMemcpyDefault, s));
    }
    if (!fused) {
        // one pass: diagonal, max off-diagonal, sortedness of the diagonal, and
        // (plain FP64 solve) hnorm; the mixed solve's conversion pass forms the
        // column sums for hnorm itself
        IPTGB_CHECK(dense_stats(dH_in, n, d.ptr, s, &hnorm, &maxabs_off, &descents, !lowp_mode));
    }
    trace_mark("dense:stats_done", s);
    const double *dH = dH_in;
    const bool permuted = descents > 0;
    if (permuted) {
        // ascending diagonal order (stable, as the reference's host
        // preparation sorts): permute H symmetrically; the statistics are
        // invariant under the permutation
        std::vector<double> hd((size_t)n);
        IPTGB_CUDA(cudaMemcpyAsync(hd.data(), d.ptr, (size_t)n * sizeof(double),
                                   cudaMemcpyDeviceToHost, s));
        IPTGB_CUDA(cudaStreamSynchronize(s));
        std::vector<int> perm((size_t)n);
        std::iota(perm.begin(), perm.end(), 0);
        std::stable_sort(perm.begin(), perm.end(),
                         [&hd](int a, int b) { return hd[(size_t)a] < hd[(size_t)b]; });
        IPTGB_CHECK(Hp.alloc((size_t)n * n, s));
        IPTGB_CHECK(dperm.alloc((size_t)n, s));
        IPTGB_CUDA(cudaMemcpyAsync(dperm.ptr, perm.data(), (size_t)n * sizeof(int),
                                   cudaMemcpyHostToDevice, s));
        dense_permute_kernel<<<blocks_for((size_t)n * n), kThreads, 0, s>>>(dH_in, dperm.ptr, n,
                                                                           Hp.ptr);
        IPTGB_LAUNCH();
        dH = Hp.ptr;
        IPTGB_CHECK(launch_extract_diagonal(dH, n, n, d.ptr, s));
        IPTGB_CHECK(Xtmp.alloc((size_t)n * k, s));
    }

    DenseApply apply;
    apply.H = dH;
    apply.n = n;
    apply.sms = device_sm_count();
    apply.s = s;
    std::unique_ptr<IptStage> stage;
    if (Hsplit.ptr != nullptr) {
        apply.Hh = Hsplit.ptr;
        apply.Hl = Hsplit.ptr + mat;
    }
    if (use_oz) {
        // the fused pass wrote the slices of the (unpermuted) matrix; any
        // other path splits the matrix the solve iterates on
        if (!fused) IPTGB_CHECK(ozd.split_from(dH, n, s));
        IPTGB_CHECK(ozp.bind(&ozd, d.ptr, s));
        apply.oz = &ozp;
    }
    if (lowp_mode && fused) {
        trace_mark("dense:operator_done", s);
        stage.reset(make_lowp_stage_on(lowp.get(), d.ptr, n, s));
    } else if (lowp_mode) {
        // one pass over H writes the low-precision Delta, the double-FP32
        // split and the partial column sums of |H|
        DeviceBuffer<double> colpart;
        const int chunks = (n + kLowpColsumChunk - 1) / kLowpColsumChunk + 1;
        IPTGB_CHECK(colpart.alloc((size_t)chunks * n, s));
        LowpDenseSetup su;
        su.maxabs = maxabs_off;
        su.symmetric = true;
        su.split_hi = Hsplit.ptr;
        su.split_lo = Hsplit.ptr ? Hsplit.ptr + mat : nullptr;
        su.colsum_part = colpart.ptr;
        lowp.reset(make_lowp_dense_operator(dH, n, kind, s, &st, &su));
        if (lowp == nullptr) {
            return st != IPT_CUDA_SUCCESS ? st : IPT_CUDA_INVALID_ARGUMENT;
        }
        if (Hsplit.ptr != nullptr && !su.split_done) {
            IPTGB_CHECK(launch_df_split(dH, mat, Hsplit.ptr, Hsplit.ptr + mat, s));
        }
        if (su.colsum_chunks > 0 && su.colsum_chunks <= chunks) {
            IPTGB_CHECK(dense_hnorm_from_colsums(colpart.ptr, su.colsum_chunks, n, s, &hnorm));
        } else {
            double m2 = 0.0;
            unsigned long long d2 = 0;
            IPTGB_CHECK(dense_stats(dH, n, d.ptr, s, &hnorm, &m2, &d2, true));
        }
        trace_mark("dense:operator_done", s);
        stage.reset(make_lowp_stage_on(lowp.get(), d.ptr, n, s));
    } else {
        stage.reset(make_fp64_dense_stage(dH, n, d.ptr, s));
    }
    std::unique_ptr<LearnedCorrection> learned;
    DeviceBuffer<double> coupling;
    if (opt.preconditioner == IPT_BLOCK_PRECOND_MLP) {
        learned.reset(make_learned_correction(opt.mlp_params, s));
        IPTGB_CHECK(coupling.alloc((size_t)n, s));
        IPTGB_CHECK(launch_dense_row_coupling(dH, n, coupling.ptr, s));
        learned->bind(coupling.ptr, hnorm);
    }
    double *xout = permuted ? Xtmp.ptr : d_vectors;
    DeviceBuffer<double> Xfb;
    bool done = false;
    if (opt.strategy == IPT_BLOCK_STRATEGY_REFINE && k <= 64) {
        RefineInput rin;
        rin.apply = &apply;
        rin.ipt = lowp_mode ? stage.get() : nullptr;
        rin.lowp = lowp.get();
        rin.d = d.ptr;
        rin.n = n;
        rin.k = k;
        rin.hnorm = hnorm;
        rin.opt = opt;
        rin.max_outer = lowp_mode ? std::min(std::max(1, opt.refine_maxiter), 12)
                                  : std::max(1, opt.refine_maxiter);
        rin.inner_maxiter = std::max(1, opt.inner_maxiter);
        rin.inner_tol = opt.inner_tol > 0.0 ? opt.inner_tol : 3e-3;
        rin.opt.ipt_maxiter = opt.ipt_maxiter;
        if (lowp_mode) {
            // the low-precision IPT stage cannot go below about twice its
            // unit roundoff (FP16 / TF32 2^-11, BF16 2^-8): stop there
            // instead of iterating into stagnation
            const double u = opt.ipt_precision == IPT_BLOCK_BF16 ? 0x1p-8 : 0x1p-11;
            rin.opt.ipt_tol = std::max(opt.ipt_tol, 2.0 * u);
        }
        IPTGB_CHECK(Xfb.alloc((size_t)n * k, s));
        bool conv = false;
        // Anderson mixing in the low-precision iterations of the refinement
        // (lowp.h set_mixing; tuning knob IPT_GB300_ANDERSON=0 turns it off)
        rin.mixing = lowp != nullptr && env_int("IPT_GB300_ANDERSON", 1) != 0;
        if (lowp) lowp->set_mixing(rin.mixing);
        IPTGB_CHECK(refine_solve(rin, xout, d_values, report, s, &conv, Xfb.ptr));
        if (lowp) lowp->set_mixing(false);
        done = conv;
    }
    if (!done) {
        // Davidson (the requested strategy, or the fallback when the IPT
        // fixed point stopped improving: restart from the refined block)
        IPTBlockReport first = *report;
        BlockSolveInput in;
        in.apply = &apply;
        in.ipt = stage.get();
        in.learned = learned.get();
        in.d = d.ptr;
        in.n = n;
        in.k = k;
        in.hnorm = hnorm;
        in.opt = opt;
        in.lowp = lowp_mode;
        if (Xfb.ptr != nullptr) {
            in.initial = Xfb.ptr;
            in.initial_cols = k;
        }
        IPTGB_CHECK(block_solve(in, xout, d_values, report, s));
        if (Xfb.ptr != nullptr) {
            report->ipt_iterations += first.ipt_iterations;
            report->lowp_matvecs += first.lowp_matvecs;
            report->fp64_matvecs += first.fp64_matvecs;
            report->total_ms += first.total_ms;
            report->ipt_ms += first.ipt_ms;
        }
    }
    if (permuted) {
        unpermute_rows_kernel<<<blocks_for((size_t)n * k), kThreads, 0, s>>>(Xtmp.ptr, dperm.ptr,
                                                                              n, k, d_vectors);
        IPTGB_LAUNCH();
    }
    trace_mark("dense:end", s);
    IPTGB_CUDA(cudaStreamSynchronize(s));
    return IPT_CUDA_SUCCESS;
}

int csr_block_device(const int *row_ptr, const int *col_ind, const double *vals, int n, int nnz,
                     int k, const IPTBlockOptions *options, const double *d_diag_sorted,
                     double *d_vectors, double *d_values, IPTBlockReport *report,
                     LearnedCorrection *hook = nullptr, const double *d_initial = nullptr,
                     int initial_cols = 0, OrthStats *orth = nullptr)
{
    IPTBlockOptions opt;
    if (options != nullptr) {
        opt = *options;
    } else {
        fill_default_options(&opt);
    }
    IPTBlockReport local;
    if (report == nullptr) report = &local;
    memset(report, 0, sizeof(*report));
    if (row_ptr == nullptr || (nnz > 0 && (col_ind == nullptr || vals == nullptr)) ||
        d_vectors == nullptr || d_values == nullptr || n <= 0 || k <= 0 || k > n || nnz < 0 ||
        !options_valid(&opt) || opt.ipt_precision != IPT_BLOCK_FP64) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)opt.stream;
    DeviceBuffer<double> d, rs;
    const double *dd = d_diag_sorted;
    if (dd == nullptr) {
        IPTGB_CHECK(d.alloc((size_t)n, s));
        IPTGB_CHECK(launch_csr64_diagonal(row_ptr, col_ind, vals, n, d.ptr, s));
        dd = d.ptr;
        // The targets are the k lowest diagonal positions in ascending order,
        // i.e. the first k rows of a diagonal-sorted matrix.  An unsorted
        // matrix goes through the host preparation (sort + symmetric
        // permutation, ipt_preparation.cu:1375-1431) and the rows of the
        // result are scattered back to the caller's order.
        std::vector<double> hd((size_t)n);
        IPTGB_CUDA(cudaMemcpyAsync(hd.data(), d.ptr, (size_t)n * sizeof(double),
                                   cudaMemcpyDeviceToHost, s));
        IPTGB_CUDA(cudaStreamSynchronize(s));
        if (!std::is_sorted(hd.begin(), hd.end())) {
            std::vector<int> rp((size_t)n + 1U), ci((size_t)nnz);
            std::vector<double> cv((size_t)nnz);
            IPTGB_CUDA(cudaMemcpyAsync(rp.data(), row_ptr, rp.size() * sizeof(int),
                                       cudaMemcpyDeviceToHost, s));
            if (nnz > 0) {
                IPTGB_CUDA(cudaMemcpyAsync(ci.data(), col_ind, ci.size() * sizeof(int),
                                           cudaMemcpyDeviceToHost, s));
                IPTGB_CUDA(cudaMemcpyAsync(cv.data(), vals, cv.size() * sizeof(double),
                                           cudaMemcpyDeviceToHost, s));
            }
            IPTGB_CUDA(cudaStreamSynchronize(s));
            PreparedCsr prep;
            IPTGB_CHECK(prepare_csc(rp.data(), ci.data(), cv.data(), n, nnz, true, &prep));
            DeviceBuffer<int> prp, pci, dperm;
            DeviceBuffer<double> pcv, pd, Xs;
            IPTGB_CHECK(prp.alloc(prep.row_ptr.size(), s));
            IPTGB_CHECK(pci.alloc(prep.col_ind.size(), s));
            IPTGB_CHECK(pcv.alloc(prep.vals.size(), s));
            IPTGB_CHECK(pd.alloc((size_t)n, s));
            IPTGB_CHECK(Xs.alloc((size_t)n * k, s));
            IPTGB_CHECK(dperm.alloc((size_t)n, s));
            IPTGB_CUDA(cudaMemcpyAsync(prp.ptr, prep.row_ptr.data(),
                                       prep.row_ptr.size() * sizeof(int), cudaMemcpyHostToDevice, s));
            if (prep.nnz > 0) {
                IPTGB_CUDA(cudaMemcpyAsync(pci.ptr, prep.col_ind.data(),
                                           prep.col_ind.size() * sizeof(int),
                                           cudaMemcpyHostToDevice, s));
                IPTGB_CUDA(cudaMemcpyAsync(pcv.ptr, prep.vals.data(),
                                           prep.vals.size() * sizeof(double),
                                           cudaMemcpyHostToDevice, s));
            }
            IPTGB_CUDA(cudaMemcpyAsync(pd.ptr, prep.diag.data(), (size_t)n * sizeof(double),
                                       cudaMemcpyHostToDevice, s));
            IPTGB_CUDA(cudaMemcpyAsync(dperm.ptr, prep.perm.data(), (size_t)n * sizeof(int),
                                       cudaMemcpyHostToDevice, s));
            if (hook != nullptr) {
                // the collector's reference vectors are in the caller's order
                return IPT_CUDA_INVALID_ARGUMENT;
            }
            IPTGB_CHECK(csr_block_device(prp.ptr, pci.ptr, pcv.ptr, n, prep.nnz, k, &opt, pd.ptr,
                                         Xs.ptr, d_values, report));
            unpermute_rows_kernel<<<blocks_for((size_t)n * k), kThreads, 0, s>>>(
                Xs.ptr, dperm.ptr, n, k, d_vectors);
            IPTGB_LAUNCH();
            IPTGB_CUDA(cudaStreamSynchronize(s));
            return IPT_CUDA_SUCCESS;
        }
    }
    IPTGB_CHECK(rs.alloc((size_t)n, s));
    csr_row_abs_sum_kernel<<<blocks_for(n), kThreads, 0, s>>>(row_ptr, vals, n, rs.ptr);
    IPTGB_LAUNCH();
    double hnorm = 0.0;
    IPTGB_CHECK(max_of_device(rs.ptr, n, s, &hnorm));
    CsrApply apply;
    apply.row_ptr = row_ptr;
    apply.col_ind = col_ind;
    apply.vals = vals;
    apply.n = n;
    apply.nnz = nnz;
    apply.s = s;
    apply.df = davidson_df_products(n);
    std::unique_ptr<IptStage> stage(make_fp64_csr_stage(row_ptr, col_ind, vals, n, dd, s));
    std::unique_ptr<LearnedCorrection> learned;
    LearnedCorrection *corr = hook;
    DeviceBuffer<double> coupling;
    if (corr == nullptr && opt.preconditioner == IPT_BLOCK_PRECOND_MLP) {
        learned.reset(make_learned_correction(opt.mlp_params, s));
        corr = learned.get();
    }
    if (corr != nullptr) {
        IPTGB_CHECK(coupling.alloc((size_t)n, s));
        IPTGB_CHECK(launch_csr_row_coupling(row_ptr, col_ind, vals, n, coupling.ptr, s));
        corr->bind(coupling.ptr, hnorm);
    }
    DeviceBuffer<double> Xfb;
    bool done = false;
    if (opt.strategy == IPT_BLOCK_STRATEGY_REFINE && k <= 64 && d_initial == nullptr) {
        RefineInput rin;
        rin.apply = &apply;
        rin.d = dd;
        rin.n = n;
        rin.k = k;
        rin.hnorm = hnorm;
        rin.opt = opt;
        rin.max_outer = std::max(1, opt.refine_maxiter);
        IPTGB_CHECK(Xfb.alloc((size_t)n * k, s));
        bool conv = false;
        IPTGB_CHECK(refine_solve(rin, d_vectors, d_values, report, s, &conv, Xfb.ptr));
        done = conv;
    }
    if (!done) {
        IPTBlockReport first = *report;
        BlockSolveInput in;
        in.apply = &apply;
        in.ipt = stage.get();
        in.learned = corr;
        in.d = dd;
        in.n = n;
        in.k = k;
        in.hnorm = hnorm;
        in.opt = opt;
        in.orth = orth;

        if (Xfb.ptr != nullptr) {
            in.initial = Xfb.ptr;
            in.initial_cols = k;
        } else if (d_initial != nullptr) {
            in.initial = d_initial;
            in.initial_cols = initial_cols;
        }
        IPTGB_CHECK(block_solve(in, d_vectors, d_values, report, s));
        if (Xfb.ptr != nullptr) {
            report->fp64_matvecs += first.fp64_matvecs;
            report->total_ms += first.total_ms;
        }
    }
    IPTGB_CUDA(cudaStreamSynchronize(s));
    return IPT_CUDA_SUCCESS;
}

}  // namespace iptgb

using namespace iptgb;

IPT_API int ipt_block_symmetric_eig(const double *d_T, int m, double *d_w, double *d_Z,
                                    void *stream)
{
    if (d_T == nullptr || d_w == nullptr || d_Z == nullptr || m <= 0 || m > 112) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    BlockOps ops;
    ops.stream = (cudaStream_t)stream;
    ops.sms = device_sm_count();
    int st = ops.symmetric_eig(d_T, m, d_w, d_Z, nullptr);
    ops.release();
    if (st == IPT_CUDA_SUCCESS && cudaStreamSynchronize(ops.stream) != cudaSuccess) {
        st = IPT_CUDA_CUDA_ERROR;
    }
    return st;
}

IPT_API int ipt_block_cholesky_inverse(const double *d_G, int m, double *d_Rinv, int *shifts,
                                       int precision, void *stream)
{
    if (d_G == nullptr || d_Rinv == nullptr || m <= 0 || m > 112 || precision < 0 ||
        precision > 1) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    BlockOps ops;
    ops.stream = (cudaStream_t)stream;
    ops.sms = device_sm_count();
    DeviceBuffer<int> st_dev;
    IPTGB_CHECK(st_dev.alloc(1, ops.stream));
    int st = ops.chol_inverse(d_G, m, d_Rinv, st_dev.ptr, nullptr, precision == 1);
    int h = -1;
    if (st == IPT_CUDA_SUCCESS &&
        (cudaMemcpyAsync(&h, st_dev.ptr, sizeof(int), cudaMemcpyDeviceToHost, ops.stream) !=
             cudaSuccess ||
         cudaStreamSynchronize(ops.stream) != cudaSuccess)) {
        st = IPT_CUDA_CUDA_ERROR;
    }
    ops.release();
    if (st != IPT_CUDA_SUCCESS) return st;
    if (shifts != nullptr) *shifts = h;
    return h < 0 ? IPT_CUDA_INVALID_ARGUMENT : IPT_CUDA_SUCCESS;
}

IPT_API void ipt_block_default_options(IPTBlockOptions *options)
{
    if (options != nullptr) {
        fill_default_options(options);
    }
}

IPT_API int ipt_block_solve_dense_device(const double *d_matrix_col_major, int n, int k,
                                         const IPTBlockOptions *options, double *d_vectors,
                                         double *d_values, IPTBlockReport *report)
{
    return dense_block_device(d_matrix_col_major, n, k, options, d_vectors, d_values, report);
}

IPT_API int ipt_block_solve_dense(const double *matrix_col_major, int n, int k,
                                  const IPTBlockOptions *options, double *vectors, double *values,
                                  IPTBlockReport *report)
{
    if (matrix_col_major == nullptr || vectors == nullptr || values == nullptr || n <= 0 ||
        k <= 0 || k > n) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    IPTBlockOptions opt;
    if (options != nullptr) {
        opt = *options;
    } else {
        fill_default_options(&opt);
    }
    cudaStream_t s = (cudaStream_t)opt.stream;
    const size_t mat = (size_t)n * n;
    trace_mark("host_dense:start", s);
    DeviceBuffer<double> dH, dX, dv;
    IPTGB_CHECK(dH.alloc(mat, s));
    IPTGB_CHECK(dX.alloc((size_t)n * k, s));
    IPTGB_CHECK(dv.alloc((size_t)k, s));
    trace_mark("host_dense:allocated", s);
    // Pinned (page-locked) host memory is readable by the GPU: the solve's
    // first pass then reads H over the host link itself and derives everything
    // it needs on the way (no separate copy, then pass).  Pageable memory is
    // copied first.
    cudaPointerAttributes attr;
    const double *host_src = nullptr;
    if (cudaPointerGetAttributes(&attr, matrix_col_major) == cudaSuccess &&
        attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr) {
        host_src = static_cast<const double *>(attr.devicePointer);
    } else {
        cudaGetLastError();  // clear a pageable-pointer query error, if any
        IPTGB_CUDA(cudaMemcpyAsync(dH.ptr, matrix_col_major, mat * sizeof(double),
                                   cudaMemcpyHostToDevice, s));
    }
    trace_mark("host_dense:h2d_done", s);
    IPTGB_CHECK(dense_block_device(dH.ptr, n, k, &opt, dX.ptr, dv.ptr, report, host_src));
    IPTGB_CUDA(cudaMemcpyAsync(vectors, dX.ptr, (size_t)n * k * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaMemcpyAsync(values, dv.ptr, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost,
                               s));
    trace_mark("host_dense:d2h_done", s);
    IPTGB_CUDA(cudaStreamSynchronize(s));
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_block_solve_csr_device(const int *d_row_ptr, const int *d_col_ind,
                                       const double *d_values_csr, int n, int nnz, int k,
                                       const IPTBlockOptions *options, double *d_vectors,
                                       double *d_values, IPTBlockReport *report)
{
    return csr_block_device(d_row_ptr, d_col_ind, d_values_csr, n, nnz, k, options, nullptr,
                            d_vectors, d_values, report);
}

IPT_API int ipt_block_mlp_collect_csr(const int *d_row_ptr, const int *d_col_ind,
                                      const double *d_values_csr, int n, int nnz, int k,
                                      const IPTBlockOptions *options,
                                      const double *d_exact_vectors, int exact_cols,
                                      float *d_rows, long long capacity, long long *rows_written,
                                      IPTBlockReport *report)
{
    if (d_exact_vectors == nullptr || exact_cols <= 0 || exact_cols > n || d_rows == nullptr ||
        capacity < 0 || rows_written == nullptr || n <= 0 || k <= 0 || k > n) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    IPTBlockOptions opt;
    if (options != nullptr) {
        opt = *options;
    } else {
        fill_default_options(&opt);
    }
    opt.strategy = IPT_BLOCK_STRATEGY_DAVIDSON;
    // with MLP parameters the rows are recorded along the learned trajectory
    const float *params =
        opt.preconditioner == IPT_BLOCK_PRECOND_MLP ? (const float *)opt.mlp_params : nullptr;
    opt.preconditioner = IPT_BLOCK_PRECOND_DIAGONAL;
    cudaStream_t s = (cudaStream_t)opt.stream;
    std::unique_ptr<LearnedCorrection> col(
        make_mlp_collector(d_exact_vectors, exact_cols, d_rows, capacity, params, s));
    DeviceBuffer<double> dX, dv;
    IPTGB_CHECK(dX.alloc((size_t)n * k, s));
    IPTGB_CHECK(dv.alloc((size_t)k, s));
    const int st = csr_block_device(d_row_ptr, d_col_ind, d_values_csr, n, nnz, k, &opt, nullptr,
                                    dX.ptr, dv.ptr, report, col.get());
    *rows_written = mlp_collector_count(col.get());
    IPTGB_CUDA(cudaStreamSynchronize(s));
    return st;
}

IPT_API int ipt_block_solve_csr(const int *row_ptr, const int *col_ind, const double *values_csr,
                                int n, int nnz, int k, const IPTBlockOptions *options,
                                double *vectors, double *values, IPTBlockReport *report)
{
    if (row_ptr == nullptr || col_ind == nullptr || values_csr == nullptr || vectors == nullptr ||
        values == nullptr || n <= 0 || k <= 0 || k > n || nnz < 0) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    // For a symmetric H the CSR arrays are the CSC arrays of the same matrix.
    PreparedCsr prep;
    IPTGB_CHECK(prepare_csc(row_ptr, col_ind, values_csr, n, nnz, true, &prep));
    IPTBlockOptions opt;
    if (options != nullptr) {
        opt = *options;
    } else {
        fill_default_options(&opt);
    }
    cudaStream_t s = (cudaStream_t)opt.stream;
    DeviceBuffer<int> rp, ci;
    DeviceBuffer<double> cv, dd, dX, dv;
    IPTGB_CHECK(rp.alloc(prep.row_ptr.size(), s));
    IPTGB_CHECK(ci.alloc(prep.col_ind.size(), s));
    IPTGB_CHECK(cv.alloc(prep.vals.size(), s));
    IPTGB_CHECK(dd.alloc((size_t)n, s));
    IPTGB_CHECK(dX.alloc((size_t)n * k, s));
    IPTGB_CHECK(dv.alloc((size_t)k, s));
    IPTGB_CUDA(cudaMemcpyAsync(rp.ptr, prep.row_ptr.data(), prep.row_ptr.size() * sizeof(int),
                               cudaMemcpyHostToDevice, s));
    if (!prep.col_ind.empty()) {
        IPTGB_CUDA(cudaMemcpyAsync(ci.ptr, prep.col_ind.data(), prep.col_ind.size() * sizeof(int),
                                   cudaMemcpyHostToDevice, s));
        IPTGB_CUDA(cudaMemcpyAsync(cv.ptr, prep.vals.data(), prep.vals.size() * sizeof(double),
                                   cudaMemcpyHostToDevice, s));
    }
    IPTGB_CUDA(cudaMemcpyAsync(dd.ptr, prep.diag.data(), (size_t)n * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    IPTGB_CHECK(csr_block_device(rp.ptr, ci.ptr, cv.ptr, n, prep.nnz, k, &opt, dd.ptr, dX.ptr,
                                 dv.ptr, report));
    IPTGB_CUDA(cudaMemcpyAsync(vectors, dX.ptr, (size_t)n * k * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaMemcpyAsync(values, dv.ptr, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost,
                               s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    unpermute_vectors(prep, vectors, k);
    return IPT_CUDA_SUCCESS;
}

// The reference's IPT_BLOCK_CLUSTER path for the sparse host entry points
// (IPT_C_GPU/src/ipt_cuda.cu:5070-5075 -> 4712-5016): requires a real
// symmetric matrix; Ritz pairs in ascending order, unit-norm vectors, the
// Davidson enrichment (IPT_DAVIDSON_ENRICH) run until the residuals reach
// IPT_DAVIDSON_CONVERGED_TOL.
int ipt_block_sparse_host_entry(const int *col_ptr, const int *row_ind, const double *vals, int n,
                                int k, int nnz, int maxiter, double tol, int use_tol,
                                IPTCudaResult *result)
{
    auto t0 = std::chrono::steady_clock::now();
    memset(result, 0, sizeof(*result));
    result->fixed_point_residual = NAN;
    result->davidson_target_index = -1;
    result->davidson_residual_before = NAN;
    result->davidson_residual_after = NAN;
    result->davidson_denom_clip = NAN;
    result->best_so_far_enabled = 1;
    result->best_so_far_step = -1;
    strcpy(result->best_so_far_source, "none");
    result->best_so_far_max_residual = NAN;
    result->best_so_far_max_residual_index = -1;
    result->adaptive_coupling_tau = NAN;
    result->adaptive_target_block_start = -1;
    result->adaptive_target_block_end = -1;
    if (!validate_csc(col_ptr, row_ind, n, nnz)) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    PreparedCsr prep;
    IPTGB_CHECK(prepare_csc(col_ptr, row_ind, vals, n, nnz, true, &prep));
    // The reference's block-cluster preparation always merges and sorts the
    // columns (duplicates summed, exact zeros dropped; ipt_cuda.cu:4568-4575)
    // and then requires a real symmetric matrix (4586-4595).  A permuted
    // preparation is merged already; otherwise merge the caller's arrays.
    std::vector<int> mcp, mri;
    std::vector<double> mva;
    const bool as_given = !prep.permuted && csc_columns_merged(col_ptr, row_ind, vals, n);
    if (!prep.permuted && !as_given) merge_csc_columns(col_ptr, row_ind, vals, n, &mcp, &mri, &mva);
    const int *m_ptr = prep.permuted ? prep.row_ptr.data() : as_given ? col_ptr : mcp.data();
    const int *m_idx = prep.permuted ? prep.col_ind.data() : as_given ? row_ind : mri.data();
    const double *m_val = prep.permuted ? prep.vals.data() : as_given ? vals : mva.data();
    if (!merged_is_symmetric(m_ptr, m_idx, m_val, n)) {
        ipt_cuda_free_result(result);
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    IPTBlockOptions opt;
    fill_default_options(&opt);
    int block_maxiter = env_int("IPT_BLOCK_CLUSTER_MAXITER", maxiter > 0 ? maxiter : 100);
    if (block_maxiter <= 0) block_maxiter = 100;
    const double block_tol = env_double("IPT_BLOCK_CLUSTER_TOL", use_tol ? tol : 1e-12);
    const double damping = env_double("IPT_BLOCK_CLUSTER_DAMPING", 1.0);
    // cluster ranges of the diagonal-sorted matrix (ipt_cuda.cu:4555-4688);
    // for a symmetric matrix the prepared CSR arrays are also its CSC arrays
    const int adaptive = env_flag("IPT_BLOCK_CLUSTER_ADAPTIVE", 0);
    const double coupling_tau = env_double("IPT_BLOCK_CLUSTER_COUPLING_TAU", 0.1);
    const int oversample = adaptive ? 0 : env_int("IPT_BLOCK_CLUSTER_OVERSAMPLE", 0);
    const int target_k = oversample > 0 ? (oversample > n - k ? n : k + oversample) : k;
    // the reference scans its permuted CSC, merged and sorted even when the
    // order did not change (ipt_cuda.cu:4568-4575); for a symmetric matrix
    // the permuted CSC equals the prepared CSR
    ClusterRanges cr;
    cluster_ranges(m_ptr, m_idx, m_val, n, target_k, k,
                   env_double("IPT_DEGENERACY_THRESHOLD", 0.0), adaptive, coupling_tau, &cr);
    int basis_cols = 0;
    for (const auto &r : cr.ranges) {
        basis_cols += r.second - r.first + 1;
        if (r.first <= k - 1 && k - 1 <= r.second) {
            result->adaptive_target_block_start = r.first;
            result->adaptive_target_block_end = r.second;
        }
    }
    result->oversample = oversample;
    result->adaptive_block_enabled = adaptive;
    result->adaptive_coupling_tau = coupling_tau;
    result->adaptive_limit_hit = cr.limit_hit;
    {
        std::string added;
        for (int i : cr.added) added += (added.empty() ? "" : ";") + std::to_string(i);
        snprintf(result->adaptive_added_indices, sizeof(result->adaptive_added_indices), "%s",
                 added.empty() ? "none" : added.c_str());
    }
    if (cr.too_large || basis_cols < k) {
        ipt_cuda_free_result(result);
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    if (basis_cols > 112) {
        // the projected eigensolve keeps the basis in one CTA's shared memory
        fprintf(stderr, "ipt_gb300: block-cluster basis of %d columns exceeds 112\n", basis_cols);
        ipt_cuda_free_result(result);
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    opt.oversample = basis_cols - k;
    opt.strategy = IPT_BLOCK_STRATEGY_DAVIDSON;
    const int enrich = env_flag("IPT_DAVIDSON_ENRICH", 0);
    const int steps = std::max(0, env_int("IPT_DAVIDSON_STEPS", 1)) +
                      std::max(0, env_int("IPT_DAVIDSON_EXTRA_STEPS", 0));
    opt.davidson_maxsteps = enrich ? std::max(1, steps) : 0;
    opt.residual_tol = env_double("IPT_DAVIDSON_CONVERGED_TOL", 1e-13);
    // The reference's Rayleigh-Ritz on the cluster basis is a Gram matrix and
    // a generalized eigensolve by default, or Householder QR and a standard
    // eigensolve with IPT_BLOCK_CLUSTER_QR (ipt_cuda.cu:3071, 3103-3218).
    // Both give the Ritz pairs of the same subspace; here the basis is always
    // orthonormalised (CholQR2) before a standard eigensolve, and the knob
    // sets rayleigh_ritz_used_qr and which basis the orthogonality figures of
    // IPT_RR_HOST_ORTHOGONALITY_STATS (ipt_cuda.cu:3072, 3191-3268) describe:
    // the cluster basis as built, or its orthonormalised form.
    const int use_qr = env_flag("IPT_BLOCK_CLUSTER_QR", 0);
    OrthStats orth;
    orth.raw_first_basis = !use_qr;
    OrthStats *orth_out = env_flag("IPT_RR_HOST_ORTHOGONALITY_STATS", 0) ? &orth : nullptr;
    result->vectors = (double *)calloc((size_t)n * k, sizeof(double));
    result->values = (double *)calloc((size_t)k, sizeof(double));
    if (result->vectors == nullptr || result->values == nullptr) {
        ipt_cuda_free_result(result);
        return IPT_CUDA_ALLOCATION_FAILED;
    }
    result->preparation_time_sec =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    IPTBlockReport rep;
    int status;
    {
        cudaStream_t s = nullptr;
        status = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess
                     ? IPT_CUDA_SUCCESS
                     : IPT_CUDA_CUDA_ERROR;
        opt.stream = s;
        DeviceBuffer<int> rp, ci;
        DeviceBuffer<double> cv, dd, dX, dv;
        if (status == IPT_CUDA_SUCCESS) status = rp.alloc(prep.row_ptr.size(), s);
        if (status == IPT_CUDA_SUCCESS) status = ci.alloc(prep.col_ind.size(), s);
        if (status == IPT_CUDA_SUCCESS) status = cv.alloc(prep.vals.size(), s);
        if (status == IPT_CUDA_SUCCESS) status = dd.alloc((size_t)n, s);
        if (status == IPT_CUDA_SUCCESS) status = dX.alloc((size_t)n * k, s);
        if (status == IPT_CUDA_SUCCESS) status = dv.alloc((size_t)k, s);
        if (status == IPT_CUDA_SUCCESS &&
            (cudaMemcpyAsync(rp.ptr, prep.row_ptr.data(), prep.row_ptr.size() * sizeof(int),
                             cudaMemcpyHostToDevice, s) != cudaSuccess ||
             (prep.nnz > 0 &&
              (cudaMemcpyAsync(ci.ptr, prep.col_ind.data(), prep.col_ind.size() * sizeof(int),
                               cudaMemcpyHostToDevice, s) != cudaSuccess ||
               cudaMemcpyAsync(cv.ptr, prep.vals.data(), prep.vals.size() * sizeof(double),
                               cudaMemcpyHostToDevice, s) != cudaSuccess)) ||
             cudaMemcpyAsync(dd.ptr, prep.diag.data(), (size_t)n * sizeof(double),
                             cudaMemcpyHostToDevice, s) != cudaSuccess)) {
            status = IPT_CUDA_CUDA_ERROR;
        }
        // the block-cluster basis (k_cluster.cu), then Rayleigh-Ritz and the
        // Davidson enrichment from it
        DeviceBuffer<double> basis;
        std::vector<int> rg((size_t)cr.ranges.size() * 2), cl_it(cr.ranges.size());
        std::vector<double> cl_res(cr.ranges.size());
        for (size_t c = 0; c < cr.ranges.size(); ++c) {
            rg[2 * c] = cr.ranges[c].first;
            rg[2 * c + 1] = cr.ranges[c].second;
        }
        if (status == IPT_CUDA_SUCCESS) status = basis.alloc((size_t)n * basis_cols, s);
        if (status == IPT_CUDA_SUCCESS) {
            auto tb = std::chrono::steady_clock::now();
            int bad = -1;
            status = cluster_basis_solve(rp.ptr, ci.ptr, cv.ptr, n, prep.nnz, dd.ptr, rg.data(),
                                         (int)cr.ranges.size(), block_maxiter, block_tol, damping,
                                         basis.ptr, cl_it.data(), cl_res.data(), &bad, s);
            if (status != IPT_CUDA_SUCCESS && bad >= 0) {
                fprintf(stderr,
                        "ipt_gb300: block-cluster solve failed for block=%d:%d size=%d\n",
                        cr.ranges[(size_t)bad].first, cr.ranges[(size_t)bad].second,
                        cr.ranges[(size_t)bad].second - cr.ranges[(size_t)bad].first + 1);
            }
            result->iteration_time_sec =
                std::chrono::duration<double>(std::chrono::steady_clock::now() - tb).count();
        }
        if (status == IPT_CUDA_SUCCESS) {
            for (size_t c = 0; c < cr.ranges.size(); ++c) {
                const int w = cr.ranges[c].second - cr.ranges[c].first + 1;
                result->iterations = std::max(result->iterations, cl_it[c]);
                result->matvecs += (long long)cl_it[c] * w;
                if (isfinite(cl_res[c]) && !(cl_res[c] <= result->fixed_point_residual)) {
                    result->fixed_point_residual = cl_res[c];
                }
            }
            status = csr_block_device(rp.ptr, ci.ptr, cv.ptr, n, prep.nnz, k, &opt, dd.ptr, dX.ptr,
                                      dv.ptr, &rep, nullptr, basis.ptr, basis_cols, orth_out);
        }
        basis.release();
        if (status == IPT_CUDA_SUCCESS &&
            (cudaMemcpyAsync(result->vectors, dX.ptr, (size_t)n * k * sizeof(double),
                             cudaMemcpyDeviceToHost, s) != cudaSuccess ||
             cudaMemcpyAsync(result->values, dv.ptr, (size_t)k * sizeof(double),
                             cudaMemcpyDeviceToHost, s) != cudaSuccess ||
             cudaStreamSynchronize(s) != cudaSuccess)) {
            status = IPT_CUDA_CUDA_ERROR;
        }
        rp.release();
        ci.release();
        cv.release();
        dd.release();
        dX.release();
        dv.release();
        if (s != nullptr) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
    if (status != IPT_CUDA_SUCCESS) {
        ipt_cuda_free_result(result);
        return status;
    }
    unpermute_vectors(prep, result->vectors, k);
    result->n = n;
    result->k = k;
    result->basis_cols = rep.basis_cols;
    result->matvecs += rep.fp64_matvecs;
    result->rayleigh_ritz_time_sec = rep.rayleigh_ritz_ms * 1e-3;
    result->davidson_time_sec = rep.davidson_ms * 1e-3;
    result->solve_time_sec = rep.total_ms * 1e-3;
    result->oversample = opt.oversample;
    result->rayleigh_ritz_used_qr = use_qr;
    result->davidson_attempted = opt.davidson_maxsteps > 0;
    result->davidson_accepted = rep.davidson_steps > 0;
    result->davidson_residual_after = rep.max_scaled_residual;
    result->davidson_restart_count = rep.restarts;
    result->accepted_steps = rep.davidson_steps;
    result->best_so_far_max_residual = rep.max_scaled_residual;
    strcpy(result->best_so_far_source, rep.davidson_steps > 0 ? "davidson" : "rayleigh_ritz");
    result->final_returned_from_best_so_far = 1;
    strcpy(result->pair28_lock_state, "inactive");
    strcpy(result->pair29_lock_state, "inactive");
    result->gap28_29 = NAN;
    result->relative_gap28_29 = NAN;
    result->cluster_residual_fro = NAN;
    result->cluster_residual_max = NAN;
    result->pair28_best_residual = NAN;
    result->pair29_best_residual = NAN;
    result->basis_orthogonality_frobenius_error = orth.basis.frobenius;
    result->basis_orthogonality_max_abs_error = orth.basis.max_abs;
    result->basis_has_nan_or_inf = orth.basis.invalid;
    result->ritz_vectors_orthogonality_frobenius_error = orth.ritz.frobenius;
    result->ritz_vectors_orthogonality_max_abs_error = orth.ritz.max_abs;
    result->ritz_vectors_has_nan_or_inf = orth.ritz.invalid;
    return IPT_CUDA_SUCCESS;
}
