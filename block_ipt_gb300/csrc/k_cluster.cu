// k_cluster.cu - the block-cluster basis solve of the IPT_BLOCK_CLUSTER path.
//
// The reference iterates, for every cluster c of diagonal positions
// [first, last] (m = last - first + 1 <= 64), the block fixed point
//     Y = H X,  h = Y[first:last, :],
//     X'[i, :] = e_{i - first}^T                          for i in the cluster,
//     (d_i I - h^T) X'[i, :]^T = d_i X[i, :]^T - Y[i, :]^T  otherwise,
// from the identity columns, until ||X' - X||_F / max(1, ||X||_F) <= tol
// (IPT_C_GPU/src/ipt_cuda.cu:2871-3037), solving each row's m x m system by
// Gauss-Jordan elimination with partial pivoting in one CTA per row
// (ipt_block_cluster_update_kernel, ipt_cuda.cu:2280-2384), one cluster
// after the other, with a device-to-host read of a singular flag and two
// norms per iteration.
//
// Here all clusters iterate together: one CSR product covers the columns of
// every cluster still iterating, one update launch solves every (row,
// cluster) system, one norm launch and a one-CTA finish kernel decide per
// cluster whether it has converged, and the host reads one small status
// block per iteration.  A converged cluster is frozen: its columns are not
// updated again, so every cluster ends with exactly the iterate the
// reference's own loop for it returns.
//
// The update gives each row's system to a team of T lanes, with the
// augmented matrix in shared memory and row e of it owned by lane e mod T.
// On GB300 the FP64 pipe (about 2 operations per clock per SM) is the bound,
// so the kernel keeps FP64 instructions to the elimination itself: T is the
// smallest power of two for which the CTA's 128/T systems fit in ~96 KB of
// shared memory (T = 1 up to m = 8: every lane works on its own row's
// system), the pivot search compares |entries| as integers, a pivot row is
// scaled by one reciprocal, and the column just eliminated (never read
// again) is not updated.  The pivot is the first row holding the largest
// |entry| (the reference's sequential scan with a strict comparison); a NaN
// diagonal entry, a pivot that is not finite or not above 64 DBL_EPSILON is
// singular.  The CPU restatement of this kernel (the oracle) performs the
// same operations in the same order and reproduces it bit for bit.
#include <float.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <utility>
#include <vector>

#include "block_solver.h"
#include "cluster.h"
#include "common.cuh"
#include "ipt_plain.h"
#include "kernels.cuh"
#include "reduce.cuh"

namespace iptgb {

constexpr int kClusterThreads = 128;
constexpr int kClusterNormSlices = 64;
constexpr size_t kClusterSmemBudget = 96 * 1024;

// Lanes per row system (a power of two, at most 32).
__host__ __device__ __forceinline__ int cluster_team(int m)
{
    int t = 1;
    while (t < 32 && (size_t)(kClusterThreads / t) * m * (m + 1) * sizeof(double) +
                             (size_t)m * m * sizeof(double) >
                         kClusterSmemBudget) {
        t <<= 1;
    }
    return t;
}

size_t cluster_update_smem(int m)
{
    const int teams = kClusterThreads / cluster_team(m);
    return ((size_t)m * m + (size_t)teams * m * (m + 1)) * sizeof(double);
}

constexpr uint64_t kAbsMask = 0x7FFFFFFFFFFFFFFFull;
constexpr uint64_t kInfBits = 0x7FF0000000000000ull;
constexpr uint64_t kTinyPivotBits = 0x3D10000000000000ull;  // 64 DBL_EPSILON = 2^-46

// info[c] = {first, m, column offset, 0}; active[c] != 0 while c iterates.
// Element (e, j) of a team's augmented system sits at ((e (m+1) + j) teams +
// team): the teams of a warp touch consecutive words.
__global__ void __launch_bounds__(kClusterThreads)
cluster_update_kernel(const double *__restrict__ X, const double *__restrict__ Y,
                      const double *__restrict__ d, int n, const int4 *__restrict__ info,
                      const int *__restrict__ active, double damping, double *__restrict__ Xn,
                      int *__restrict__ flags)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const int c = blockIdx.y;
    if (active[c] == 0) return;
    const int4 ci = info[c];
    const int first = ci.x, m = ci.y, off = ci.z;
    const int T = cluster_team(m);
    const int teams = blockDim.x / T;
    const int ld = m + 1;
    extern __shared__ double cl_smem[];
    double *h = cl_smem;  // h[u + e m] = Y[first + u, off + e]
    const int team = threadIdx.x / T;
    const int t = threadIdx.x % T;
    double *aug = cl_smem + (size_t)m * m + team;
#define AUG(e, j) aug[((size_t)(e) * ld + (j)) * teams]
    const unsigned lane = threadIdx.x & 31u;
    const unsigned tmask =
        T == 32 ? 0xffffffffu : (((1u << T) - 1u) << (lane / (unsigned)T * (unsigned)T));
    const double *Xc = X + (size_t)off * n;
    const double *Yc = Y + (size_t)off * n;
    double *Xnc = Xn + (size_t)off * n;
    for (int i = threadIdx.x; i < m * m; i += blockDim.x) {
        const int u = i % m, e = i / m;
        h[i] = Yc[(size_t)(first + u) + (size_t)e * n];
    }
    __syncthreads();
    for (int row0 = blockIdx.x * teams; row0 < n; row0 += gridDim.x * teams) {
        const int row = row0 + team;
        if (row >= n) continue;
        if (row >= first && row < first + m) {
            for (int e = t; e < m; e += T) Xnc[(size_t)row + (size_t)e * n] = row == first + e ? 1.0 : 0.0;
            continue;
        }
        const double dr = d[row];
        for (int e = t; e < m; e += T) {
            for (int u = 0; u < m; ++u) {
                const double hv = h[u + e * m];
                AUG(e, u) = u == e ? dr - hv : -hv;
            }
            AUG(e, m) = fma(dr, Xc[(size_t)row + (size_t)e * n], -Yc[(size_t)row + (size_t)e * n]);
        }
        __syncwarp(tmask);
        bool singular = false;
        for (int p = 0; p < m; ++p) {
            // pivot: largest |entry| of column p in rows p.., first on ties,
            // compared as integers (the order of non-negative doubles)
            uint64_t best = 0;
            int bi = m;
            bool diag_nan = false;
            for (int e = t + ((p - t + T - 1) / T) * T; e < m; e += T) {
                const uint64_t key = (uint64_t)__double_as_longlong(AUG(e, p)) & kAbsMask;
                if (key > kInfBits) {
                    diag_nan = diag_nan || e == p;
                } else if (key > best || (key == best && e < bi)) {
                    best = key;
                    bi = e;
                }
            }
            for (int o = T >> 1; o >= 1; o >>= 1) {
                const uint64_t ok = __shfl_xor_sync(tmask, (unsigned long long)best, o, T);
                const int oi = __shfl_xor_sync(tmask, bi, o, T);
                if (ok > best || (ok == best && oi < bi)) {
                    best = ok;
                    bi = oi;
                }
            }
            if (T > 1) diag_nan = __any_sync(tmask, diag_nan);
            if (diag_nan || best >= kInfBits || best <= kTinyPivotBits) {
                singular = true;
                break;
            }
            if (bi != p) {
                for (int j = p + t; j <= m; j += T) {
                    const double tmp = AUG(p, j);
                    AUG(p, j) = AUG(bi, j);
                    AUG(bi, j) = tmp;
                }
                __syncwarp(tmask);
            }
            const double r = 1.0 / AUG(p, p);
            __syncwarp(tmask);
            for (int j = p + 1 + t; j <= m; j += T) AUG(p, j) = AUG(p, j) * r;
            __syncwarp(tmask);
            for (int e = t; e < m; e += T) {
                if (e == p) continue;
                const double f = AUG(e, p);
                for (int j = p + 1; j <= m; ++j) AUG(e, j) = fma(-f, AUG(p, j), AUG(e, j));
            }
            __syncwarp(tmask);
        }
        if (!singular) {
            for (int e = t; e < m; e += T) {
                double v = AUG(e, m);
                if (damping < 1.0) v = fma(damping, v, (1.0 - damping) * Xc[(size_t)row + (size_t)e * n]);
                if (((uint64_t)__double_as_longlong(v) & kInfBits) == kInfBits) {
                    singular = true;
                    v = 0.0;
                }
                Xnc[(size_t)row + (size_t)e * n] = v;
            }
        }
#undef AUG
        if (singular) atomicOr(&flags[c], 1);
        __syncwarp(tmask);
    }
}

// Per cluster and slice: sum (Xn - X)^2 and sum X^2 over the cluster's
// columns (contiguous in column-major order), in a fixed order.
__global__ void cluster_norms_kernel(const double *__restrict__ X, const double *__restrict__ Xn,
                                     int n, const int4 *__restrict__ info,
                                     const int *__restrict__ active, double2 *__restrict__ part)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const int c = blockIdx.y;
    if (active[c] == 0) return;
    const int4 ci = info[c];
    const size_t beg = (size_t)ci.z * n;
    const size_t cnt = (size_t)ci.y * n;
    double dd = 0.0, bb = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt;
         i += (size_t)gridDim.x * blockDim.x) {
        const double x = X[beg + i];
        const double dx = Xn[beg + i] - x;
        dd = fma(dx, dx, dd);
        bb = fma(x, x, bb);
    }
    const double2 s = block_sum2(dd, bb);
    if (threadIdx.x == 0) part[(size_t)c * gridDim.x + blockIdx.x] = s;
}

// One thread per cluster: the fixed-point residual, the stop decision and
// the status block st = {error, clusters still iterating, active[0..C)}.
__global__ void cluster_finish_kernel(const double2 *__restrict__ part, int slices, int C,
                                      int *__restrict__ active, int *__restrict__ iters,
                                      int *__restrict__ flags, double *__restrict__ resid,
                                      int maxiter, double tol, int *__restrict__ st)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    __shared__ int live;
    __shared__ int err;
    if (threadIdx.x == 0) {
        live = 0;
        err = 0;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
        if (active[c] == 0) continue;
        double dd = 0.0, bb = 0.0;
        for (int s = 0; s < slices; ++s) {
            const double2 p = part[(size_t)c * slices + s];
            dd += p.x;
            bb += p.y;
        }
        const double dn = sqrt(dd), bn = sqrt(bb);
        if ((flags[c] & 1) != 0 || !isfinite(dn) || !isfinite(bn) || bn <= 0.0) {
            flags[c] |= 2;
            active[c] = 0;
            atomicOr(&err, 1);
            continue;
        }
        const int it = iters[c] + 1;
        iters[c] = it;
        const double r = dn / fmax(1.0, bn);
        resid[c] = r;
        if (r <= tol || it >= maxiter) {
            active[c] = 0;
        } else {
            atomicAdd(&live, 1);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        st[0] = err;
        st[1] = live;
    }
    for (int c = threadIdx.x; c < C; c += blockDim.x) st[2 + c] = active[c];
}

// Columns of the identity start: X[first_c + j, off_c + j] = 1.
__global__ void cluster_identity_kernel(double *__restrict__ X, int n, const int4 *__restrict__ info)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const int4 ci = info[blockIdx.y];
    const size_t cnt = (size_t)ci.y * n;
    double *Xc = X + (size_t)ci.z * n;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt;
         i += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(i / (size_t)n);
        const int r = (int)(i - (size_t)j * n);
        Xc[i] = r == ci.x + j ? 1.0 : 0.0;
    }
}

// The clusters whose last iterate sits in the scratch buffer (an odd
// iteration count) are copied into the result.
__global__ void cluster_collect_kernel(double *__restrict__ X, const double *__restrict__ B, int n,
                                       const int4 *__restrict__ info, const int *__restrict__ iters)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    const int c = blockIdx.y;
    if ((iters[c] & 1) == 0) return;
    const int4 ci = info[c];
    const size_t beg = (size_t)ci.z * n;
    const size_t cnt = (size_t)ci.y * n;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt;
         i += (size_t)gridDim.x * blockDim.x) {
        X[beg + i] = B[beg + i];
    }
}

static int cluster_grid_x(int n, int C, int teams)
{
    const int sms = device_sm_count();
    const int want = std::max(1, (8 * sms + C - 1) / std::max(1, C));
    return std::max(1, std::min((n + teams - 1) / teams, want));
}

// The opt-in shared-memory size is an attribute of the current device's
// context: every launch that needs more than 48 KB sets it (a cheap host
// call), to the largest size any width up to 64 needs, clamped to what the
// current device allows, so launches from several threads never undercut
// each other; only a launch that itself needs more than the device allows
// fails.
static int set_cluster_smem(size_t bytes)
{
    static const size_t largest = [] {
        size_t mx = 0;
        for (int m = 1; m <= kClusterMaxWidth; ++m) mx = std::max(mx, cluster_update_smem(m));
        return mx;
    }();
    if (bytes > 48 * 1024) {
        int dev = 0, optin = 0;
        IPTGB_CUDA(cudaGetDevice(&dev));
        IPTGB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        if (bytes > (size_t)optin) {
            fprintf(stderr, "ipt_gb300: block-cluster update needs %zu bytes of shared memory, "
                            "the device allows %d\n", bytes, optin);
            return IPT_CUDA_INVALID_ARGUMENT;
        }
        IPTGB_CUDA(cudaFuncSetAttribute(cluster_update_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)std::min(std::max(bytes, largest), (size_t)optin)));
    }
    return IPT_CUDA_SUCCESS;
}

// smem: the largest cluster_update_smem() over the clusters (it is not
// monotonic in m: the team count drops when m passes a power of two).
int launch_cluster_update(const double *X, const double *Y, const double *d, int n,
                          const int *info4, const int *active, int C, int max_m, size_t smem,
                          double damping, double *Xn, int *flags, cudaStream_t s)
{
    IPTGB_CHECK(set_cluster_smem(smem));
    const int teams = kClusterThreads / cluster_team(max_m);
    dim3 grid(cluster_grid_x(n, C, teams), C);
    return launch_pdl(cluster_update_kernel, grid, dim3(kClusterThreads), smem, s, X, Y, d, n,
                      reinterpret_cast<const int4 *>(info4), active, damping, Xn, flags);
}

int cluster_basis_solve(const int *row_ptr, const int *col_ind, const double *vals, int n,
                        int nnz, const double *d, const int *ranges, int C, int maxiter, double tol,
                        double damping, double *X, int *iterations, double *residuals,
                        int *first_error_cluster, cudaStream_t s)
{
    if (first_error_cluster != nullptr) *first_error_cluster = -1;
    if (C <= 0 || n <= 0 || ranges == nullptr || X == nullptr || d == nullptr ||
        row_ptr == nullptr) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    std::vector<int> info((size_t)C * 4);
    int cols = 0, max_m = 0;
    size_t smem = 0;
    for (int c = 0; c < C; ++c) {
        const int first = ranges[2 * c], last = ranges[2 * c + 1];
        const int m = last - first + 1;
        if (first < 0 || last >= n || m < 1 || m > kClusterMaxWidth ||
            (c > 0 && first <= ranges[2 * c - 1])) {
            return IPT_CUDA_INVALID_ARGUMENT;  // ranges must be ascending and disjoint
        }
        info[4 * c] = first;
        info[4 * c + 1] = m;
        info[4 * c + 2] = cols;
        info[4 * c + 3] = 0;
        cols += m;
        max_m = std::max(max_m, m);
        smem = std::max(smem, cluster_update_smem(m));
    }
    if (!(damping > 0.0 && damping <= 1.0)) damping = 1.0;  // ipt_cuda.cu:4289-4294
    const double eff_tol = tol > 0.0 ? tol : 1.0e-12;
    const size_t nb = (size_t)n * cols;
    DeviceBuffer<double> B, Y, R;
    DeviceBuffer<int> I;
    DeviceBuffer<double2> part;
    IPTGB_CHECK(B.alloc(nb, s));
    IPTGB_CHECK(Y.alloc(nb, s));
    IPTGB_CHECK(R.alloc((size_t)C, s));
    // info (4C) | active (C) | iters (C) | flags (C) | status (2 + C)
    IPTGB_CHECK(I.alloc((size_t)C * 8 + 2, s));
    IPTGB_CHECK(part.alloc((size_t)C * kClusterNormSlices, s));
    int *d_info = I.ptr;
    int *d_active = d_info + 4 * C;
    int *d_iters = d_active + C;
    int *d_flags = d_iters + C;
    int *d_st = d_flags + C;
    std::vector<int> init((size_t)C * 8 + 2, 0);
    memcpy(init.data(), info.data(), info.size() * sizeof(int));
    for (int c = 0; c < C; ++c) init[(size_t)4 * C + c] = maxiter > 0 ? 1 : 0;
    IPTGB_CUDA(cudaMemcpyAsync(I.ptr, init.data(), init.size() * sizeof(int),
                               cudaMemcpyHostToDevice, s));
    IPTGB_CHECK(launch_pdl(cluster_identity_kernel, dim3(std::max(1, std::min(64, blocks_for((size_t)n * max_m))), C),
                           dim3(kThreads), 0, s, X, n, reinterpret_cast<const int4 *>(d_info)));
    // large matrices: the products in double-float on the FP32 pipe, the
    // Davidson products' policy (davidson_df_products)
    DeviceBuffer<float> vsplit;
    const bool df = nnz > 0 && davidson_df_products(n);
    if (df) {
        IPTGB_CHECK(vsplit.alloc(2 * (size_t)nnz, s));
        IPTGB_CHECK(launch_df_split(vals, (size_t)nnz, vsplit.ptr, vsplit.ptr + nnz, s));
    }
    std::vector<int> hst((size_t)C + 2, 0);
    std::vector<char> live((size_t)C, maxiter > 0 ? 1 : 0);
    double *cur = X, *nxt = B.ptr;
    bool failed = false;
    for (int it = 0; it < maxiter; ++it) {
        // the product covers the column span of the clusters still iterating
        int lo = -1, hi = -1;
        for (int c = 0; c < C; ++c) {
            if (!live[(size_t)c]) continue;
            if (lo < 0) lo = info[4 * c + 2];
            hi = info[4 * c + 2] + info[4 * c + 1];
        }
        if (lo < 0) break;
        {
            KernelTimerScope timer(kProfCsrProduct, s);
            if (df) {
                IPTGB_CHECK(launch_csr_df_spmm(row_ptr, col_ind, vsplit.ptr, vsplit.ptr + nnz, n,
                                               cur + (size_t)lo * n, hi - lo,
                                               Y.ptr + (size_t)lo * n, s));
            } else {
                IPTGB_CHECK(launch_csr64_spmm(row_ptr, col_ind, vals, n, cur + (size_t)lo * n,
                                              hi - lo, Y.ptr + (size_t)lo * n, s));
            }
        }
        {
            KernelTimerScope timer(kProfClusterUpdate, s);
            IPTGB_CHECK(launch_cluster_update(cur, Y.ptr, d, n, d_info, d_active, C, max_m, smem,
                                              damping, nxt, d_flags, s));
        }
        IPTGB_CHECK(launch_pdl(cluster_norms_kernel, dim3(kClusterNormSlices, C), dim3(kThreads), 0,
                               s, cur, nxt, n, reinterpret_cast<const int4 *>(d_info), d_active,
                               part.ptr));
        IPTGB_CHECK(launch_pdl(cluster_finish_kernel, dim3(1), dim3(128), 0, s, part.ptr,
                               kClusterNormSlices, C, d_active, d_iters, d_flags, R.ptr, maxiter,
                               eff_tol, d_st));
        IPTGB_CUDA(cudaMemcpyAsync(hst.data(), d_st, hst.size() * sizeof(int),
                                   cudaMemcpyDeviceToHost, s));
        IPTGB_CUDA(cudaStreamSynchronize(s));
        std::swap(cur, nxt);
        if (hst[0] != 0) {
            failed = true;
            break;
        }
        for (int c = 0; c < C; ++c) live[(size_t)c] = (char)(hst[(size_t)2 + c] != 0);
        if (hst[1] == 0) break;
    }
    // every cluster's last iterate into X
    IPTGB_CHECK(launch_pdl(cluster_collect_kernel, dim3(std::max(1, std::min(64, blocks_for((size_t)n * max_m))), C),
                           dim3(kThreads), 0, s, X, B.ptr, n,
                           reinterpret_cast<const int4 *>(d_info), d_iters));
    std::vector<int> h_it((size_t)C), h_fl((size_t)C);
    std::vector<double> h_r((size_t)C);
    IPTGB_CUDA(cudaMemcpyAsync(h_it.data(), d_iters, (size_t)C * sizeof(int),
                               cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaMemcpyAsync(h_fl.data(), d_flags, (size_t)C * sizeof(int),
                               cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaMemcpyAsync(h_r.data(), R.ptr, (size_t)C * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    for (int c = 0; c < C; ++c) {
        if (iterations != nullptr) iterations[c] = h_it[(size_t)c];
        if (residuals != nullptr) residuals[c] = h_it[(size_t)c] > 0 ? h_r[(size_t)c] : NAN;
        if (failed && h_fl[(size_t)c] != 0 && first_error_cluster != nullptr &&
            *first_error_cluster < 0) {
            *first_error_cluster = c;
        }
    }
    return failed ? IPT_CUDA_INVALID_ARGUMENT : IPT_CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------
// Cluster ranges from a device CSR: the O(nnz) scans on the GPU (one warp per
// row: the diagonal as the sum of the row's diagonal entries, and the largest
// off-diagonal magnitude), the rules of the reference's detection on the host
// (prep.cpp) with the few matrix rows they read fetched on demand.
// ---------------------------------------------------------------------------
__global__ void csr_diag_offmax_kernel(const int *__restrict__ row_ptr,
                                       const int *__restrict__ col_ind,
                                       const double *__restrict__ vals, int n,
                                       double *__restrict__ diag, double *__restrict__ offmax)
{
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;
    const int row = (int)warp;
    double dsum = 0.0, m = 0.0;
    for (int p = row_ptr[row] + lane; p < row_ptr[row + 1]; p += 32) {
        const double v = vals[p];
        if (col_ind[p] == row) {
            dsum += v;
        } else {
            m = fmax(m, fabs(v));
        }
    }
    // a merged row holds at most one diagonal entry, so the sum is exact
    for (int off = 16; off > 0; off >>= 1) {
        dsum += __shfl_xor_sync(0xffffffffu, dsum, off);
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    }
    if (lane == 0) {
        diag[row] = dsum;
        offmax[row] = m;
    }
}

namespace {

// Rows of a symmetric device CSR, fetched on demand: for a symmetric matrix
// CSC column c is CSR row c, and H[r, c] can be read from either row.
struct DeviceCsrView final : ClusterMatrixView {
    const int *row_ptr = nullptr;
    const int *col_ind = nullptr;
    const double *vals = nullptr;
    cudaStream_t s = nullptr;
    std::vector<int> h_row_ptr;
    std::vector<std::vector<std::pair<int, double>>> rows;
    std::vector<char> have;
    int status = IPT_CUDA_SUCCESS;

    // rows [r0, r1) in one copy
    void fetch(int r0, int r1)
    {
        const int p0 = h_row_ptr[(size_t)r0], p1 = h_row_ptr[(size_t)r1];
        std::vector<int> ci((size_t)(p1 - p0));
        std::vector<double> va((size_t)(p1 - p0));
        if (p1 > p0 &&
            (cudaMemcpyAsync(ci.data(), col_ind + p0, ci.size() * sizeof(int),
                             cudaMemcpyDeviceToHost, s) != cudaSuccess ||
             cudaMemcpyAsync(va.data(), vals + p0, va.size() * sizeof(double),
                             cudaMemcpyDeviceToHost, s) != cudaSuccess ||
             cudaStreamSynchronize(s) != cudaSuccess)) {
            status = IPT_CUDA_CUDA_ERROR;
        }
        for (int r = r0; r < r1; ++r) {
            auto &row = rows[(size_t)r];
            row.clear();
            for (int p = h_row_ptr[(size_t)r]; p < h_row_ptr[(size_t)r + 1]; ++p) {
                if (status == IPT_CUDA_SUCCESS) {
                    row.emplace_back(ci[(size_t)(p - p0)], va[(size_t)(p - p0)]);
                }
            }
            have[(size_t)r] = 1;
        }
    }
    const std::vector<std::pair<int, double>> &row(int r)
    {
        if (!have[(size_t)r]) fetch(r, r + 1);
        return rows[(size_t)r];
    }
    static double find(const std::vector<std::pair<int, double>> &row, int c)
    {
        auto it = std::lower_bound(row.begin(), row.end(), c,
                                   [](const std::pair<int, double> &e, int v) { return e.first < v; });
        return (it != row.end() && it->first == c) ? it->second : 0.0;
    }
    double entry(int r, int c) override
    {
        if (have[(size_t)c]) return find(rows[(size_t)c], r);
        if (have[(size_t)r]) return find(rows[(size_t)r], c);
        return find(row(c), r);
    }
    void column(int c, std::vector<std::pair<int, double>> *e) override { *e = row(c); }
};

}  // namespace

int cluster_ranges_device(const int *row_ptr, const int *col_ind, const double *vals, int n,
                          int k, int requested_k, double degeneracy_threshold, int adaptive,
                          double coupling_tau, ClusterRanges *out, cudaStream_t s)
{
    DeviceBuffer<double> dd, dm;
    IPTGB_CHECK(dd.alloc((size_t)n, s));
    IPTGB_CHECK(dm.alloc((size_t)n, s));
    csr_diag_offmax_kernel<<<(unsigned)(((long long)n * 32 + 255) / 256), 256, 0, s>>>(
        row_ptr, col_ind, vals, n, dd.ptr, dm.ptr);
    IPTGB_LAUNCH();
    std::vector<double> diag((size_t)n), offmax((size_t)n);
    DeviceCsrView view;
    view.row_ptr = row_ptr;
    view.col_ind = col_ind;
    view.vals = vals;
    view.s = s;
    view.h_row_ptr.resize((size_t)n + 1);
    view.rows.resize((size_t)n);
    view.have.assign((size_t)n, 0);
    IPTGB_CUDA(cudaMemcpyAsync(diag.data(), dd.ptr, (size_t)n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaMemcpyAsync(offmax.data(), dm.ptr, (size_t)n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaMemcpyAsync(view.h_row_ptr.data(), row_ptr, ((size_t)n + 1) * sizeof(int),
                               cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    // the target rows are the first k: one copy
    view.fetch(0, std::min(k, n));
    cluster_ranges_from(view, n, diag, offmax, k, requested_k, degeneracy_threshold, adaptive,
                        coupling_tau, out);
    return view.status;
}

}  // namespace iptgb

#define IPT_API extern "C" __attribute__((visibility("default")))

// Device CSR: the cluster ranges of ipt_block_cluster_ranges (same rules,
// same ranges) for a symmetric matrix whose rows are sorted by column
// without duplicates and whose diagonal is ascending (the prepared matrix of
// the block-cluster path); the scans over the nonzeros run on the GPU.
IPT_API int ipt_block_cluster_ranges_device(const int *d_row_ptr, const int *d_col_ind,
                                            const double *d_vals, int n, int nnz, int k,
                                            int requested_k, double degeneracy_threshold,
                                            int adaptive, double coupling_tau, int *ranges,
                                            int capacity, int *count, int *limit_hit,
                                            void *stream)
{
    if (count != nullptr) *count = 0;
    if (limit_hit != nullptr) *limit_hit = 0;
    if (d_row_ptr == nullptr || d_col_ind == nullptr || d_vals == nullptr || count == nullptr ||
        n <= 0 || nnz < 0 || k <= 0 || k > n || requested_k <= 0 || requested_k > k) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    iptgb::ClusterRanges cr;
    IPTGB_CHECK(iptgb::cluster_ranges_device(d_row_ptr, d_col_ind, d_vals, n, k, requested_k,
                                             degeneracy_threshold, adaptive, coupling_tau, &cr,
                                             static_cast<cudaStream_t>(stream)));
    *count = (int)cr.ranges.size();
    if (limit_hit != nullptr) *limit_hit = cr.limit_hit;
    if (cr.too_large || *count > capacity || ranges == nullptr) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    for (size_t i = 0; i < cr.ranges.size(); ++i) {
        ranges[2 * i] = cr.ranges[i].first;
        ranges[2 * i + 1] = cr.ranges[i].second;
    }
    return IPT_CUDA_SUCCESS;
}

using namespace iptgb;

IPT_API int ipt_block_cluster_basis(const int *d_row_ptr, const int *d_col_ind,
                                    const double *d_vals, int n, int nnz, const double *d_diag,
                                    const int *ranges, int nclusters, int maxiter, double tol,
                                    double damping, double *d_basis, int *iterations,
                                    double *residuals, void *stream)
{
    if (d_row_ptr == nullptr || (nnz > 0 && (d_col_ind == nullptr || d_vals == nullptr)) ||
        d_diag == nullptr || d_basis == nullptr || ranges == nullptr || n <= 0 || nnz < 0 ||
        nclusters <= 0 || maxiter < 0) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    return cluster_basis_solve(d_row_ptr, d_col_ind, d_vals, n, nnz, d_diag, ranges, nclusters,
                               maxiter, tol, damping, d_basis, iterations, residuals, nullptr,
                               (cudaStream_t)stream);
}

IPT_API int ipt_block_cluster_update(const double *d_basis, const double *d_y,
                                     const double *d_diag, int n, int first, int m,
                                     double damping, double *d_next, int *singular, void *stream)
{
    if (d_basis == nullptr || d_y == nullptr || d_diag == nullptr || d_next == nullptr || n <= 0 ||
        m < 1 || m > kClusterMaxWidth || first < 0 || first + m > n) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    DeviceBuffer<int> I;
    IPTGB_CHECK(I.alloc(6, s));
    const int h[6] = {first, m, 0, 0, 1, 0};  // info, active, flags
    IPTGB_CUDA(cudaMemcpyAsync(I.ptr, h, sizeof(h), cudaMemcpyHostToDevice, s));
    IPTGB_CHECK(launch_cluster_update(d_basis, d_y, d_diag, n, I.ptr, I.ptr + 4, 1, m,
                                      cluster_update_smem(m), damping, d_next, I.ptr + 5, s));
    int flag = 0;
    IPTGB_CUDA(cudaMemcpyAsync(&flag, I.ptr + 5, sizeof(int), cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    if (singular != nullptr) *singular = flag & 1;
    return IPT_CUDA_SUCCESS;
}
