// k_eig.cu - symmetric eigensolver for the projected Rayleigh-Ritz matrices.
//
// The m x m projected matrix (m <= 112) needs FP64-accurate eigenpairs.  One
// GB300 SM retires only ~2 FP64 FMAs (or double<->float conversions) per
// clock, so the solve keeps FP64 work off single-CTA kernels:
//
//   Everything works on T' = sym(T) - mu I (mu = mean diagonal): the shift
//   leaves the eigenvectors unchanged but makes every rounding error, FP32
//   and FP64 alike, relative to the spread of the spectrum rather than to its
//   offset (in the refinement below the non-orthogonality of Z enters
//   S = Z^T T Z scaled by the eigenvalues themselves).
//
//   1. FP32 approximate eigenvectors of T':
//        a. conversion + shift + symmetrisation, many CTAs;
//        b. Householder tridiagonalisation, one CTA (four barriers per
//           column);
//        c. bisection (Sturm counts) for every eigenvalue, one thread each,
//           then inverse iteration with a partially pivoted tridiagonal LU,
//           with modified Gram-Schmidt inside clusters of eigenvalues closer
//           than 1e-3 ||T|| between iterations (block inverse iteration),
//           so that clustered vectors span the cluster's invariant subspace;
//        d. back-transformation by the Householder reflectors, one warp per
//           column on many SMs.
//   2. FP64 iterative refinement of the eigenvector matrix, the published
//      method of Ogita and Aishima (Japan J. Indust. Appl. Math. 35 (2018),
//      "Iterative refinement for symmetric eigenvalue decomposition"):
//        R = I - Z^T Z,  S = Z^T T' Z,  l_i = S_ii / (1 - R_ii),
//        delta = 2 (||S - diag(l)|| + ||T'|| ||R||),
//        E_ij = (S_ij + l_j R_ij) / (l_j - l_i)  if |l_i - l_j| > delta,
//               R_ij / 2                          otherwise (and i = j),
//        Z <- Z + Z E,
//      which converges quadratically (three steps), then one symmetric
//      re-orthogonalisation Z <- Z (I + R/2).  The m x m products run as
//      8 x 8 tiles on many SMs and accumulate the norms of R and
//      S - diag(l) in their epilogues; E is formed element-wise on many SMs.
//   3. An FP64 Jacobi polish of Z^T T' Z, which after the refinement has
//      off-diagonal mass only inside clusters closer than the refinement
//      threshold: rotations act only on the rows with an entry above the
//      rounding floor of the product (none for a well separated spectrum).
//   4. Rayleigh quotients, one more re-orthogonalisation, ascending sort of
//      (l + mu, Z).
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "block_ops.h"
#include "common.cuh"
#include "reduce.cuh"

namespace iptgb {

namespace {

constexpr int kEigMax = 112;
constexpr int kEigPad = kEigMax + 1;
constexpr int kMaxTiles = 14 * 14;   // 8 x 8 tiles of a 112 x 112 product
constexpr int kMaxConvBlocks = 64;   // conversion CTAs (m*m / 256 <= 49)

__device__ __forceinline__ double warp_sum_d(double v)
{
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

__device__ __forceinline__ float warp_sum_f(float v)
{
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// ---------------------------------------------------------------------------
// 1a. Tp = sym(T) - mu I (FP64), Af = float(Tp); fro_part[block] = sum of
// Tp_ij^2; block 0 stores mu in *mu_out.
// ---------------------------------------------------------------------------
__global__ void eig_convert_kernel(const double *__restrict__ T, int m, double *__restrict__ Tp,
                                   float *__restrict__ Af, double *__restrict__ fro_part,
                                   double *__restrict__ mu_out)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    __shared__ double mu_sh;
    const int tid = threadIdx.x;
    if (tid < 32) {
        double s = 0.0;
        for (int i = tid; i < m; i += 32) s += T[(size_t)i * m + i];
        s = warp_sum_d(s);
        if (tid == 0) {
            mu_sh = s / m;
            if (blockIdx.x == 0) *mu_out = s / m;
        }
    }
    __syncthreads();
    const int e = blockIdx.x * blockDim.x + tid;
    double t2 = 0.0;
    if (e < m * m) {
        const int j = e / m;
        const int i = e - j * m;
        const double sym = 0.5 * (T[e] + T[(size_t)i * m + j]);
        const double t = i == j ? sym - mu_sh : sym;
        t2 = t * t;
        Tp[e] = t;
        Af[e] = (float)t;
    }
    const double2 s = block_sum2(t2, 0.0);
    if (tid == 0) fro_part[blockIdx.x] = s.x;
}

// ---------------------------------------------------------------------------
// 1b. Householder tridiagonalisation of the symmetric Af (one CTA, 512
// threads, four barriers per column).  Column j: v = x - alpha e1 with alpha = -sign(x0) ||x||,
// H_j = I - tau_j v v^T acting on rows j+1..m-1; the trailing block is
// updated as A <- A - v w^T - w v^T, w = p - (tau/2)(v^T p) v, p = tau A v.
// Outputs the diagonal d, off-diagonal e, reflectors vh (column j holds v
// in rows j+1..m-1) and tau.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(512)
eig_tridiag_kernel(const float *__restrict__ Af, int m, float *__restrict__ vh,
                   float *__restrict__ tau, float *__restrict__ d, float *__restrict__ e)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    extern __shared__ float A[];  // row-major, ld kEigPad
    __shared__ float vs[kEigMax];
    __shared__ float pp[4][kEigMax];
    __shared__ float ws[kEigMax];
    __shared__ float scal[2];
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    for (int x = tid; x < m * m; x += blockDim.x) {
        const int c = x / m;
        const int r = x - c * m;
        A[r * kEigPad + c] = Af[x];
    }
    __syncthreads();
    for (int j = 0; j + 2 < m; ++j) {
        const int L = m - j - 1;
        const int base = j + 1;
        if (warp == 0) {
            float sig = 0.f;
            for (int r = 1 + lane; r < L; r += 32) {
                const float x = A[(base + r) * kEigPad + j];
                sig = fmaf(x, x, sig);
            }
            sig = warp_sum_f(sig);
            const float x0 = A[base * kEigPad + j];
            float alpha = x0, t = 0.f, v0 = 1.f;
            if (sig > 0.f) {
                const float nrm = sqrtf(fmaf(x0, x0, sig));
                alpha = x0 >= 0.f ? -nrm : nrm;
                v0 = x0 - alpha;
                t = 2.f / fmaf(v0, v0, sig);
            }
            for (int r = lane; r < L; r += 32) {
                vs[r] = r == 0 ? v0 : A[(base + r) * kEigPad + j];
            }
            if (lane == 0) {
                scal[0] = alpha;
                scal[1] = t;
                d[j] = A[j * kEigPad + j];
                e[j] = alpha;
                tau[j] = t;
            }
        }
        __syncthreads();
        const float t = scal[1];
        for (int r = tid; r < L; r += blockDim.x) vh[(size_t)j * m + base + r] = vs[r];
        if (t != 0.f) {
            // p = tau A v, rows split over 4 groups of columns
            {
                const int r = tid & 127;
                const int g = tid >> 7;
                if (r < L) {
                    const int q = (L + 3) >> 2;
                    const int c0 = g * q;
                    const int c1 = min(L, c0 + q);
                    float s = 0.f;
                    const float *row = A + (base + r) * kEigPad + base;
                    for (int c = c0; c < c1; ++c) s = fmaf(row[c], vs[c], s);
                    pp[g][r] = s;
                }
            }
            __syncthreads();
            // w = p - K v with K = (tau/2) v^T p; warp 0 forms w in ws
            if (warp == 0) {
                float vp = 0.f;
                for (int r = lane; r < L; r += 32) {
                    const float p = t * (pp[0][r] + pp[1][r] + pp[2][r] + pp[3][r]);
                    ws[r] = p;
                    vp = fmaf(vs[r], p, vp);
                }
                const float K = 0.5f * t * warp_sum_f(vp);
                for (int r = lane; r < L; r += 32) ws[r] -= K * vs[r];
            }
            __syncthreads();
            for (int r = warp; r < L; r += nwarps) {
                const float vr = vs[r];
                const float wr = ws[r];
                float *row = A + (base + r) * kEigPad + base;
                for (int c = lane; c < L; c += 32) row[c] -= vr * ws[c] + wr * vs[c];
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (m >= 2) {
            d[m - 2] = A[(m - 2) * kEigPad + m - 2];
            e[m - 2] = A[(m - 1) * kEigPad + m - 2];
            tau[m - 2] = 0.f;
        }
        d[m - 1] = A[(m - 1) * kEigPad + m - 1];
    }
}

// ---------------------------------------------------------------------------
// 1c. Eigenvalues of the tridiagonal (d, e) by bisection and eigenvectors by
// inverse iteration, one CTA of 128 threads, thread i <-> eigenvalue i.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int sturm_count(const float *d, const float *e2, int m, float x,
                                           float pivmin)
{
    float q = d[0] - x;
    if (fabsf(q) < pivmin) q = -pivmin;
    int cnt = q < 0.f;
    for (int j = 1; j < m; ++j) {
        q = (d[j] - x) - __fdividef(e2[j - 1], q);
        if (fabsf(q) < pivmin) q = -pivmin;
        cnt += q < 0.f;
    }
    return cnt;
}

__device__ __forceinline__ float start_value(int i, int l)
{
    uint32_t h = (uint32_t)(i * 0x9E3779B1u) ^ (uint32_t)(l * 0x85EBCA77u + 0x27D4EB2Fu);
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return (float)(h & 0xFFFFu) * (1.f / 65536.f) + 0.25f;
}

size_t tri_vectors_smem_bytes(int m)
{
    return ((size_t)m * kEigPad + 3 * (size_t)m * m) * sizeof(float);
}

__global__ void __launch_bounds__(128)
eig_tri_vectors_kernel(const float *__restrict__ dg, const float *__restrict__ eg, int m,
                       float *__restrict__ Y, int *info)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    // Ys: the vectors, column-major with ld kEigPad (thread i's right-hand
    // side and solution live in column i); U0..U2: the U rows of every
    // thread's factorisation, element l of thread i at [l * m + i]
    extern __shared__ float Ys[];
    float *U0 = Ys + (size_t)m * kEigPad;
    float *U1 = U0 + (size_t)m * m;
    float *U2 = U1 + (size_t)m * m;
    __shared__ float d[kEigMax], e[kEigMax], e2[kEigMax], lam[kEigMax];
    __shared__ int cstart[kEigMax], csize[kEigMax];
    __shared__ int ncl;
    __shared__ float tnorm_sh, pivmin_sh, glo_sh, ghi_sh;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    for (int j = tid; j < m; j += blockDim.x) {
        d[j] = dg[j];
        const float ej = j + 1 < m ? eg[j] : 0.f;
        e[j] = ej;
        e2[j] = ej * ej;
    }
    __syncthreads();
    // Gershgorin interval; the tridiagonal is then scaled by 1 / its bound so
    // that the pivot floors below are independent of the matrix scale (a
    // zero matrix gives one cluster at 0 and an orthonormal basis)
    if (tid == 0) {
        float lo = INFINITY, hi = -INFINITY;
        for (int j = 0; j < m; ++j) {
            const float r = (j > 0 ? fabsf(e[j - 1]) : 0.f) + (j + 1 < m ? fabsf(e[j]) : 0.f);
            lo = fminf(lo, d[j] - r);
            hi = fmaxf(hi, d[j] + r);
        }
        const float bound = fmaxf(fabsf(lo), fabsf(hi));
        const float scale = bound > 0.f ? 1.f / bound : 1.f;
        tnorm_sh = scale;
        glo_sh = lo * scale;
        ghi_sh = hi * scale;
    }
    __syncthreads();
    {
        const float scale = tnorm_sh;
        for (int j = tid; j < m; j += blockDim.x) {
            d[j] *= scale;
            e[j] *= scale;
            e2[j] = e[j] * e[j];
        }
    }
    __syncthreads();
    if (tid == 0) {
        float emax = 0.f;
        for (int j = 0; j < m; ++j) emax = fmaxf(emax, e2[j]);
        pivmin_sh = FLT_MIN * fmaxf(1.f, emax);
    }
    __syncthreads();
    const float tnorm = 1.f;
    const float pivmin = pivmin_sh;
    if (tid < m) {
        float lo = glo_sh - 2.f * FLT_EPSILON * tnorm;
        float hi = ghi_sh + 2.f * FLT_EPSILON * tnorm;
        const float tol = 2.f * FLT_EPSILON * tnorm;
        for (int it = 0; it < 64 && hi - lo > tol; ++it) {
            const float mid = 0.5f * (lo + hi);
            if (mid <= lo || mid >= hi) break;
            if (sturm_count(d, e2, m, mid, pivmin) > tid) hi = mid;
            else lo = mid;
        }
        lam[tid] = 0.5f * (lo + hi);
    }
    __syncthreads();
    // clusters of eigenvalues closer than 1e-3 ||T||; members' shifts are
    // pulled apart to at least 10 eps ||T|| so their factorisations differ
    if (tid == 0) {
        int n = 0;
        const float gap = 1e-3f * tnorm;
        const float sep = 10.f * FLT_EPSILON * tnorm;
        for (int i = 0; i < m; ++i) {
            if (i == 0 || lam[i] - lam[i - 1] > gap) {
                cstart[n] = i;
                csize[n] = 1;
                ++n;
            } else {
                ++csize[n - 1];
                if (lam[i] < lam[i - 1] + sep) lam[i] = lam[i - 1] + sep;
            }
        }
        ncl = n;
        if (info != nullptr) *info = n;
    }
    __syncthreads();
    // inverse iteration: (Tri - lam I) y = b by Gaussian elimination with
    // partial pivoting (U rows hold up to three entries), tiny pivots
    // replaced by eps ||T||
    const float shift = tid < m ? lam[tid] : 0.f;
    const float tiny = FLT_EPSILON * tnorm;
    float *rhs = Ys + (size_t)(tid < m ? tid : 0) * kEigPad;
    if (tid < m) {
        for (int l = 0; l < m; ++l) rhs[l] = start_value(tid, l);
    }
    for (int it = 0; it < 3; ++it) {
        if (tid < m) {
            float *u0 = U0 + tid;
            float *u1 = U1 + tid;
            float *u2 = U2 + tid;
            float a = d[0] - shift;  // working row: a at col j, b at col j+1
            float b = m > 1 ? e[0] : 0.f;
            float w = rhs[0];
            for (int j = 0; j + 1 < m; ++j) {
                const float sub = e[j];
                const float dn = d[j + 1] - shift;
                const float sup = j + 2 < m ? e[j + 1] : 0.f;
                const float rn = rhs[j + 1];
                if (fabsf(a) >= fabsf(sub)) {
                    const float piv = fabsf(a) < tiny ? copysignf(tiny, a) : a;
                    const float lm = sub / piv;
                    u0[j * m] = piv;
                    u1[j * m] = b;
                    u2[j * m] = 0.f;
                    rhs[j] = w;
                    a = dn - lm * b;
                    b = sup;
                    w = rn - lm * w;
                } else {
                    const float lm = a / sub;
                    u0[j * m] = sub;
                    u1[j * m] = dn;
                    u2[j * m] = sup;
                    rhs[j] = rn;
                    a = b - lm * dn;
                    b = -lm * sup;
                    w = w - lm * rn;
                }
            }
            u0[(m - 1) * m] = fabsf(a) < tiny ? copysignf(tiny, a) : a;
            rhs[m - 1] = w;
            // back substitution, rescaled against overflow
            float ymax = 0.f;
            for (int j = m - 1; j >= 0; --j) {
                float s = rhs[j];
                if (j + 1 < m) s -= u1[j * m] * rhs[j + 1];
                if (j + 2 < m) s -= u2[j * m] * rhs[j + 2];
                const float y = s / u0[j * m];
                rhs[j] = y;
                ymax = fmaxf(ymax, fabsf(y));
                if (ymax > 1e30f) {
                    const float sc = 1.f / ymax;
                    for (int l = j; l < m; ++l) rhs[l] *= sc;
                    ymax = 1.f;
                }
            }
            const float sc = ymax > 0.f ? 1.f / ymax : 1.f;
            float nrm = 0.f;
            for (int l = 0; l < m; ++l) {
                rhs[l] *= sc;
                nrm = fmaf(rhs[l], rhs[l], nrm);
            }
            const float inv = nrm > 0.f ? rsqrtf(nrm) : 0.f;
            for (int l = 0; l < m; ++l) rhs[l] *= inv;
        }
        __syncthreads();
        // modified Gram-Schmidt inside each cluster, one warp per cluster
        for (int c = warp; c < ncl; c += blockDim.x >> 5) {
            const int s0 = cstart[c];
            const int sz = csize[c];
            for (int t = 1; t < sz; ++t) {
                float *ya = Ys + (s0 + t) * kEigPad;
                for (int s = 0; s < t; ++s) {
                    const float *yb = Ys + (s0 + s) * kEigPad;
                    float dot = 0.f;
                    for (int l = lane; l < m; l += 32) dot = fmaf(ya[l], yb[l], dot);
                    dot = warp_sum_f(dot);
                    for (int l = lane; l < m; l += 32) ya[l] -= dot * yb[l];
                    __syncwarp();
                }
                float nrm = 0.f;
                for (int l = lane; l < m; l += 32) nrm = fmaf(ya[l], ya[l], nrm);
                nrm = warp_sum_f(nrm);
                const float inv = nrm > 0.f ? rsqrtf(nrm) : 0.f;
                for (int l = lane; l < m; l += 32) ya[l] *= inv;
                __syncwarp();
            }
        }
        __syncthreads();
    }
    for (int x = tid; x < m * m; x += blockDim.x) {
        const int c = x / m;
        const int l = x - c * m;
        Y[x] = Ys[c * kEigPad + l];
    }
}

// ---------------------------------------------------------------------------
// 1d. Z0 = H_0 H_1 ... H_{m-3} Y: the reflectors are staged in shared memory
// (m*m + m floats), one warp per column, 8 columns per CTA.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
eig_backtransform_kernel(const float *__restrict__ Y, const float *__restrict__ vh,
                         const float *__restrict__ tau, int m, double *__restrict__ Z)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    extern __shared__ float vs_all[];
    float *ts = vs_all + (size_t)m * m;
    for (int x = threadIdx.x; x < m * m; x += blockDim.x) vs_all[x] = vh[x];
    for (int x = threadIdx.x; x < m; x += blockDim.x) ts[x] = x + 2 < m ? tau[x] : 0.f;
    __syncthreads();
    const int col = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (col >= m) return;
    const int lane = threadIdx.x & 31;
    float y[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int l = lane + 32 * t;
        y[t] = l < m ? Y[(size_t)col * m + l] : 0.f;
    }
    for (int j = m - 3; j >= 0; --j) {
        const float tj = ts[j];
        if (tj == 0.f) continue;
        float v[4];
        float dot = 0.f;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int l = lane + 32 * t;
            v[t] = (l > j && l < m) ? vs_all[j * m + l] : 0.f;
            dot = fmaf(v[t], y[t], dot);
        }
        dot = tj * warp_sum_f(dot);
#pragma unroll
        for (int t = 0; t < 4; ++t) y[t] -= dot * v[t];
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int l = lane + 32 * t;
        if (l < m) Z[(size_t)col * m + l] = (double)y[t];
    }
}

// ---------------------------------------------------------------------------
// Small FP64 GEMMs, up to two independent jobs per launch (blockIdx.z):
// C = op(A) B (+ D), all m x m column-major.  8 x 8 output tile per 64-thread
// CTA with the 8 x m panel of op(A) and the m x 8 panel of B in shared
// memory, so an m = 96 product spreads over 144 CTAs.  Optional epilogue
// statistics, one FP64 partial per tile: stats = 1 sums (delta_ij - C_ij)^2
// (the refinement's R), stats = 2 sums (C_ij - delta_ij C_ii / Gd_ii)^2
// (S - diag(l)).
// ---------------------------------------------------------------------------
struct SmallGemmJob {
    const double *A;
    const double *B;
    const double *D;   // added when non-null (may alias A or B, never C)
    double *C;
    int transA;
    int stats;
    const double *Gd;  // stats = 2: the Gram matrix of the same vectors
    double *part;      // stats != 0: per-tile partial sums
};

__global__ void __launch_bounds__(64)
small_gemm64_kernel(SmallGemmJob j0, SmallGemmJob j1, int m)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    __shared__ double As[8][kEigPad];
    __shared__ double Bs[kEigMax][9];
    __shared__ double red[2];
    const SmallGemmJob &job = blockIdx.z == 0 ? j0 : j1;
    const int i0 = blockIdx.x * 8;
    const int jb = blockIdx.y * 8;
    const int tid = threadIdx.x;
    if (job.transA) {
        for (int x = tid; x < 8 * m; x += 64) {
            const int r = x / m;
            const int l = x - r * m;
            As[r][l] = i0 + r < m ? job.A[(size_t)(i0 + r) * m + l] : 0.0;
        }
    } else {
        for (int x = tid; x < 8 * m; x += 64) {
            const int l = x >> 3;
            const int r = x & 7;
            As[r][l] = i0 + r < m ? job.A[(size_t)l * m + i0 + r] : 0.0;
        }
    }
    for (int x = tid; x < 8 * m; x += 64) {
        const int c = x / m;
        const int l = x - c * m;
        Bs[l][c] = jb + c < m ? job.B[(size_t)(jb + c) * m + l] : 0.0;
    }
    __syncthreads();
    const int r = tid & 7;
    const int c = tid >> 3;
    double s = 0.0;
    for (int l = 0; l < m; ++l) s = fma(As[r][l], Bs[l][c], s);
    const int i = i0 + r;
    const int j = jb + c;
    double st = 0.0;
    if (i < m && j < m) {
        const size_t o = (size_t)j * m + i;
        if (job.D != nullptr) s += job.D[o];
        job.C[o] = s;
        if (job.stats == 1) {
            const double rr = (i == j ? 1.0 : 0.0) - s;
            st = rr * rr;
        } else if (job.stats == 2) {
            const double dv = i == j ? s - s / job.Gd[o] : s;
            st = dv * dv;
        }
    }
    if (job.stats != 0) {
        st = warp_sum_d(st);
        if ((tid & 31) == 0) red[tid >> 5] = st;
        __syncthreads();
        if (tid == 0) job.part[blockIdx.y * gridDim.x + blockIdx.x] = red[0] + red[1];
    }
}

// ---------------------------------------------------------------------------
// 2. E from G, S and the partial norms (every CTA sums the partials in the
// same order, so delta is identical everywhere).  Besides the published gap
// test |l_i - l_j| > delta, a pair whose first-order rotation would exceed
// `ebound` is also treated as clustered (orthogonalised only), so every
// applied update is small; the FP64 Jacobi polish resolves the pairs left
// coupled.  ebound = 0 gives the pure orthogonalisation E = R / 2
// (Z <- Z (I + R/2), a first-order Z (Z^T Z)^{-1/2}).  Block 0 writes the
// eigenvalue estimates l.
// ---------------------------------------------------------------------------
__global__ void oa_e_kernel(const double *__restrict__ G, const double *__restrict__ S,
                            const double *__restrict__ fro_part, int nfro,
                            const double *__restrict__ r_part, const double *__restrict__ s_part,
                            int ntiles, int m, double ebound, double *__restrict__ E,
                            double *__restrict__ lam)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    __shared__ double delta_sh;
    const int tid = threadIdx.x;
    if (tid < 32) {
        double f = 0.0, rr = 0.0, ss = 0.0;
        for (int x = tid; x < nfro; x += 32) f += fro_part[x];
        for (int x = tid; x < ntiles; x += 32) {
            rr += r_part[x];
            ss += s_part[x];
        }
        f = warp_sum_d(f);
        rr = warp_sum_d(rr);
        ss = warp_sum_d(ss);
        if (tid == 0) delta_sh = 2.0 * (sqrt(ss) + sqrt(f) * sqrt(rr));
    }
    __syncthreads();
    if (blockIdx.x == 0) {
        for (int i = tid; i < m; i += blockDim.x) {
            const size_t o = (size_t)i * m + i;
            lam[i] = S[o] / G[o];
        }
    }
    const int x = blockIdx.x * blockDim.x + tid;
    if (x >= m * m) return;
    const int j = x / m;
    const int i = x - j * m;
    const double r = (i == j ? 1.0 : 0.0) - G[x];
    double val = 0.5 * r;
    if (i != j && ebound > 0.0) {
        const double li = S[(size_t)i * m + i] / G[(size_t)i * m + i];
        const double lj = S[(size_t)j * m + j] / G[(size_t)j * m + j];
        const double gap = lj - li;
        if (fabs(gap) > delta_sh) {
            const double num = S[x] + lj * r;
            // the transposed entry's numerator, for a symmetric decision
            const double num_t = S[(size_t)i * m + j] + li * r;
            if (fmax(fabs(num), fabs(num_t)) <= ebound * fabs(gap)) {
                val = num / gap;
            }
        }
    }
    E[x] = val;
}

// ---------------------------------------------------------------------------
// 3. FP64 Jacobi polish of a nearly diagonal symmetric matrix (one CTA, 512
// threads).  Off-diagonal entries at or below the rounding floor of a
// length-m FP64 product, 4 sqrt(m) eps ||T||_F, are treated as zero, so the
// rotations act only on the index set I of rows with an entry above it:
// cyclic Jacobi runs on the principal submatrix T[I, I] (2 barriers per
// round: the c/2 disjoint rotations of a round are computed, then each
// thread rotates its own 2x2 blocks of B and column pairs of V) and W is the
// identity outside I x I.  Dynamic smem: C*(C+1) + C*C + 2*C doubles + 2*C +
// m ints, C = m rounded up to even.  *applied = |I|.
// ---------------------------------------------------------------------------
size_t polish_smem_bytes(int m)
{
    const size_t M = (size_t)((m + 1) & ~1);
    return (M * (M + 1) + M * M + 2 * M) * sizeof(double) + (2 * M + m) * sizeof(int);
}

__global__ void __launch_bounds__(512)
jacobi_polish_kernel(const double *__restrict__ T, int m, double *__restrict__ W,
                     int max_sweeps, int *applied)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    extern __shared__ unsigned char sm_raw[];
    const int Mfull = (m + 1) & ~1;
    double *B = reinterpret_cast<double *>(sm_raw);  // row-major, ld C+1
    double *V = B + (size_t)Mfull * (Mfull + 1);      // column-major, ld C
    double *cs = V + (size_t)Mfull * Mfull;           // c[half], s[half]
    int *pr = (int *)(cs + Mfull);                    // p[half], q[half]
    int *idx = pr + Mfull;                            // I, then flags
    __shared__ double fro_sh;
    __shared__ int flag[kEigMax];
    __shared__ int c_sh, n_above;
    const int tid = threadIdx.x;
    const int nt = blockDim.x;
    double fro = 0.0;
    for (int x = tid; x < m * m; x += nt) {
        const double t = T[x];
        fro += t * t;
    }
    for (int i = tid; i < m; i += nt) flag[i] = 0;
    const double2 f = block_sum2(fro, 0.0);
    if (tid == 0) fro_sh = f.x;
    __syncthreads();
    const double floor_ = 4.0 * sqrt((double)m) * 1.1102230246251565e-16 * sqrt(fro_sh) + 1e-300;
    for (int x = tid; x < m * m; x += nt) {
        const int j = x / m;
        const int i = x - j * m;
        if (i < j && fabs(0.5 * (T[x] + T[(size_t)i * m + j])) > floor_) {
            flag[i] = 1;
            flag[j] = 1;
        }
    }
    __syncthreads();
    if (tid == 0) {
        int c = 0;
        for (int i = 0; i < m; ++i) {
            if (flag[i]) idx[c++] = i;
        }
        c_sh = c;
    }
    for (int x = tid; x < m * m; x += nt) {
        const int j = x / m;
        const int i = x - j * m;
        W[x] = i == j ? 1.0 : 0.0;
    }
    __syncthreads();
    const int c = c_sh;
    if (tid == 0 && applied != nullptr) *applied = c;
    if (c == 0) return;
    const int M = (c + 1) & ~1;
    const int LB = M + 1;
    const int half = M / 2;
    for (int x = tid; x < M * M; x += nt) {
        const int a = x / M;
        const int b = x - a * M;
        double v = 0.0;
        if (a < c && b < c) {
            const size_t ia = idx[a], ib = idx[b];
            v = 0.5 * (T[ib * m + ia] + T[ia * m + ib]);
        }
        B[a * LB + b] = v;
        V[b * M + a] = a == b ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        if (tid == 0) n_above = 0;
        __syncthreads();
        int above = 0;
        for (int x = tid; x < M * M; x += nt) {
            const int a = x / M;
            const int b = x - a * M;
            above += (a != b) && fabs(B[a * LB + b]) > floor_;
        }
        if (above) atomicAdd(&n_above, above);
        __syncthreads();
        if (n_above == 0) break;
        for (int r = 0; r < M - 1; ++r) {
            for (int k = tid; k < half; k += nt) {
                int p, q;
                if (k == 0) {
                    p = M - 1;
                    q = r;
                } else {
                    p = (r + k) % (M - 1);
                    q = (r - k + M - 1) % (M - 1);
                }
                if (p > q) {
                    const int tmp = p;
                    p = q;
                    q = tmp;
                }
                double cc = 1.0, ss = 0.0;
                const double apq = B[p * LB + q];
                if (q < c && fabs(apq) > floor_) {
                    const double theta = (B[q * LB + q] - B[p * LB + p]) / (2.0 * apq);
                    const double tt = (theta >= 0.0 ? 1.0 : -1.0) /
                                      (fabs(theta) + sqrt(theta * theta + 1.0));
                    cc = 1.0 / sqrt(tt * tt + 1.0);
                    ss = tt * cc;
                }
                cs[k] = cc;
                cs[half + k] = ss;
                pr[k] = p;
                pr[half + k] = q;
            }
            __syncthreads();
            for (int x = tid; x < half * half; x += nt) {
                const int kr = x / half;
                const int kc = x - kr * half;
                const double sr = cs[half + kr];
                const double sc = cs[half + kc];
                if (sr == 0.0 && sc == 0.0) continue;
                const double cr = cs[kr], cc = cs[kc];
                const int prw = pr[kr], qrw = pr[half + kr];
                const int pc = pr[kc], qc = pr[half + kc];
                const double a = B[prw * LB + pc], b = B[prw * LB + qc];
                const double c2 = B[qrw * LB + pc], dd = B[qrw * LB + qc];
                const double a1 = cc * a - sc * b, b1 = sc * a + cc * b;
                const double c1 = cc * c2 - sc * dd, d1 = sc * c2 + cc * dd;
                B[prw * LB + pc] = cr * a1 - sr * c1;
                B[prw * LB + qc] = cr * b1 - sr * d1;
                B[qrw * LB + pc] = sr * a1 + cr * c1;
                B[qrw * LB + qc] = sr * b1 + cr * d1;
            }
            for (int x = tid; x < half * M; x += nt) {
                const int kc = x / M;
                const double sn = cs[half + kc];
                if (sn == 0.0) continue;
                const int l = x - kc * M;
                const double cn = cs[kc];
                const int p = pr[kc], q = pr[half + kc];
                const double vp = V[p * M + l], vq = V[q * M + l];
                V[p * M + l] = cn * vp - sn * vq;
                V[q * M + l] = sn * vp + cn * vq;
            }
            __syncthreads();
        }
    }
    // W[I, I] = V (W was set to the identity above)
    for (int x = tid; x < c * c; x += nt) {
        const int b = x / c;
        const int a = x - b * c;
        W[(size_t)idx[b] * m + idx[a]] = V[b * M + a];
    }
}

// 4. ascending sort of (lam + mu, Z) into (w, Zout).  Keys are the
// order-preserving integer images of the doubles; ties keep the input order.
__device__ __forceinline__ long long sort_key(double x)
{
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

__global__ void eig_sort_kernel(const double *__restrict__ lam, const double *__restrict__ mu,
                                const double *__restrict__ Zin, int m, double *__restrict__ w,
                                double *__restrict__ Zout)
{
    pdl_wait();  // programmatic dependent launch: predecessor done
    pdl_trigger();
    __shared__ long long keys[kEigMax];
    __shared__ int rank_sh[kEigMax];
    const int tid = threadIdx.x;
    for (int i = tid; i < m; i += blockDim.x) keys[i] = sort_key(lam[i]);
    __syncthreads();
    for (int i = tid; i < m; i += blockDim.x) {
        const long long ki = keys[i];
        int rank = 0;
        for (int j = 0; j < m; ++j) {
            const long long kj = keys[j];
            rank += (kj < ki) || (kj == ki && j < i);
        }
        rank_sh[i] = rank;
        w[rank] = lam[i] + *mu;
    }
    __syncthreads();
    for (int x = tid; x < m * m; x += blockDim.x) {
        const int i = x / m;
        const int l = x - i * m;
        Zout[(size_t)rank_sh[i] * m + l] = Zin[x];
    }
}

}  // namespace

int BlockOps::symmetric_eig(const double *T, int m, double *w, double *Z, int *info_dev)
{
    if (m <= 0 || m > kEigMax) {  // the FP64 polish keeps two m x m matrices in shared memory
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    const size_t mm = (size_t)m * m;
    const size_t nfloat = 3 * mm + 3 * (size_t)m;
    const size_t need = 8 * mm + m + kMaxConvBlocks + 2 * kMaxTiles + (nfloat + 1) / 2;
    if (eig_capacity < need) {
        if (eig_scratch != nullptr) {
            cudaFreeAsync(eig_scratch, stream);
            eig_scratch = nullptr;
        }
        IPTGB_CUDA(cudaMallocAsync((void **)&eig_scratch, need * sizeof(double), stream));
        eig_capacity = need;
    }
    double *Tp = eig_scratch;
    double *Z0 = Tp + mm;
    double *Z1 = Z0 + mm;
    double *G = Z1 + mm;
    double *TZ = G + mm;
    double *S = TZ + mm;
    double *E = S + mm;
    double *W = E + mm;
    double *lam = W + mm;
    double *fro_part = lam + m;
    double *mu_dev = fro_part + kMaxConvBlocks - 1;  // the last slot holds mu
    double *r_part = fro_part + kMaxConvBlocks;
    double *s_part = r_part + kMaxTiles;
    float *Af = reinterpret_cast<float *>(s_part + kMaxTiles);
    float *vh = Af + mm;
    float *Yf = vh + mm;
    float *tau = Yf + mm;
    float *dg = tau + m;
    float *eg = dg + m;
    KernelTimerScope timer(kProfSmallEig, stream);

    // 1. FP32 eigenvectors of T'
    const int cgrid = blocks_for(mm);
    IPTGB_CHECK(launch_pdl(eig_convert_kernel, dim3(cgrid), dim3(kThreads), 0, stream, T, m, Tp, Af,
                           fro_part, mu_dev));
    const size_t tri_smem = (size_t)m * kEigPad * sizeof(float);
    IPTGB_CUDA(cudaFuncSetAttribute(eig_tridiag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)tri_smem));
    IPTGB_CHECK(launch_pdl(eig_tridiag_kernel, dim3(1), dim3(512), tri_smem, stream, Af, m, vh,
                           tau, dg, eg));
    const size_t vec_smem = tri_vectors_smem_bytes(m);
    IPTGB_CUDA(cudaFuncSetAttribute(eig_tri_vectors_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)vec_smem));
    IPTGB_CHECK(launch_pdl(eig_tri_vectors_kernel, dim3(1), dim3(128), vec_smem, stream, dg, eg, m,
                           Yf, info_dev));
    const size_t bt_smem = ((size_t)m * m + m) * sizeof(float);
    IPTGB_CUDA(cudaFuncSetAttribute(eig_backtransform_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bt_smem));
    IPTGB_CHECK(launch_pdl(eig_backtransform_kernel, dim3((m + 7) / 8), dim3(256), bt_smem, stream,
                           Yf, vh, tau, m, Z0));

    // 2. FP64 refinement on T'
    const int tiles = (m + 7) / 8;
    const int ntiles = tiles * tiles;
    const int egrid = blocks_for(mm);
    auto gemm = [&](SmallGemmJob a, SmallGemmJob b, int count) -> int {
        return launch_pdl(small_gemm64_kernel, dim3(tiles, tiles, count), dim3(64), 0, stream, a,
                          b, m);
    };
    auto refine_step = [&](double *cur, double *nxt, double ebound) -> int {
        IPTGB_CHECK((gemm({cur, cur, nullptr, G, 1, 1, nullptr, r_part},      // G = Z^T Z, ||R||
                          {Tp, cur, nullptr, TZ, 0, 0, nullptr, nullptr}, 2)));  // TZ = T' Z
        IPTGB_CHECK((gemm({cur, TZ, nullptr, S, 1, 2, G, s_part}, {}, 1)));  // S = Z^T T' Z
        IPTGB_CHECK(launch_pdl(oa_e_kernel, dim3(egrid), dim3(kThreads), 0, stream, G, S,
                               fro_part, cgrid, r_part, s_part, ntiles, m, ebound, E, lam));
        IPTGB_CHECK((gemm({cur, E, cur, nxt, 0, 0, nullptr, nullptr}, {}, 1)));  // Z <- Z + Z E
        return IPT_CUDA_SUCCESS;
    };
    // a rotation bound of a few 1e-3 keeps every applied update small; pairs
    // above it are left to the polish
    const double ebounds[4] = {3e-3, 1e-3, 1e-3, 0.0};
    double *cur = Z0;
    double *nxt = Z1;
    for (int it = 0; it < 4; ++it) {
        IPTGB_CHECK(refine_step(cur, nxt, ebounds[it]));
        double *t = cur;
        cur = nxt;
        nxt = t;
    }
    // 3. FP64 Jacobi polish of Z^T T' Z, folded into Z
    IPTGB_CHECK((gemm({Tp, cur, nullptr, TZ, 0, 0, nullptr, nullptr}, {}, 1)));
    IPTGB_CHECK((gemm({cur, TZ, nullptr, S, 1, 0, nullptr, nullptr}, {}, 1)));
    const size_t pol_smem = polish_smem_bytes(m);
    IPTGB_CUDA(cudaFuncSetAttribute(jacobi_polish_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pol_smem));
    IPTGB_CHECK(launch_pdl(jacobi_polish_kernel, dim3(1), dim3(512), pol_smem, stream, S, m, W,
                           30, nullptr));
    IPTGB_CHECK((gemm({cur, W, nullptr, nxt, 0, 0, nullptr, nullptr}, {}, 1)));
    // 4. Rayleigh quotients of the polished vectors and one symmetric
    // re-orthogonalisation, then the sort
    IPTGB_CHECK(refine_step(nxt, cur, 0.0));
    IPTGB_CHECK(launch_pdl(eig_sort_kernel, dim3(1), dim3(256), 0, stream, lam, mu_dev, cur, m, w,
                           Z));
    return IPT_CUDA_SUCCESS;
}

}  // namespace iptgb
