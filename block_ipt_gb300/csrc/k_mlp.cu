// k_mlp.cu - learned Davidson preconditioner: a per-row MLP (6 -> 64 -> 64
// -> 1, ReLU) that replaces the plain diagonal correction
// t_i = r_i / (d_i - theta) of the reference's Davidson step
// (IPT_C_GPU/src/ipt_cuda.cu:2449-2465, clip rule :3389-3403).
//
// The exact correction of a Ritz pair (theta, x, r) is (H - theta)^-1 r; with
// H = D + Delta its Neumann series starts t1 + u with the plain correction
// t1 = (D - theta)^-1 r and the second-order term u = -(D - theta)^-1 Delta t1,
// which costs one product with H (H t1, the diagonal part taken off).  The
// learned correction is t_i = t1_i + o_i u_i with the network's per-row
// weight o_i = sigmoid(z_i), z_i its linear output: o -> 1 everywhere is the
// two-term Neumann correction, near which training starts (output bias 4:
// o = 0.982), o -> 0 the plain preconditioner.  The two-term correction is
// a strong baseline on the FCI-like family (it saves about 40 % of the
// Davidson steps of the plain one); the network learns per row how much of
// the second-order term to keep, never more than all of it.  Features of
// row i, all O(1):
//   f0 = t1_i sqrt(n) / ||t1||       plain correction, normalised
//   f1 = u_i sqrt(n) / ||t1||        second-order term, same units
//   f2 = x_i sqrt(n)                 Ritz vector (unit norm)
//   f3 = asinh((d_i - theta) / s_i)  gap in units of the row's off-diagonal
//                                    coupling s_i = ||H[i, j != i]||_2
//   f4 = asinh(s_i / (|d_i - theta| + clip))
//   f5 = log10(||r|| / max(1, ||H||_inf)) / 8   convergence level
//
// Training target (what the collector records while the plain solver runs
// against the converged eigenvectors x*): the part of the exact error that
// lies outside the current search space V, e = (I - V V^T)(s x*_l - x)
// (x*_l the converged vector that overlaps x most, s its sign), scaled by
// the least-squares fit e ~ alpha (I - V V^T)(t1 + u).  Davidson keeps only
// the part of a correction outside V, so the targets compare projected
// vectors: with p = (I - V V^T) t1 and q = (I - V V^T) u, per row the weight
// that reproduces the scaled error, y_i = (e_i / alpha - p_i) / q_i, with
// weight w_i = n q_i^2 / ||t1||^2, so that the weighted loss
// sum_i w_i (o_i - y_i)^2 equals ||p + o o q - e / alpha||^2 in the units
// of f1: for o = 1 (the two-term correction) and o = 0 (the plain one) it is
// the error of exactly the direction the Davidson step adds.  (Comparing the
// unprojected t1 + o u instead ranks the two-term correction below the plain
// one, although it saves Davidson steps: its components inside V count
// against it there and are discarded by the step.)
//
// Training runs on the GPU: a fused forward/backward kernel over 128-row
// tiles of a batch (per-tile gradient partials, no atomics) and an Adam
// kernel that sums the partials in a fixed order, so a training run is
// deterministic for a given seed.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "block_ops.h"
#include "block_solver.h"
#include "common.cuh"
#include "ipt_plain.h"
#include "reduce.cuh"

namespace iptgb {
namespace mlp {

constexpr int kIn = 6;
constexpr int kH = 64;
constexpr int kRow = kIn + 2;  // features, target, weight
constexpr int oW1 = 0;
constexpr int oB1 = oW1 + kH * kIn;
constexpr int oW2 = oB1 + kH;
constexpr int oB2 = oW2 + kH * kH;
constexpr int oW3 = oB2 + kH;
constexpr int oB3 = oW3 + kH;
constexpr int kParams = oB3 + 1;  // 4673
constexpr int kTile = 128;        // rows per CTA of the training kernel
constexpr int kLd = kH + 1;

__host__ __device__ constexpr int param_count() { return kParams; }

__device__ __forceinline__ unsigned long long splitmix(unsigned long long x)
{
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

__device__ __forceinline__ float clampf(float v, float lim)
{
    if (!(v == v)) return 0.f;  // NaN
    return fminf(fmaxf(v, -lim), lim);
}


__device__ __forceinline__ void row_features(double t, double tn, double u, double rn, double x,
                                             double delta, double sigma, double clip,
                                             double hnorm, int n, float f[kIn])
{
    const double sn = sqrt((double)n);
    f[0] = clampf((float)(tn > 0.0 ? t * sn / tn : 0.0), 40.f);
    f[1] = clampf((float)(tn > 0.0 ? u * sn / tn : 0.0), 40.f);
    f[2] = clampf((float)(x * sn), 40.f);
    const double s = sigma + 1e-12 * fmax(1.0, fabs(hnorm));
    f[3] = clampf((float)asinh(delta / s), 40.f);
    f[4] = clampf((float)asinh(sigma / (fabs(delta) + clip)), 40.f);
    f[5] = clampf((float)(log10(rn / fmax(1.0, hnorm) + 1e-300) / 8.0), 40.f);
}

// Weight of the second-order term from the network's linear output z.
constexpr float kOutBias = 4.f;  // initial z: o = sigmoid(4) = 0.982
__device__ __forceinline__ float weight_of(float z) { return 1.f / (1.f + expf(-z)); }

// o = sigmoid(z), z = W3 relu(W2 relu(W1 f + b1) + b2) + b3, with the
// parameters in shared memory
__device__ __forceinline__ float forward_row(const float *__restrict__ P, const float f[kIn])
{
    float h1[kH];
#pragma unroll
    for (int j = 0; j < kH; ++j) {
        float s = P[oB1 + j];
#pragma unroll
        for (int q = 0; q < kIn; ++q) s = fmaf(P[oW1 + j * kIn + q], f[q], s);
        h1[j] = fmaxf(s, 0.f);
    }
    float o = P[oB3];
    for (int j = 0; j < kH; ++j) {
        const float4 *w = reinterpret_cast<const float4 *>(P + oW2 + j * kH);
        float s = P[oB2 + j];
#pragma unroll
        for (int l4 = 0; l4 < kH / 4; ++l4) {
            const float4 ww = w[l4];
            s = fmaf(ww.x, h1[4 * l4 + 0], s);
            s = fmaf(ww.y, h1[4 * l4 + 1], s);
            s = fmaf(ww.z, h1[4 * l4 + 2], s);
            s = fmaf(ww.w, h1[4 * l4 + 3], s);
        }
        o = fmaf(P[oW3 + j], fmaxf(s, 0.f), o);
    }
    return weight_of(o);
}

__device__ __forceinline__ void load_params(const float *__restrict__ g, float *s)
{
    for (int p = threadIdx.x; p < kParams; p += blockDim.x) s[p] = g[p];
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Initialisation: weights U(-a, a) with a = sqrt(6 / fan_in) (ReLU layers) and
// 0.1 sqrt(3 / fan_in) (linear output), hidden biases 0, output bias
// kOutBias (so o starts near 1, the two-term correction); counter-based,
// seeded.
// ---------------------------------------------------------------------------
__global__ void mlp_init_kernel(float *__restrict__ params, unsigned long long seed)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kParams) return;
    float a = 0.f;
    if (p < oB1) a = sqrtf(6.f / kIn);
    else if (p >= oW2 && p < oB2) a = sqrtf(6.f / kH);
    else if (p >= oW3 && p < oB3) a = 0.1f * sqrtf(3.f / kH);
    const unsigned long long h = splitmix(seed * 0x100000001B3ULL + (unsigned long long)p);
    const float u = (float)((h >> 11) * (1.0 / 9007199254740992.0));  // [0, 1)
    params[p] = p == oB3 ? kOutBias : a * (2.f * u - 1.f);
}

// ---------------------------------------------------------------------------
// Inference on stored feature rows (row stride `ld` floats): out[r] = MLP(f).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
mlp_forward_rows_kernel(const float *__restrict__ params, const float *__restrict__ rows,
                        long long nrows, int ld, float *__restrict__ out)
{
    __shared__ __align__(16) float P[kParams + 3];
    load_params(params, P);
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    float f[kIn];
#pragma unroll
    for (int q = 0; q < kIn; ++q) f[q] = rows[r * ld + q];
    out[r] = forward_row(P, f);
}

// ---------------------------------------------------------------------------
// Fused forward + backward over one 128-row tile of a batch.  Loss: mean
// over the batch of w (o - y)^2 with o = sigmoid(z) (row = f0..f5, y, w).  Row b of the batch is row b of `rows`
// (sample = 0) or a seeded hash of (seed, step, b) modulo nrows (sample = 1).
// partials[tile][p] = d loss / d param_p restricted to the tile, and
// partials[tile][kParams] = the tile's sum of weighted squared errors.
// Dynamic smem: kParams + 4 * kTile * kLd + kTile * (kIn + 1) floats.
// ---------------------------------------------------------------------------
size_t fwd_bwd_smem_bytes()
{
    return ((size_t)kParams + 3 + 4 * (size_t)kTile * kLd + (size_t)kTile * (kIn + 1)) * sizeof(float);
}

__global__ void __launch_bounds__(kTile)
mlp_fwd_bwd_kernel(const float *__restrict__ params, const float *__restrict__ rows,
                   long long nrows, int batch, int sample, unsigned long long seed, int step,
                   float *__restrict__ partials)
{
    extern __shared__ __align__(16) float sm[];
    float *P = sm;                                // kParams (+3 pad)
    float *H1 = P + kParams + 3;                  // [kTile][kLd]
    float *H2 = H1 + kTile * kLd;
    float *D1 = H2 + kTile * kLd;
    float *D2 = D1 + kTile * kLd;
    float *F = D2 + kTile * kLd;                  // [kTile][kIn]
    float *dO = F + kTile * kIn;                  // [kTile]
    __shared__ float sq[kTile];
    load_params(params, P);
    const int t = threadIdx.x;
    const int b = blockIdx.x * kTile + t;
    const bool valid = b < batch;
    float f[kIn] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float y = 0.f, wgt = 0.f;
    if (valid) {
        long long r = b;
        if (sample) {
            const unsigned long long h =
                splitmix(seed ^ ((unsigned long long)step << 32) ^ (unsigned long long)b);
            r = (long long)(h % (unsigned long long)nrows);
        }
#pragma unroll
        for (int q = 0; q < kIn; ++q) f[q] = rows[r * kRow + q];
        y = rows[r * kRow + kIn];
        wgt = rows[r * kRow + kIn + 1];
    }
    // forward, keeping the activations of the tile in shared memory
    float *h1 = H1 + t * kLd;
    float *h2 = H2 + t * kLd;
#pragma unroll 4
    for (int j = 0; j < kH; ++j) {
        float s = P[oB1 + j];
#pragma unroll
        for (int q = 0; q < kIn; ++q) s = fmaf(P[oW1 + j * kIn + q], f[q], s);
        h1[j] = fmaxf(s, 0.f);
    }
    float o = P[oB3];
    for (int j = 0; j < kH; ++j) {
        float s = P[oB2 + j];
        for (int l = 0; l < kH; ++l) s = fmaf(P[oW2 + j * kH + l], h1[l], s);
        h2[j] = fmaxf(s, 0.f);
        o = fmaf(P[oW3 + j], h2[j], o);
    }
    const float sg = weight_of(o);
    const float err = valid ? sg - y : 0.f;
    // d loss / d z through o = sigmoid(z)
    const float g = valid ? 2.f * wgt * err * sg * (1.f - sg) / (float)batch : 0.f;
    dO[t] = g;
    sq[t] = wgt * err * err;
#pragma unroll
    for (int q = 0; q < kIn; ++q) F[t * kIn + q] = f[q];
    // backward through the tile's rows
    float *d2 = D2 + t * kLd;
    float *d1 = D1 + t * kLd;
    for (int j = 0; j < kH; ++j) d2[j] = h2[j] > 0.f ? P[oW3 + j] * g : 0.f;
    for (int l = 0; l < kH; ++l) {
        float s = 0.f;
        for (int j = 0; j < kH; ++j) s = fmaf(P[oW2 + j * kH + l], d2[j], s);
        d1[l] = h1[l] > 0.f ? s : 0.f;
    }
    __syncthreads();
    // tile gradients
    float *out = partials + (size_t)blockIdx.x * (kParams + 1);
    {
        // dW2[j][l] = sum_t D2[t][j] H1[t][l]; thread -> j = t / 2, 32 l's
        const int j = t >> 1;
        const int l0 = (t & 1) * 32;
        float acc[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) acc[q] = 0.f;
        for (int r = 0; r < kTile; ++r) {
            const float dj = D2[r * kLd + j];
            const float *hr = H1 + r * kLd + l0;
#pragma unroll
            for (int q = 0; q < 32; ++q) acc[q] = fmaf(dj, hr[q], acc[q]);
        }
#pragma unroll
        for (int q = 0; q < 32; ++q) out[oW2 + j * kH + l0 + q] = acc[q];
    }
    for (int p = t; p < kH * kIn; p += kTile) {
        const int j = p / kIn;
        const int q = p - j * kIn;
        float s = 0.f;
        for (int r = 0; r < kTile; ++r) s = fmaf(D1[r * kLd + j], F[r * kIn + q], s);
        out[oW1 + p] = s;
    }
    if (t < kH) {
        float s1 = 0.f, s2 = 0.f, s3 = 0.f;
        for (int r = 0; r < kTile; ++r) {
            s1 += D1[r * kLd + t];
            s2 += D2[r * kLd + t];
            s3 = fmaf(dO[r], H2[r * kLd + t], s3);
        }
        out[oB1 + t] = s1;
        out[oB2 + t] = s2;
        out[oW3 + t] = s3;
    } else if (t == kH) {
        float s = 0.f;
        for (int r = 0; r < kTile; ++r) s += dO[r];
        out[oB3] = s;
    } else if (t == kH + 1) {
        float s = 0.f;
        for (int r = 0; r < kTile; ++r) s += sq[r];
        out[kParams] = s;
    }
}

// Sum of the tile partials in tile order: grad[p] (p < kParams) and
// grad[kParams] = the batch loss.
__global__ void mlp_grad_finish_kernel(const float *__restrict__ partials, int tiles, int batch,
                                       float *__restrict__ grad)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > kParams) return;
    float s = 0.f;
    for (int b = 0; b < tiles; ++b) s += partials[(size_t)b * (kParams + 1) + p];
    grad[p] = p == kParams ? s / (float)batch : s;
}

// Adam (Kingma & Ba 2015): m = b1 m + (1-b1) g, v = b2 v + (1-b2) g^2,
// p -= lr m_hat / (sqrt(v_hat) + eps); step is 1-based.
__global__ void mlp_adam_kernel(float *__restrict__ params, float *__restrict__ m,
                                float *__restrict__ v, const float *__restrict__ partials,
                                int tiles, int batch, int step, float lr,
                                float *__restrict__ loss_hist)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > kParams) return;
    float g = 0.f;
    for (int b = 0; b < tiles; ++b) g += partials[(size_t)b * (kParams + 1) + p];
    if (p == kParams) {
        if (loss_hist != nullptr) loss_hist[step - 1] = g / (float)batch;
        return;
    }
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float mm = b1 * m[p] + (1.f - b1) * g;
    const float vv = b2 * v[p] + (1.f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    const float mh = mm / (1.f - powf(b1, (float)step));
    const float vh = vv / (1.f - powf(b2, (float)step));
    params[p] -= lr * mh / (sqrtf(vh) + eps);
}

// ---------------------------------------------------------------------------
// Davidson use.  second_order_kernel turns U = H t1 into the second-order
// term u = -(D - theta)^-1 (H t1 - D t1) (denominators clipped like the plain
// correction); mlp_correct_kernel computes the features of every (row,
// selected pair), runs the MLP and leaves t1 + clamp(o) u in T.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double clipped_gap(double d, double theta, double clip)
{
    double den = d - theta;
    if (fabs(den) < clip) den = den < 0.0 ? -clip : clip;
    return den;
}

__global__ void second_order_kernel(const double *__restrict__ T, const double *__restrict__ d,
                                    const double *__restrict__ theta, const int *__restrict__ sel,
                                    int nsel, int n, double clip, double *__restrict__ U)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)n * nsel) return;
    const int i = (int)(idx % (size_t)n);
    const int c = (int)(idx / (size_t)n);
    const double den = clipped_gap(d[i], theta[sel[c]], clip);
    U[idx] = -(U[idx] - d[i] * T[idx]) / den;
}

__global__ void __launch_bounds__(256)
mlp_correct_kernel(const float *__restrict__ params, const double *__restrict__ U,
                   const double *__restrict__ X, const double *__restrict__ d,
                   const double *__restrict__ theta, const int *__restrict__ sel, int nsel,
                   int n, double clip, double hnorm, const double *__restrict__ sigma,
                   const double *__restrict__ tnorm, const double *__restrict__ rnorm,
                   double *__restrict__ T)
{
    __shared__ __align__(16) float P[kParams + 3];
    load_params(params, P);
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)n * nsel) return;
    const int i = (int)(idx % (size_t)n);
    const int c = (int)(idx / (size_t)n);
    const int j = sel[c];
    float f[kIn];
    const double u = U[idx];
    row_features(T[idx], tnorm[c], u, rnorm[j], X[(size_t)i + (size_t)j * n], d[i] - theta[j],
                 sigma[i], clip, hnorm, n, f);
    const float o = forward_row(P, f);
    T[idx] = fma((double)o, u, T[idx]);
}

__global__ void add_kernel(double *__restrict__ A, const double *__restrict__ B, size_t count)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count) A[e] += B[e];
}

// Collector: E[:, c] = s_c Xstar[:, l_c] - X[:, sel_c] (n x nsel).
__global__ void collect_error_kernel(const double *__restrict__ Xstar, const int *__restrict__ lidx,
                                     const double *__restrict__ sgn, const double *__restrict__ X,
                                     const int *__restrict__ sel, int nsel, int n,
                                     double *__restrict__ E)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)n * nsel) return;
    const int i = (int)(idx % (size_t)n);
    const int c = (int)(idx / (size_t)n);
    E[idx] = sgn[c] * Xstar[(size_t)lidx[c] * n + i] - X[(size_t)i + (size_t)sel[c] * n];
}

// Collector pass 1: per selected pair c: dots[3c] = <E_c, T_c>,
// dots[3c+1] = <T_c, T_c>, dots[3c+2] = <E_c, E_c> (T: the projected
// two-term correction).
__global__ void collect_dots_kernel(const double *__restrict__ E, const double *__restrict__ T,
                                    int n, double *__restrict__ dots)
{
    const int c = blockIdx.x;
    const double *ec = E + (size_t)c * n;
    const double *t = T + (size_t)c * n;
    double et = 0.0, tt = 0.0, ee = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double e = ec[i];
        et = fma(e, t[i], et);
        tt = fma(t[i], t[i], tt);
        ee = fma(e, e, ee);
    }
    const double2 a = block_sum2(et, tt);
    const double2 b = block_sum2(ee, 0.0);
    if (threadIdx.x == 0) {
        dots[3 * c] = a.x;
        dots[3 * c + 1] = a.y;
        dots[3 * c + 2] = b.x;
    }
}

// Collector pass 2: rows (f0..f5, target scale, weight) of the valid pairs;
// slot[c] >= 0 is the pair's first row in `out`, alpha[c] the fit of E by T_c.
// Collector pass 2: rows (f0..f5, target weight, row weight) of the valid
// pairs; slot[c] >= 0 is the pair's first row in `out`, alpha[c] the fit of
// E by the projected two-term correction.
__global__ void collect_rows_kernel(const double *__restrict__ E, const double *__restrict__ alpha,
                                    const long long *__restrict__ slot,
                                    const double *__restrict__ U, const double *__restrict__ X,
                                    const double *__restrict__ d, const double *__restrict__ theta,
                                    const int *__restrict__ sel, int nsel, int n, double clip,
                                    double hnorm, const double *__restrict__ sigma,
                                    const double *__restrict__ tnorm,
                                    const double *__restrict__ rnorm, const double *__restrict__ T,
                                    const double *__restrict__ Tp, const double *__restrict__ Up,
                                    float *__restrict__ out)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)n * nsel) return;
    const int i = (int)(idx % (size_t)n);
    const int c = (int)(idx / (size_t)n);
    if (slot[c] < 0) return;
    const int j = sel[c];
    const double tn = tnorm[c];
    float f[kIn];
    const double x = X[(size_t)i + (size_t)j * n];
    const double u = U[idx];
    row_features(T[idx], tn, u, rnorm[j], x, d[i] - theta[j], sigma[i], clip, hnorm, n, f);
    // the per-row weight of the projected u that reproduces the scaled exact
    // error with the projected t1; rows where it vanishes carry (almost) no
    // weight
    const double up = Up[idx];
    const double y = fabs(up) > 0.0 ? (E[idx] / alpha[c] - Tp[idx]) / up : 1.0;
    const float g = tn > 0.0 ? (float)(up * sqrt((double)n) / tn) : 0.f;
    float *o = out + (size_t)(slot[c] + i) * kRow;
#pragma unroll
    for (int q = 0; q < kIn; ++q) o[q] = f[q];
    o[kIn] = clampf((float)y, 5.f);
    o[kIn + 1] = g * g;
}

// Row coupling s_i = ||H[i, j != i]||_2 of a CSR matrix (one warp per row).
__global__ void csr_offdiag_norm_kernel(const int *__restrict__ row_ptr,
                                        const int *__restrict__ col_ind,
                                        const double *__restrict__ vals, int n,
                                        double *__restrict__ sigma)
{
    const int row = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    double s = 0.0;
    for (int p = row_ptr[row] + lane; p < row_ptr[row + 1]; p += 32) {
        const double v = col_ind[p] == row ? 0.0 : vals[p];
        s = fma(v, v, s);
    }
    s = warp_sum(s);
    if (lane == 0) sigma[row] = sqrt(s);
}

// Same for a dense symmetric column-major H (column i = row i; one CTA per row).
__global__ void dense_offdiag_norm_kernel(const double *__restrict__ H, int n,
                                          double *__restrict__ sigma)
{
    const int row = blockIdx.x;
    const double *col = H + (size_t)row * n;
    double s = 0.0;
    for (int l = threadIdx.x; l < n; l += blockDim.x) {
        const double v = l == row ? 0.0 : col[l];
        s = fma(v, v, s);
    }
    const double2 t = block_sum2(s, 0.0);
    if (threadIdx.x == 0) sigma[row] = sqrt(t.x);
}

}  // namespace mlp

int launch_csr_row_coupling(const int *row_ptr, const int *col_ind, const double *vals, int n,
                            double *sigma, cudaStream_t s)
{
    mlp::csr_offdiag_norm_kernel<<<blocks_for((size_t)n * 32), kThreads, 0, s>>>(row_ptr, col_ind,
                                                                                 vals, n, sigma);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

int launch_dense_row_coupling(const double *H, int n, double *sigma, cudaStream_t s)
{
    mlp::dense_offdiag_norm_kernel<<<n, 256, 0, s>>>(H, n, sigma);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

// T <- (I - V V^T) T for the n x nsel correction block (one pass; the solver
// re-orthogonalises every correction against V afterwards anyway).
static int project_out(BlockOps &ops, const CorrectionArgs &a, double *T, DeviceBuffer<double> &G)
{
    if (a.V == nullptr || a.m <= 0) return IPT_CUDA_SUCCESS;
    if (G.count < (size_t)a.m * a.nsel) IPTGB_CHECK(G.alloc((size_t)a.m * a.nsel, ops.stream));
    IPTGB_CHECK(ops.gram(a.V, a.n, a.m, T, a.n, a.nsel, a.n, G.ptr, a.m));
    return ops.tall_gemm(a.V, a.n, G.ptr, a.m, T, a.n, a.n, a.m, a.nsel, -1.0, 1.0);
}

// t1 (plain correction, in T) and the second-order term u (in U) of the
// selected pairs; tn = ||t1|| per pair.
static int plain_and_second_order(BlockOps &ops, const CorrectionArgs &a, double *T,
                                  DeviceBuffer<double> &U, double *tn)
{
    cudaStream_t s = ops.stream;
    const size_t nc = (size_t)a.n * a.nsel;
    IPTGB_CHECK(ops.diag_correction(a.R, a.d, a.theta, a.sel, a.nsel, a.n, a.clip, T));
    if (U.count < nc) IPTGB_CHECK(U.alloc(nc, s));
    if (a.apply == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    IPTGB_CHECK(a.apply->apply(T, a.nsel, U.ptr));
    mlp::second_order_kernel<<<blocks_for(nc), kThreads, 0, s>>>(T, a.d, a.theta, a.sel, a.nsel,
                                                                 a.n, a.clip, U.ptr);
    IPTGB_LAUNCH();
    return ops.column_norms(T, a.n, a.n, a.nsel, tn);
}

namespace {

// The learned correction used by the Davidson driver.
struct MlpCorrection final : LearnedCorrection {
    const float *params = nullptr;
    const double *sigma = nullptr;
    double hnorm = 1.0;
    BlockOps ops;
    DeviceBuffer<double> tn, U;
    void bind(const double *row_coupling, double h) override
    {
        sigma = row_coupling;
        hnorm = h;
    }
    bool learned() const override { return true; }
    int correct(const CorrectionArgs &a, double *T) override
    {
        KernelTimerScope timer(kProfMlp, ops.stream);
        if (tn.count < (size_t)a.nsel) IPTGB_CHECK(tn.alloc((size_t)a.nsel, ops.stream));
        IPTGB_CHECK(plain_and_second_order(ops, a, T, U, tn.ptr));
        mlp::mlp_correct_kernel<<<blocks_for((size_t)a.n * a.nsel), 256, 0, ops.stream>>>(
            params, U.ptr, a.X, a.d, a.theta, a.sel, a.nsel, a.n, a.clip, hnorm, sigma, tn.ptr,
            a.rnorm, T);
        IPTGB_LAUNCH();
        return IPT_CUDA_SUCCESS;
    }
    ~MlpCorrection() override { ops.release(); }
};

}  // namespace

// Records (features, target, weight) rows while returning the plain
// diagonal correction, so the solver follows the plain trajectory; with
// `params` set it returns the learned correction instead, so that rows are
// recorded along the learned trajectory (for a further round of training).
struct MlpCollector final : LearnedCorrection {
    const float *params = nullptr;
    const double *Xstar = nullptr;
    int kstar = 0;
    const double *sigma = nullptr;
    double hnorm = 1.0;
    float *out = nullptr;
    long long capacity = 0;
    long long count = 0;
    BlockOps ops;
    DeviceBuffer<double> tn, Xs, O, dots, sgn_d, alpha_d, E, G, U, B, Tp, Up;
    DeviceBuffer<int> lidx_d;
    DeviceBuffer<long long> slot_d;
    void bind(const double *row_coupling, double h) override
    {
        sigma = row_coupling;
        hnorm = h;
    }
    bool learned() const override { return false; }
    int correct(const CorrectionArgs &a, double *T) override
    {
        cudaStream_t s = ops.stream;
        const int c = a.nsel;
        const int n = a.n;
        if (count + (long long)a.nsel * a.n > capacity || sigma == nullptr) {
            return ops.diag_correction(a.R, a.d, a.theta, a.sel, a.nsel, a.n, a.clip, T);
        }
        if (tn.count < (size_t)c) {
            IPTGB_CHECK(tn.alloc((size_t)c, s));
            IPTGB_CHECK(dots.alloc(3 * (size_t)c, s));
            IPTGB_CHECK(sgn_d.alloc((size_t)c, s));
            IPTGB_CHECK(alpha_d.alloc((size_t)c, s));
            IPTGB_CHECK(lidx_d.alloc((size_t)c, s));
            IPTGB_CHECK(slot_d.alloc((size_t)c, s));
            IPTGB_CHECK(O.alloc((size_t)kstar * c, s));
        }
        if (Xs.count < (size_t)n * c) {
            IPTGB_CHECK(Xs.alloc((size_t)n * c, s));
            IPTGB_CHECK(E.alloc((size_t)n * c, s));
            IPTGB_CHECK(B.alloc((size_t)n * c, s));
            IPTGB_CHECK(Tp.alloc((size_t)n * c, s));
            IPTGB_CHECK(Up.alloc((size_t)n * c, s));
        }
        IPTGB_CHECK(plain_and_second_order(ops, a, T, U, tn.ptr));
        // overlaps of the current Ritz vectors with the converged ones
        IPTGB_CHECK(ops.gather_columns(a.X, n, a.sel, nullptr, n, c, Xs.ptr, n));
        IPTGB_CHECK(ops.gram(Xstar, n, kstar, Xs.ptr, n, c, n, O.ptr, kstar));
        std::vector<double> hO((size_t)kstar * c);
        IPTGB_CUDA(cudaMemcpyAsync(hO.data(), O.ptr, hO.size() * sizeof(double),
                                   cudaMemcpyDeviceToHost, s));
        IPTGB_CUDA(cudaStreamSynchronize(s));
        std::vector<int> li((size_t)c);
        std::vector<double> sg((size_t)c);
        for (int q = 0; q < c; ++q) {
            int best = 0;
            for (int l = 1; l < kstar; ++l) {
                if (fabs(hO[(size_t)q * kstar + l]) > fabs(hO[(size_t)q * kstar + best])) best = l;
            }
            li[(size_t)q] = best;
            sg[(size_t)q] = hO[(size_t)q * kstar + best] < 0.0 ? -1.0 : 1.0;
        }
        IPTGB_CUDA(cudaMemcpyAsync(lidx_d.ptr, li.data(), (size_t)c * sizeof(int),
                                   cudaMemcpyHostToDevice, s));
        IPTGB_CUDA(cudaMemcpyAsync(sgn_d.ptr, sg.data(), (size_t)c * sizeof(double),
                                   cudaMemcpyHostToDevice, s));
        mlp::collect_error_kernel<<<blocks_for((size_t)n * c), kThreads, 0, s>>>(
            Xstar, lidx_d.ptr, sgn_d.ptr, a.X, a.sel, c, n, E.ptr);
        IPTGB_LAUNCH();
        // keep only the part of the error outside the search space (two
        // passes), and fit it by the projected two-term correction t1 + u
        for (int pass = 0; pass < 2; ++pass) IPTGB_CHECK(project_out(ops, a, E.ptr, G));
        IPTGB_CUDA(cudaMemcpyAsync(B.ptr, T, (size_t)n * c * sizeof(double),
                                   cudaMemcpyDeviceToDevice, s));
        mlp::add_kernel<<<blocks_for((size_t)n * c), kThreads, 0, s>>>(B.ptr, U.ptr,
                                                                      (size_t)n * c);
        IPTGB_LAUNCH();
        IPTGB_CHECK(project_out(ops, a, B.ptr, G));
        // the projected t1 and u of the per-row targets
        IPTGB_CUDA(cudaMemcpyAsync(Tp.ptr, T, (size_t)n * c * sizeof(double),
                                   cudaMemcpyDeviceToDevice, s));
        IPTGB_CUDA(cudaMemcpyAsync(Up.ptr, U.ptr, (size_t)n * c * sizeof(double),
                                   cudaMemcpyDeviceToDevice, s));
        for (int pass = 0; pass < 2; ++pass) {
            IPTGB_CHECK(project_out(ops, a, Tp.ptr, G));
            IPTGB_CHECK(project_out(ops, a, Up.ptr, G));
        }
        mlp::collect_dots_kernel<<<c, 256, 0, s>>>(E.ptr, B.ptr, n, dots.ptr);
        IPTGB_LAUNCH();
        std::vector<double> hd(3 * (size_t)c);
        IPTGB_CUDA(cudaMemcpyAsync(hd.data(), dots.ptr, hd.size() * sizeof(double),
                                   cudaMemcpyDeviceToHost, s));
        IPTGB_CUDA(cudaStreamSynchronize(s));
        std::vector<double> al((size_t)c, 1.0);
        std::vector<long long> slot((size_t)c, -1);
        for (int q = 0; q < c; ++q) {
            const double et = hd[3 * (size_t)q], tt = hd[3 * (size_t)q + 1],
                         ee = hd[3 * (size_t)q + 2];
            // skip pairs whose exact correction is (numerically) orthogonal to
            // the two-term one, or already converged
            if (!(tt > 0.0) || !(ee > 1e-28) || fabs(et) < 0.05 * sqrt(tt * ee)) continue;
            al[(size_t)q] = et / tt;
            slot[(size_t)q] = count;
            count += n;
        }
        IPTGB_CUDA(cudaMemcpyAsync(alpha_d.ptr, al.data(), (size_t)c * sizeof(double),
                                   cudaMemcpyHostToDevice, s));
        IPTGB_CUDA(cudaMemcpyAsync(slot_d.ptr, slot.data(), (size_t)c * sizeof(long long),
                                   cudaMemcpyHostToDevice, s));
        mlp::collect_rows_kernel<<<blocks_for((size_t)n * c), kThreads, 0, s>>>(
            E.ptr, alpha_d.ptr, slot_d.ptr, U.ptr, a.X, a.d, a.theta, a.sel, c, n, a.clip, hnorm,
            sigma, tn.ptr, a.rnorm, T, Tp.ptr, Up.ptr, out);
        IPTGB_LAUNCH();
        if (params != nullptr) {
            mlp::mlp_correct_kernel<<<blocks_for((size_t)n * c), 256, 0, s>>>(
                params, U.ptr, a.X, a.d, a.theta, a.sel, c, n, a.clip, hnorm, sigma, tn.ptr,
                a.rnorm, T);
            IPTGB_LAUNCH();
        }
        IPTGB_CUDA(cudaStreamSynchronize(s));
        return IPT_CUDA_SUCCESS;
    }
    ~MlpCollector() override { ops.release(); }
};

LearnedCorrection *make_learned_correction(const float *params, cudaStream_t stream)
{
    if (params == nullptr) return nullptr;
    auto *m = new MlpCorrection();
    m->params = params;
    m->ops.stream = stream;
    m->ops.sms = device_sm_count();
    return m;
}

LearnedCorrection *make_mlp_collector(const double *Xstar, int kstar, float *out,
                                      long long capacity, const float *params, cudaStream_t stream)
{
    auto *m = new MlpCollector();
    m->params = params;
    m->Xstar = Xstar;
    m->kstar = kstar;
    m->out = out;
    m->capacity = capacity;
    m->ops.stream = stream;
    m->ops.sms = device_sm_count();
    return m;
}

long long mlp_collector_count(const LearnedCorrection *c)
{
    const auto *m = dynamic_cast<const MlpCollector *>(c);
    return m != nullptr ? m->count : 0;
}

}  // namespace iptgb

// ---------------------------------------------------------------------------
// C ABI of the learned preconditioner (include/ipt_block.h)
// ---------------------------------------------------------------------------
using namespace iptgb;

#define IPT_API extern "C" __attribute__((visibility("default")))

IPT_API int ipt_block_mlp_param_count(void) { return mlp::kParams; }

IPT_API int ipt_block_mlp_init(float *d_params, unsigned long long seed, void *stream)
{
    if (d_params == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    mlp::mlp_init_kernel<<<blocks_for(mlp::kParams), kThreads, 0, s>>>(d_params, seed);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_block_mlp_forward(const float *d_params, const float *d_rows, long long rows,
                                  int row_stride, float *d_out, void *stream)
{
    if (d_params == nullptr || d_rows == nullptr || d_out == nullptr || rows < 0 ||
        row_stride < mlp::kIn) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    if (rows == 0) return IPT_CUDA_SUCCESS;
    cudaStream_t s = (cudaStream_t)stream;
    mlp::mlp_forward_rows_kernel<<<(unsigned)((rows + 255) / 256), 256, 0, s>>>(
        d_params, d_rows, rows, row_stride, d_out);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_block_mlp_loss_grad(const float *d_params, const float *d_rows, long long rows,
                                    float *d_grad, void *stream)
{
    if (d_params == nullptr || d_rows == nullptr || d_grad == nullptr || rows <= 0 ||
        rows > (1LL << 30)) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int batch = (int)rows;
    const int tiles = (batch + mlp::kTile - 1) / mlp::kTile;
    DeviceBuffer<float> part;
    IPTGB_CHECK(part.alloc((size_t)tiles * (mlp::kParams + 1), s));
    const size_t smem = mlp::fwd_bwd_smem_bytes();
    IPTGB_CUDA(cudaFuncSetAttribute(mlp::mlp_fwd_bwd_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mlp::mlp_fwd_bwd_kernel<<<tiles, mlp::kTile, smem, s>>>(d_params, d_rows, rows, batch, 0, 0,
                                                            0, part.ptr);
    IPTGB_LAUNCH();
    mlp::mlp_grad_finish_kernel<<<blocks_for(mlp::kParams + 1), kThreads, 0, s>>>(part.ptr, tiles,
                                                                                  batch, d_grad);
    IPTGB_LAUNCH();
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_block_mlp_train(float *d_params, const float *d_rows, long long rows, int steps,
                                int batch, float lr, unsigned long long seed,
                                float *d_loss_history, void *stream)
{
    if (d_params == nullptr || d_rows == nullptr || rows <= 0 || steps < 0 || batch <= 0 ||
        batch > (1 << 20) || !(lr > 0.f)) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int tiles = (batch + mlp::kTile - 1) / mlp::kTile;
    DeviceBuffer<float> part, mv;
    IPTGB_CHECK(part.alloc((size_t)tiles * (mlp::kParams + 1), s));
    IPTGB_CHECK(mv.alloc(2 * (size_t)mlp::kParams, s));
    IPTGB_CUDA(cudaMemsetAsync(mv.ptr, 0, 2 * (size_t)mlp::kParams * sizeof(float), s));
    const size_t smem = mlp::fwd_bwd_smem_bytes();
    IPTGB_CUDA(cudaFuncSetAttribute(mlp::mlp_fwd_bwd_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    KernelTimerScope timer(kProfMlp, s);
    for (int it = 1; it <= steps; ++it) {
        mlp::mlp_fwd_bwd_kernel<<<tiles, mlp::kTile, smem, s>>>(d_params, d_rows, rows, batch, 1,
                                                                seed, it, part.ptr);
        IPTGB_LAUNCH();
        mlp::mlp_adam_kernel<<<blocks_for(mlp::kParams + 1), kThreads, 0, s>>>(
            d_params, mv.ptr, mv.ptr + mlp::kParams, part.ptr, tiles, batch, it, lr,
            d_loss_history);
        IPTGB_LAUNCH();
    }
    return IPT_CUDA_SUCCESS;
}
