// k_fci.cu - matrix-free sigma build Y = H X for FCI-like Hamiltonians over
// all (alpha, beta) occupation-string pairs, and the Davidson solve on top of
// it.  H is never stored: every matrix element is regenerated from integer
// hashes of the determinant pair when it is needed.
//
// The reference has no matrix-free path; its FCI structure (strings, single
// and double excitation links, alpha-beta products) is in
// IPT_C_GPU/test/sparse/H2O/benchmark_h2o_631g_cas10e10o_primme_vs_ipt.cu:
// 390-766, where the Hamiltonian is assembled into CSC from PySCF integrals.
// Here the integrals are replaced by a seeded synthetic rule (the same rule
// as the FCI-like CSR workload), evaluated in FP32 by deterministic code of
// this file, so that a CPU restatement reproduces every element bit for bit:
//
//   strings   all nel-subsets of norb orbitals, lexicographic; determinant
//             I = ia * n_beta_strings + ib
//   eps_p     0.5 p + 0.05 g(seed, 31, p, 0)
//   E(I)      sum of eps over the occupied orbitals of both strings
//   H_II      E(I) + 0.01 g(seed, 32, I, 0)
//   H_IJ      0.05 g(seed, 33, min(I,J), max(I,J)) exp(-|E(J) - E(I)|) for J
//             a single or double excitation of I (alpha, beta, alpha-alpha,
//             beta-beta, alpha-beta), 0 otherwise
//
// g is a standard normal deviate by the Box-Muller transform of two uniforms
// u1 = U(seed, s), u2 = U(seed, s + 7919) built from a splitmix64 hash of
// the canonical index pair (u = float((h >> 11) | 1) 2^-53, correctly
// rounded); log, cos and exp are evaluated by the range reductions and
// polynomials below (atanh series for log, Taylor series for cos on
// [0, pi/2] and for exp after Cody-Waite reduction), every FP32 operation
// rounded to nearest with no contraction.  The off-diagonal energy gap is
// formed in FP32 from FP32 string energies, |(eA(ja) - eA(ia)) + (eB(jb) -
// eB(ib))|, so that no element needs the (slow) FP64 pipe.
//
// Sigma kernel: one warp per determinant row; the lanes stride over the
// row's couplings (alpha singles, beta singles, alpha-alpha and beta-beta
// doubles, then the alpha-single x beta-single products), generate H_IJ and
// accumulate H_IJ X[J, :] for a block of KC columns.  X is a row-major copy
// (KC values per determinant, so one gather per coupling).  Low precision:
// X in BF16 or FP32, FP32 accumulation.  FP64-accurate: X as an unevaluated
// sum of two floats (hi + lo), products split exactly with an FMA
// (Dekker/Knuth two-product) and summed in double-float arithmetic
// (two-sum), the lane partials reduced in FP64 - FP32 pipe throughput with
// ~48-bit accuracy (the elements themselves are exact FP32 numbers).
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <numeric>
#include <vector>

#include "block_ops.h"
#include "block_solver.h"
#include "common.cuh"
#include "ipt_plain.h"

#define IPT_API extern "C" __attribute__((visibility("default")))

namespace iptgb {
namespace fci {

// ---------------------------------------------------------------------------
// Hashes (bit-identical to block_ipt_gb300/workloads.py)
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t splitmix(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ULL;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__host__ __device__ __forceinline__ uint64_t stream_key(uint64_t seed, uint64_t stream)
{
    return splitmix(seed * 0x10001ULL + stream);
}

__host__ __device__ __forceinline__ float bits_to_float(uint32_t b)
{
    float f;
    memcpy(&f, &b, 4);
    return f;
}

__host__ __device__ __forceinline__ uint32_t float_to_bits(float f)
{
    uint32_t b;
    memcpy(&b, &f, 4);
    return b;
}

// Round-to-nearest-even conversion of 1 <= v < 2^53 to float with integer
// operations only (GB300 runs 64-bit integer to float conversions on its
// FP64 unit); equal to the correctly rounded (float)v.
__host__ __device__ __forceinline__ float u53_to_float(uint64_t v)
{
#ifdef __CUDA_ARCH__
    const int msb = 63 - __clzll((long long)v);
#else
    const int msb = 63 - __builtin_clzll(v);
#endif
    uint32_t m;
    int e = msb;
    if (msb <= 23) {
        m = (uint32_t)(v << (23 - msb));
    } else {
        const int sh = msb - 23;
        uint64_t q = v >> sh;
        const uint64_t rem = v & ((1ULL << sh) - 1);
        const uint64_t half = 1ULL << (sh - 1);
        if (rem > half || (rem == half && (q & 1))) ++q;
        if (q == (1ULL << 24)) {
            q >>= 1;
            ++e;
        }
        m = (uint32_t)q;
    }
    return bits_to_float(((uint32_t)(e + 127) << 23) | (m & 0x7fffffu));
}

// second stage of the pair hash: h1 = splitmix(key ^ lo), hm = hi * M;
// u = float((h >> 11) | 1) 2^-53
__host__ __device__ __forceinline__ float pair_uniform(uint64_t h1, uint64_t hm)
{
    const uint64_t h = splitmix(h1 ^ hm);
    return u53_to_float((h >> 11) | 1ULL) * 0x1p-53f;
}

__host__ __device__ __forceinline__ uint64_t pair_mult(uint64_t hi)
{
    return hi * 0xD1B54A32D192ED03ULL;
}

// ---------------------------------------------------------------------------
// FP32 elementary functions, every operation rounded to nearest explicitly
// ---------------------------------------------------------------------------
#ifdef __CUDA_ARCH__
#define F_ADD(a, b) __fadd_rn((a), (b))
#define F_SUB(a, b) __fsub_rn((a), (b))
#define F_MUL(a, b) __fmul_rn((a), (b))
#define F_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define F_DIV(a, b) __fdiv_rn((a), (b))
#define F_SQRT(a) __fsqrt_rn(a)
#else
#define F_ADD(a, b) ((float)((a) + (b)))
#define F_SUB(a, b) ((float)((a) - (b)))
#define F_MUL(a, b) ((float)((a) * (b)))
#define F_FMA(a, b, c) fmaf((a), (b), (c))
#define F_DIV(a, b) ((float)((a) / (b)))
#define F_SQRT(a) sqrtf(a)
#endif

// natural log of a positive normal float: x = m 2^e, m in [sqrt(2)/2, sqrt(2)),
// log(m) = 2 atanh(s), s = (m - 1) / (m + 1), series to s^9
__host__ __device__ __forceinline__ float log32(float x)
{
    const uint32_t b = float_to_bits(x);
    int e = (int)((b >> 23) & 0xffu) - 127;
    float m = bits_to_float((b & 0x7fffffu) | 0x3f800000u);
    if (m > 1.41421356f) {
        m = F_MUL(m, 0.5f);
        e += 1;
    }
    const float f = F_SUB(m, 1.0f);
    const float s = F_DIV(f, F_ADD(2.0f, f));
    const float s2 = F_MUL(s, s);
    float p = F_FMA(s2, 0.222222222f, 0.285714286f);
    p = F_FMA(s2, p, 0.4f);
    p = F_FMA(s2, p, 0.666666667f);
    p = F_FMA(s2, p, 2.0f);
    return F_FMA((float)e, 0.693147181f, F_MUL(s, p));
}

// cos(2 pi u) for u in (0, 1): reflect to an angle in [0, pi/2], Taylor to x^12
__host__ __device__ __forceinline__ float cos2pi32(float u)
{
    float a = fabsf(F_SUB(u, 0.5f));  // cos(2 pi u) = -cos(2 pi a)
    float sign = -1.0f;
    if (a > 0.25f) {
        a = F_SUB(0.5f, a);
        sign = 1.0f;
    }
    const float x = F_MUL(a, 6.28318531f);
    const float x2 = F_MUL(x, x);
    float c = F_FMA(x2, 2.08767570e-9f, -2.75573192e-7f);
    c = F_FMA(x2, c, 2.48015873e-5f);
    c = F_FMA(x2, c, -1.38888889e-3f);
    c = F_FMA(x2, c, 4.16666667e-2f);
    c = F_FMA(x2, c, -0.5f);
    c = F_FMA(x2, c, 1.0f);
    return F_MUL(sign, c);
}

// exp(y) for y <= 0: y = n ln2 + r (ln2 split in two), Taylor to r^7, 2^n by bits
__host__ __device__ __forceinline__ float exp32(float y)
{
    if (y < -87.0f) return 0.0f;
    const float n = rintf(F_MUL(y, 1.44269504f));
    float r = F_FMA(-n, 0.693145752f, y);
    r = F_FMA(-n, 1.42860677e-6f, r);
    float p = F_FMA(r, 1.98412698e-4f, 1.38888889e-3f);
    p = F_FMA(r, p, 8.33333333e-3f);
    p = F_FMA(r, p, 4.16666667e-2f);
    p = F_FMA(r, p, 0.166666667f);
    p = F_FMA(r, p, 0.5f);
    p = F_FMA(r, p, 1.0f);
    p = F_FMA(r, p, 1.0f);
    const int ni = (int)n;
    if (ni < -126) return 0.0f;
    return F_MUL(p, bits_to_float((uint32_t)(ni + 127) << 23));
}

__host__ __device__ __forceinline__ float normal32(float u1, float u2)
{
    const float r = F_SQRT(F_MUL(-2.0f, log32(u1)));
    return F_MUL(r, cos2pi32(u2));
}

// g(seed, stream, a, b) as a float
__host__ __device__ __forceinline__ float gauss(uint64_t k1, uint64_t k2, uint64_t a, uint64_t b)
{
    const uint64_t bm = pair_mult(b);
    const float u1 = pair_uniform(splitmix(k1 ^ a), bm);
    const float u2 = pair_uniform(splitmix(k2 ^ a), bm);
    return normal32(u1, u2);
}

// H_IJ for a connected pair: gap = FP32 energy difference E(J) - E(I);
// hI1, hI2, hIm: the row's first-stage hashes of I and I * M (used as lo
// when I < J, as hi otherwise)
__host__ __device__ __forceinline__ float offdiag(uint64_t k1, uint64_t k2, uint64_t I, uint64_t J,
                                                  uint64_t hI1, uint64_t hI2, uint64_t hIm,
                                                  float gap, float sigma)
{
    uint64_t h1, h2, hm;
    if (I < J) {
        h1 = hI1;
        h2 = hI2;
        hm = pair_mult(J);
    } else {
        h1 = splitmix(k1 ^ J);
        h2 = splitmix(k2 ^ J);
        hm = hIm;
    }
    const float z = normal32(pair_uniform(h1, hm), pair_uniform(h2, hm));
    return F_MUL(F_MUL(sigma, z), exp32(-fabsf(gap)));
}

// ---------------------------------------------------------------------------
// Tables (host-built, device-resident)
// ---------------------------------------------------------------------------
struct Tables {
    int norb = 0, na = 0, nb = 0;
    uint64_t seed = 0;
    float sigma = 0.05f;
    int nsa = 0, nsb = 0;          // number of alpha / beta strings
    int sA = 0, sB = 0, dA = 0, dB = 0;  // links per string
    long long n = 0;
    std::vector<double> eps, occA, occB;
    std::vector<float> occAf, occBf;
    std::vector<int> singA, singB, doubA, doubB;  // [string][link] -> target string
};

static std::vector<int> make_strings(int norb, int nel, std::vector<int> &index)
{
    std::vector<int> out;
    index.assign((size_t)1 << norb, -1);
    std::vector<int> c(nel);
    for (int i = 0; i < nel; ++i) c[i] = i;
    while (true) {
        int bits = 0;
        for (int i = 0; i < nel; ++i) bits |= 1 << c[i];
        index[bits] = (int)out.size();
        out.push_back(bits);
        int i = nel - 1;
        while (i >= 0 && c[i] == norb - nel + i) --i;
        if (i < 0) break;
        ++c[i];
        for (int j = i + 1; j < nel; ++j) c[j] = c[j - 1] + 1;
    }
    return out;
}

static void make_links(int norb, const std::vector<int> &strs, const std::vector<int> &index,
                       std::vector<int> &sing, std::vector<int> &doub, int &ns, int &nd)
{
    sing.clear();
    doub.clear();
    for (int s : strs) {
        std::vector<int> occ, vir;
        for (int o = 0; o < norb; ++o) (s >> o & 1 ? occ : vir).push_back(o);
        for (int h : occ)
            for (int p : vir) sing.push_back(index[s ^ (1 << h) ^ (1 << p)]);
        for (size_t a = 0; a < occ.size(); ++a)
            for (size_t b = a + 1; b < occ.size(); ++b)
                for (size_t c = 0; c < vir.size(); ++c)
                    for (size_t d = c + 1; d < vir.size(); ++d)
                        doub.push_back(index[s ^ (1 << occ[a]) ^ (1 << occ[b]) ^ (1 << vir[c]) ^
                                             (1 << vir[d])]);
    }
    const int nel = __builtin_popcount((unsigned)strs[0]);
    ns = nel * (norb - nel);
    nd = nel * (nel - 1) / 2 * ((norb - nel) * (norb - nel - 1) / 2);
}

int build_tables(int norb, int na, int nb, unsigned long long seed, double sigma, Tables *t)
{
    if (norb < 2 || norb > 16 || na < 1 || nb < 1 || na >= norb || nb >= norb) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    t->norb = norb;
    t->na = na;
    t->nb = nb;
    t->seed = seed;
    t->sigma = (float)sigma;
    const uint64_t k31a = stream_key(seed, 31), k31b = stream_key(seed, 31 + 7919);
    t->eps.resize(norb);
    for (int p = 0; p < norb; ++p) {
        t->eps[p] = 0.5 * p + 0.05 * (double)gauss(k31a, k31b, (uint64_t)p, 0);
    }
    std::vector<int> ia_index, ib_index;
    const std::vector<int> sa = make_strings(norb, na, ia_index);
    const std::vector<int> sb = make_strings(norb, nb, ib_index);
    t->nsa = (int)sa.size();
    t->nsb = (int)sb.size();
    t->n = (long long)t->nsa * t->nsb;
    auto occ_energy = [&](int s) {
        double e = 0.0;
        for (int o = 0; o < norb; ++o)
            if (s >> o & 1) e += t->eps[o];
        return e;
    };
    t->occA.resize(sa.size());
    t->occB.resize(sb.size());
    for (size_t i = 0; i < sa.size(); ++i) t->occA[i] = occ_energy(sa[i]);
    for (size_t i = 0; i < sb.size(); ++i) t->occB[i] = occ_energy(sb[i]);
    t->occAf.assign(t->occA.begin(), t->occA.end());
    t->occBf.assign(t->occB.begin(), t->occB.end());
    make_links(norb, sa, ia_index, t->singA, t->doubA, t->sA, t->dA);
    make_links(norb, sb, ib_index, t->singB, t->doubB, t->sB, t->dB);
    return IPT_CUDA_SUCCESS;
}

struct DevTables {
    const double *occA, *occB;
    const float *occAf, *occBf;
    const int *singA, *singB, *doubA, *doubB;
    long long n;
    int nsb, sA, sB, dA, dB;
    uint64_t k33a, k33b;
    float sigma;
    const double *diag;
};

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
__global__ void fci_diag_kernel(DevTables t, uint64_t k32a, uint64_t k32b, double *__restrict__ diag)
{
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= t.n) return;
    const int ia = (int)(I / t.nsb);
    const int ib = (int)(I - (long long)ia * t.nsb);
    diag[I] = (t.occA[ia] + t.occB[ib]) + 0.01 * (double)gauss(k32a, k32b, (uint64_t)I, 0);
}

// X operand types of the sigma kernel and how a term is accumulated
struct XDF {      // FP64-accurate: x = hi + lo (floats), double-float sums
    float hi, lo;
};

__device__ __forceinline__ float load_x(__nv_bfloat16 x) { return __bfloat162float(x); }
__device__ __forceinline__ float load_x(float x) { return x; }

// s = sh + sl (double-float) += v * (xh + xl): exact two-product of v * xh,
// two-sum into sh, the rounding errors and v * xl into sl
__device__ __forceinline__ void df_accumulate(float &sh, float &sl, float v, const XDF &x)
{
    const float p = __fmul_rn(v, x.hi);
    const float pe = __fmaf_rn(v, x.hi, -p);
    const float t = __fadd_rn(sh, p);
    const float bp = __fsub_rn(t, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    sh = t;
    sl = __fadd_rn(sl, __fadd_rn(err, __fmaf_rn(v, x.lo, pe)));
}

template <typename XT>
struct SigmaAcc {  // FP32 accumulation of a low-precision X
    float s = 0.f;
    __device__ __forceinline__ void add(float v, const XT &x) { s = fmaf(v, load_x(x), s); }
    __device__ __forceinline__ double value() const { return (double)s; }
};

template <>
struct SigmaAcc<XDF> {
    float sh = 0.f, sl = 0.f;
    __device__ __forceinline__ void add(float v, const XDF &x) { df_accumulate(sh, sl, v, x); }
    __device__ __forceinline__ double value() const { return (double)sh + (double)sl; }
};

// Y[:, c0:c0+KC] (column-major, ld n) = H X for the KC-column block of the
// row-major Xr (row J holds X[J, c0:c0+KC]); one warp per row.  The lane
// partials are summed in FP64.
template <typename XT, int KC>
__global__ void __launch_bounds__(256)
fci_sigma_kernel(DevTables t, const XT *__restrict__ Xr, int c0, int k, double *__restrict__ Y)
{
    const long long I = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (I >= t.n) return;
    const int ia = (int)(I / t.nsb);
    const int ib = (int)(I - (long long)ia * t.nsb);
    const float eIa = t.occAf[ia], eIb = t.occBf[ib];
    const uint64_t hI1 = splitmix(t.k33a ^ (uint64_t)I);
    const uint64_t hI2 = splitmix(t.k33b ^ (uint64_t)I);
    const uint64_t hIm = pair_mult((uint64_t)I);
    SigmaAcc<XT> acc[KC];
    const int *sa = t.singA + (size_t)ia * t.sA;
    const int *sb = t.singB + (size_t)ib * t.sB;
    const int *da = t.doubA + (size_t)ia * t.dA;
    const int *db = t.doubB + (size_t)ib * t.dB;
    const int b1 = t.sA, b2 = b1 + t.sB, b3 = b2 + t.dA, b4 = b3 + t.dB;
    const int total = b4 + t.sA * t.sB;
    for (int q = lane; q < total; q += 32) {
        int ja, jb;
        if (q < b1) {
            ja = sa[q];
            jb = ib;
        } else if (q < b2) {
            ja = ia;
            jb = sb[q - b1];
        } else if (q < b3) {
            ja = da[q - b2];
            jb = ib;
        } else if (q < b4) {
            ja = ia;
            jb = db[q - b3];
        } else {
            const int r = q - b4;
            const int a = r / t.sB;
            ja = sa[a];
            jb = sb[r - a * t.sB];
        }
        const long long J = (long long)ja * t.nsb + jb;
        const float gap = F_ADD(F_SUB(t.occAf[ja], eIa), F_SUB(t.occBf[jb], eIb));
        const float v = offdiag(t.k33a, t.k33b, (uint64_t)I, (uint64_t)J, hI1, hI2, hIm, gap,
                                t.sigma);
        const XT *x = Xr + (size_t)J * KC;
#pragma unroll
        for (int j = 0; j < KC; ++j) acc[j].add(v, x[j]);
    }
    double out = 0.0;
#pragma unroll
    for (int j = 0; j < KC; ++j) {
        double s = acc[j].value();
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        out = lane == j ? s : out;
    }
    if (lane < KC && c0 + lane < k) {
        // the diagonal term in FP64
        const size_t e = (size_t)I * KC + lane;
        double xv;
        if constexpr (sizeof(XT) == sizeof(XDF)) {
            const XDF xd = reinterpret_cast<const XDF *>(Xr)[e];
            xv = (double)xd.hi + (double)xd.lo;
        } else {
            xv = (double)load_x(Xr[e]);
        }
        Y[(size_t)I + (size_t)(c0 + lane) * t.n] = fma(t.diag[I], xv, out);
    }
}

// Per row: absolute row sum of H (for ||H||_inf) and the 2-norm of the
// off-diagonal part (the row coupling of the learned preconditioner); one
// warp per row, the same coupling enumeration as the sigma kernel.
__global__ void __launch_bounds__(256)
fci_rowstats_kernel(DevTables t, double *__restrict__ rowabs, double *__restrict__ coupling)
{
    const long long I = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (I >= t.n) return;
    const int ia = (int)(I / t.nsb);
    const int ib = (int)(I - (long long)ia * t.nsb);
    const float eIa = t.occAf[ia], eIb = t.occBf[ib];
    const uint64_t hI1 = splitmix(t.k33a ^ (uint64_t)I);
    const uint64_t hI2 = splitmix(t.k33b ^ (uint64_t)I);
    const uint64_t hIm = pair_mult((uint64_t)I);
    const int *sa = t.singA + (size_t)ia * t.sA;
    const int *sb = t.singB + (size_t)ib * t.sB;
    const int *da = t.doubA + (size_t)ia * t.dA;
    const int *db = t.doubB + (size_t)ib * t.dB;
    const int b1 = t.sA, b2 = b1 + t.sB, b3 = b2 + t.dA, b4 = b3 + t.dB;
    const int total = b4 + t.sA * t.sB;
    double sabs = 0.0, s2 = 0.0;
    for (int q = lane; q < total; q += 32) {
        int ja, jb;
        if (q < b1) {
            ja = sa[q];
            jb = ib;
        } else if (q < b2) {
            ja = ia;
            jb = sb[q - b1];
        } else if (q < b3) {
            ja = da[q - b2];
            jb = ib;
        } else if (q < b4) {
            ja = ia;
            jb = db[q - b3];
        } else {
            const int r = q - b4;
            const int a = r / t.sB;
            ja = sa[a];
            jb = sb[r - a * t.sB];
        }
        const long long J = (long long)ja * t.nsb + jb;
        const float gap = F_ADD(F_SUB(t.occAf[ja], eIa), F_SUB(t.occBf[jb], eIb));
        const double v = (double)offdiag(t.k33a, t.k33b, (uint64_t)I, (uint64_t)J, hI1, hI2, hIm,
                                         gap, t.sigma);
        sabs += fabs(v);
        s2 += v * v;
    }
    for (int off = 16; off > 0; off >>= 1) {
        sabs += __shfl_xor_sync(0xffffffffu, sabs, off);
        s2 += __shfl_xor_sync(0xffffffffu, s2, off);
    }
    if (lane == 0) {
        rowabs[I] = sabs + fabs(t.diag[I]);
        coupling[I] = sqrt(s2);
    }
}

// Xr[J * KC + j] = X[J + (c0 + j) n] (zero beyond k), converted to XT
__device__ __forceinline__ void store_x(__nv_bfloat16 &o, double v) { o = __double2bfloat16(v); }
__device__ __forceinline__ void store_x(float &o, double v) { o = (float)v; }
__device__ __forceinline__ void store_x(XDF &o, double v)
{
    o.hi = __double2float_rn(v);
    o.lo = __double2float_rn(v - (double)o.hi);
}

template <typename XT, int KC>
__global__ void fci_pack_kernel(const double *__restrict__ X, long long n, int c0, int k,
                                XT *__restrict__ Xr)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * KC) return;
    const long long J = e / KC;
    const int j = (int)(e - J * KC);
    const double v = c0 + j < k ? X[J + (long long)(c0 + j) * n] : 0.0;
    store_x(Xr[e], v);
}

}  // namespace fci

// ---------------------------------------------------------------------------
// Operator: device tables + sigma in a chosen precision
// ---------------------------------------------------------------------------
enum FciPrecision { kFciF64 = 0, kFciF32 = 1, kFciBF16 = 2 };
constexpr int kFciKC = 8;

struct FciOperator final : Fp64Apply {
    fci::Tables host;
    fci::DevTables dev{};
    DeviceBuffer<double> occA, occB, diag;
    DeviceBuffer<float> occAf, occBf;
    DeviceBuffer<int> singA, singB, doubA, doubB;
    DeviceBuffer<unsigned char> xr;
    int precision = kFciF64;
    cudaStream_t s = nullptr;

    int init(int norb, int na, int nb, unsigned long long seed, double sigma, cudaStream_t st)
    {
        s = st;
        IPTGB_CHECK(fci::build_tables(norb, na, nb, seed, sigma, &host));
        auto up_d = [&](DeviceBuffer<double> &b, const std::vector<double> &v) -> int {
            IPTGB_CHECK(b.alloc(v.size(), s));
            IPTGB_CUDA(cudaMemcpyAsync(b.ptr, v.data(), v.size() * sizeof(double),
                                       cudaMemcpyHostToDevice, s));
            return IPT_CUDA_SUCCESS;
        };
        auto up_i = [&](DeviceBuffer<int> &b, const std::vector<int> &v) -> int {
            IPTGB_CHECK(b.alloc(std::max<size_t>(1, v.size()), s));
            if (!v.empty()) {
                IPTGB_CUDA(cudaMemcpyAsync(b.ptr, v.data(), v.size() * sizeof(int),
                                           cudaMemcpyHostToDevice, s));
            }
            return IPT_CUDA_SUCCESS;
        };
        IPTGB_CHECK(up_d(occA, host.occA));
        IPTGB_CHECK(up_d(occB, host.occB));
        IPTGB_CHECK(occAf.alloc(host.occAf.size(), s));
        IPTGB_CHECK(occBf.alloc(host.occBf.size(), s));
        IPTGB_CUDA(cudaMemcpyAsync(occAf.ptr, host.occAf.data(), host.occAf.size() * sizeof(float),
                                   cudaMemcpyHostToDevice, s));
        IPTGB_CUDA(cudaMemcpyAsync(occBf.ptr, host.occBf.data(), host.occBf.size() * sizeof(float),
                                   cudaMemcpyHostToDevice, s));
        IPTGB_CHECK(up_i(singA, host.singA));
        IPTGB_CHECK(up_i(singB, host.singB));
        IPTGB_CHECK(up_i(doubA, host.doubA));
        IPTGB_CHECK(up_i(doubB, host.doubB));
        IPTGB_CHECK(diag.alloc((size_t)host.n, s));
        dev.occA = occA.ptr;
        dev.occB = occB.ptr;
        dev.occAf = occAf.ptr;
        dev.occBf = occBf.ptr;
        dev.singA = singA.ptr;
        dev.singB = singB.ptr;
        dev.doubA = doubA.ptr;
        dev.doubB = doubB.ptr;
        dev.n = host.n;
        dev.nsb = host.nsb;
        dev.sA = host.sA;
        dev.sB = host.sB;
        dev.dA = host.dA;
        dev.dB = host.dB;
        dev.k33a = fci::stream_key(seed, 33);
        dev.k33b = fci::stream_key(seed, 33 + 7919);
        dev.sigma = host.sigma;
        dev.diag = diag.ptr;
        fci::fci_diag_kernel<<<(unsigned)((host.n + 255) / 256), 256, 0, s>>>(
            dev, fci::stream_key(seed, 32), fci::stream_key(seed, 32 + 7919), diag.ptr);
        IPTGB_LAUNCH();
        return IPT_CUDA_SUCCESS;
    }

    template <typename XT>
    int sigma_t(const double *X, int c, double *Y)
    {
        const long long n = host.n;
        const size_t need = (size_t)n * kFciKC * sizeof(XT);
        if (xr.count < need) IPTGB_CHECK(xr.alloc(need, s));
        XT *Xr = reinterpret_cast<XT *>(xr.ptr);
        const unsigned warps_blocks = (unsigned)((n * 32 + 255) / 256);
        for (int c0 = 0; c0 < c; c0 += kFciKC) {
            fci::fci_pack_kernel<XT, kFciKC><<<(unsigned)((n * kFciKC + 255) / 256), 256, 0, s>>>(
                X, n, c0, c, Xr);
            IPTGB_LAUNCH();
            fci::fci_sigma_kernel<XT, kFciKC><<<warps_blocks, 256, 0, s>>>(dev, Xr, c0, c, Y);
            IPTGB_LAUNCH();
        }
        return IPT_CUDA_SUCCESS;
    }

    int sigma(const double *X, int c, double *Y, int prec)
    {
        KernelTimerScope timer(kProfCsrProduct, s);
        if (prec == kFciF64) return sigma_t<fci::XDF>(X, c, Y);
        if (prec == kFciF32) return sigma_t<float>(X, c, Y);
        return sigma_t<__nv_bfloat16>(X, c, Y);
    }

    int apply(const double *V, int c, double *AV) override { return sigma(V, c, AV, precision); }
};

// The same operator at a fixed precision: the learned correction's own
// products (a preconditioner term needs no FP64 accuracy), BF16 sigma.
struct FciFixedPrecision final : Fp64Apply {
    FciOperator *op = nullptr;
    int precision = kFciBF16;
    int apply(const double *V, int c, double *AV) override
    {
        return op->sigma(V, c, AV, precision);
    }
};

}  // namespace iptgb

// ---------------------------------------------------------------------------
// C ABI (include/ipt_block.h)
// ---------------------------------------------------------------------------
using namespace iptgb;

static int fci_precision(int p)
{
    return p == IPT_BLOCK_FP64 ? kFciF64 : p == IPT_BLOCK_BF16 ? kFciBF16 : p == IPT_BLOCK_FP32 ? kFciF32 : -1;
}

IPT_API int ipt_fci_dimension(const IPTFciSpec *spec, long long *n)
{
    if (spec == nullptr || n == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    fci::Tables t;
    IPTGB_CHECK(fci::build_tables(spec->norb, spec->nalpha, spec->nbeta, spec->seed,
                                  spec->offdiag_sigma, &t));
    *n = t.n;
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_fci_diagonal(const IPTFciSpec *spec, double *d_diag, void *stream)
{
    if (spec == nullptr || d_diag == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    FciOperator op;
    IPTGB_CHECK(op.init(spec->norb, spec->nalpha, spec->nbeta, spec->seed, spec->offdiag_sigma,
                        (cudaStream_t)stream));
    IPTGB_CUDA(cudaMemcpyAsync(d_diag, op.diag.ptr, (size_t)op.host.n * sizeof(double),
                               cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    IPTGB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_fci_sigma(const IPTFciSpec *spec, const double *d_X, int k, double *d_Y,
                          int precision, void *stream)
{
    if (spec == nullptr || d_X == nullptr || d_Y == nullptr || k <= 0 ||
        fci_precision(precision) < 0) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    FciOperator op;
    IPTGB_CHECK(op.init(spec->norb, spec->nalpha, spec->nbeta, spec->seed, spec->offdiag_sigma,
                        (cudaStream_t)stream));
    IPTGB_CHECK(op.sigma(d_X, k, d_Y, fci_precision(precision)));
    IPTGB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return IPT_CUDA_SUCCESS;
}

namespace {

__global__ void unit_columns_kernel(const int *__restrict__ rows, int p, long long n,
                                    double *__restrict__ X)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * p) return;
    const int c = (int)(e / n);
    const long long i = e - (long long)c * n;
    X[e] = i == rows[c] ? 1.0 : 0.0;
}

}  // namespace

IPT_API int ipt_block_solve_fci(const IPTFciSpec *spec, int k, const IPTBlockOptions *options,
                                double *d_vectors, double *d_values, IPTBlockReport *report)
{
    if (spec == nullptr || d_vectors == nullptr || d_values == nullptr || k <= 0 || k > 64) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    IPTBlockOptions opt;
    if (options != nullptr) {
        opt = *options;
    } else {
        ipt_block_default_options(&opt);
    }
    const int lowp = opt.ipt_precision == IPT_BLOCK_FP64 ? -1 : fci_precision(opt.ipt_precision);
    if (opt.ipt_precision != IPT_BLOCK_FP64 && lowp < 0) return IPT_CUDA_INVALID_ARGUMENT;
    IPTBlockReport local;
    if (report == nullptr) report = &local;
    memset(report, 0, sizeof(*report));
    cudaStream_t s = (cudaStream_t)opt.stream;
    FciOperator op;
    IPTGB_CHECK(op.init(spec->norb, spec->nalpha, spec->nbeta, spec->seed, spec->offdiag_sigma, s));
    const long long n = op.host.n;
    if (k > n || n > INT_MAX) return IPT_CUDA_INVALID_ARGUMENT;
    // ||H||_inf is bounded by max |H_II| + sigma-scaled couplings; the row sums
    // are not formed (H is never stored): use max |H_II| + 0.25 * couplings per row
    std::vector<double> hd((size_t)n);
    IPTGB_CUDA(cudaMemcpyAsync(hd.data(), op.diag.ptr, (size_t)n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    const int p = std::min<long long>(n, k + std::max(8, k / 4));
    std::vector<int> idx((size_t)n);
    std::iota(idx.begin(), idx.end(), 0);
    std::partial_sort(idx.begin(), idx.begin() + p, idx.end(),
                      [&](int a, int b) { return hd[a] < hd[b] || (hd[a] == hd[b] && a < b); });
    // ||H||_inf and the row couplings from one pass over the generated elements
    DeviceBuffer<double> rowabs, coupling;
    IPTGB_CHECK(rowabs.alloc((size_t)n, s));
    IPTGB_CHECK(coupling.alloc((size_t)n, s));
    fci::fci_rowstats_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(op.dev, rowabs.ptr,
                                                                             coupling.ptr);
    IPTGB_LAUNCH();
    std::vector<double> ra((size_t)n);
    IPTGB_CUDA(cudaMemcpyAsync(ra.data(), rowabs.ptr, (size_t)n * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    double hnorm = 0.0;
    for (double v : ra) hnorm = std::max(hnorm, v);
    DeviceBuffer<int> rows;
    DeviceBuffer<double> X0;
    IPTGB_CHECK(rows.alloc((size_t)p, s));
    IPTGB_CHECK(X0.alloc((size_t)n * p, s));
    IPTGB_CUDA(cudaMemcpyAsync(rows.ptr, idx.data(), (size_t)p * sizeof(int),
                               cudaMemcpyHostToDevice, s));
    unit_columns_kernel<<<(unsigned)(((long long)n * p + 255) / 256), 256, 0, s>>>(rows.ptr, p, n,
                                                                                 X0.ptr);
    IPTGB_LAUNCH();
    std::unique_ptr<LearnedCorrection> learned;
    if (opt.preconditioner == IPT_BLOCK_PRECOND_MLP && opt.mlp_params != nullptr) {
        learned.reset(make_learned_correction(opt.mlp_params, s));
        learned->bind(coupling.ptr, hnorm);
    }
    // the learned correction's second-order term: FP32 sigma by default
    // (BF16 with IPT_GB300_FCI_PRECOND=16, FP64-accurate with =64)
    FciFixedPrecision precond_op;
    precond_op.op = &op;
    {
        const int pp = env_int("IPT_GB300_FCI_PRECOND", 32);
        precond_op.precision = pp == 16 ? kFciBF16 : pp == 64 ? kFciF64 : kFciF32;
    }
    BlockSolveInput in;
    in.apply = &op;
    in.precond_apply = &precond_op;
    in.learned = learned.get();
    in.d = op.diag.ptr;
    in.n = (int)n;
    in.k = k;
    in.hnorm = hnorm;
    in.opt = opt;
    in.opt.oversample = p - k;
    in.initial = X0.ptr;
    in.initial_cols = p;
    DeviceBuffer<double> Xl;
    IPTBlockReport first{};
    if (lowp >= 0) {
        // low-precision sigma until its residual floor, then FP64 from the Ritz vectors
        op.precision = lowp;
        in.opt.residual_tol = lowp == kFciBF16 ? 1e-2 : 1e-5;
        IPTGB_CHECK(Xl.alloc((size_t)n * k, s));
        IPTGB_CHECK(block_solve(in, Xl.ptr, d_values, &first, s));
        in.initial = Xl.ptr;
        in.initial_cols = k;
        in.opt.residual_tol = opt.residual_tol;
    }
    op.precision = kFciF64;
    IPTGB_CHECK(block_solve(in, d_vectors, d_values, report, s));
    if (lowp >= 0) {
        report->lowp_matvecs = first.fp64_matvecs;
        report->davidson_steps += first.davidson_steps;
        report->total_ms += first.total_ms;
    }
    report->matrix_norm_inf = hnorm;
    return IPT_CUDA_SUCCESS;
}
