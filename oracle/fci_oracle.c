/*
 * fci_oracle.c - CPU restatement of the matrix-free FCI-like Hamiltonian of
 * block_ipt_gb300/csrc/k_fci.cu (ipt_fci_* in include/ipt_block.h).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU sigma build; the product
 * never links or calls it.  The construction has no counterpart in the
 * reference (whose FCI matrices come from PySCF integrals,
 * IPT_C_GPU/test/sparse/H2O/benchmark_h2o_631g_cas10e10o_primme_vs_ipt.cu:
 * 390-766, strings and excitation links as there); it is the seeded rule
 * of the FCI-like CSR workload (block_ipt_gb300/workloads.py fci_like_csr)
 * with the normal deviates evaluated in FP32:
 *   g(s, a, b) = sqrt(-2 ln u1) cos(2 pi u2), u1 = U(s, a, b),
 *   u2 = U(s + 7919, a, b), U = float((h >> 11) | 1) 2^-53 from splitmix64
 *   hashes h of (seed, stream, a, b);
 *   eps_p = 0.5 p + 0.05 g(31, p, 0);  E(I) = occupied eps of both strings;
 *   H_II = E(I) + 0.01 g(32, I, 0) (FP64 sums);
 *   H_IJ = 0.05 g(33, min, max) exp(-|gap|) for singles/doubles, with the
 *   gap (eA(ja) - eA(ia)) + (eB(jb) - eB(ib)) formed in FP32 from the
 *   string energies rounded to FP32.
 * ln, cos and exp: range reduction + atanh / Taylor series, written from the
 * mathematics; every FP32 operation is separately rounded (compiled with
 * -ffp-contract=off, fmaf only where a fused operation is meant), so the
 * matrix elements match the GPU's bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_API __attribute__((visibility("default")))

static uint64_t sm64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ULL;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static uint64_t skey(uint64_t seed, uint64_t stream) { return sm64(seed * 0x10001ULL + stream); }

static float unif(uint64_t h1, uint64_t hi)
{
    const uint64_t h = sm64(h1 ^ (hi * 0xD1B54A32D192ED03ULL));
    return (float)((h >> 11) | 1ULL) * 0x1p-53f;
}

static float f_log(float x)
{
    uint32_t b;
    memcpy(&b, &x, 4);
    int e = (int)((b >> 23) & 0xffu) - 127;
    uint32_t mb = (b & 0x7fffffu) | 0x3f800000u;
    float m;
    memcpy(&m, &mb, 4);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float f = m - 1.0f;
    const float s = f / (2.0f + f);
    const float s2 = s * s;
    float p = fmaf(s2, 0.222222222f, 0.285714286f);
    p = fmaf(s2, p, 0.4f);
    p = fmaf(s2, p, 0.666666667f);
    p = fmaf(s2, p, 2.0f);
    return fmaf((float)e, 0.693147181f, s * p);
}

static float f_cos2pi(float u)
{
    float a = fabsf(u - 0.5f);
    float sign = -1.0f;
    if (a > 0.25f) {
        a = 0.5f - a;
        sign = 1.0f;
    }
    const float x = a * 6.28318531f;
    const float x2 = x * x;
    float c = fmaf(x2, 2.08767570e-9f, -2.75573192e-7f);
    c = fmaf(x2, c, 2.48015873e-5f);
    c = fmaf(x2, c, -1.38888889e-3f);
    c = fmaf(x2, c, 4.16666667e-2f);
    c = fmaf(x2, c, -0.5f);
    c = fmaf(x2, c, 1.0f);
    return sign * c;
}

static float f_exp(float y)
{
    if (y < -87.0f) return 0.0f;
    const float n = rintf(y * 1.44269504f);
    float r = fmaf(-n, 0.693145752f, y);
    r = fmaf(-n, 1.42860677e-6f, r);
    float p = fmaf(r, 1.98412698e-4f, 1.38888889e-3f);
    p = fmaf(r, p, 8.33333333e-3f);
    p = fmaf(r, p, 4.16666667e-2f);
    p = fmaf(r, p, 0.166666667f);
    p = fmaf(r, p, 0.5f);
    p = fmaf(r, p, 1.0f);
    p = fmaf(r, p, 1.0f);
    const int ni = (int)n;
    if (ni < -126) return 0.0f;
    const uint32_t eb = (uint32_t)(ni + 127) << 23;
    float sc;
    memcpy(&sc, &eb, 4);
    return p * sc;
}

static float gauss(uint64_t k1, uint64_t k2, uint64_t a, uint64_t b)
{
    const float u1 = unif(sm64(k1 ^ a), b);
    const float u2 = unif(sm64(k2 ^ a), b);
    const float r = sqrtf(-2.0f * f_log(u1));
    return r * f_cos2pi(u2);
}

/* ---- strings and links (lexicographic, as itertools.combinations) ---- */
typedef struct {
    int ns, nsing, ndoub;
    int *bits, *sing, *doub;
    double *occ;
    float *occf;
} Strs;

static int build_strs(int norb, int nel, const double *eps, Strs *s)
{
    int *index = (int *)malloc(sizeof(int) << norb);
    int c[32];
    for (int i = 0; i < nel; ++i) c[i] = i;
    long long cnt = 1;
    for (int i = 0; i < nel; ++i) cnt = cnt * (norb - i) / (i + 1);
    const int cap = (int)cnt;
    s->ns = cap;
    s->bits = (int *)malloc(sizeof(int) * cap);
    s->occ = (double *)malloc(sizeof(double) * cap);
    s->occf = (float *)malloc(sizeof(float) * cap);
    int n = 0;
    for (;;) {
        int bits = 0;
        for (int i = 0; i < nel; ++i) bits |= 1 << c[i];
        index[bits] = n;
        s->bits[n++] = bits;
        int i = nel - 1;
        while (i >= 0 && c[i] == norb - nel + i) --i;
        if (i < 0) break;
        ++c[i];
        for (int j = i + 1; j < nel; ++j) c[j] = c[j - 1] + 1;
    }
    const int nv = norb - nel;
    s->nsing = nel * nv;
    s->ndoub = nel * (nel - 1) / 2 * (nv * (nv - 1) / 2);
    s->sing = (int *)malloc(sizeof(int) * (size_t)cap * (s->nsing > 0 ? s->nsing : 1));
    s->doub = (int *)malloc(sizeof(int) * (size_t)cap * (s->ndoub > 0 ? s->ndoub : 1));
    for (int t = 0; t < cap; ++t) {
        const int b = s->bits[t];
        int occ[32], vir[32], no = 0, nvv = 0;
        double e = 0.0;
        for (int o = 0; o < norb; ++o) {
            if (b >> o & 1) {
                occ[no++] = o;
                e += eps[o];
            } else {
                vir[nvv++] = o;
            }
        }
        s->occ[t] = e;
        s->occf[t] = (float)e;
        int q = 0;
        for (int h = 0; h < no; ++h)
            for (int p = 0; p < nvv; ++p) s->sing[(size_t)t * s->nsing + q++] = index[b ^ (1 << occ[h]) ^ (1 << vir[p])];
        q = 0;
        for (int a1 = 0; a1 < no; ++a1)
            for (int a2 = a1 + 1; a2 < no; ++a2)
                for (int v1 = 0; v1 < nvv; ++v1)
                    for (int v2 = v1 + 1; v2 < nvv; ++v2)
                        s->doub[(size_t)t * s->ndoub + q++] =
                            index[b ^ (1 << occ[a1]) ^ (1 << occ[a2]) ^ (1 << vir[v1]) ^ (1 << vir[v2])];
    }
    free(index);
    return 0;
}

static void free_strs(Strs *s)
{
    free(s->bits);
    free(s->sing);
    free(s->doub);
    free(s->occ);
    free(s->occf);
}

typedef struct {
    Strs A, B;
    uint64_t k33a, k33b, k32a, k32b;
    float sigma;
    long long n;
} Fci;

static void fci_build(int norb, int na, int nb, uint64_t seed, double sigma, Fci *f)
{
    double eps[32];
    const uint64_t k31a = skey(seed, 31), k31b = skey(seed, 31 + 7919);
    for (int p = 0; p < norb; ++p) eps[p] = 0.5 * p + 0.05 * (double)gauss(k31a, k31b, (uint64_t)p, 0);
    build_strs(norb, na, eps, &f->A);
    build_strs(norb, nb, eps, &f->B);
    f->k33a = skey(seed, 33);
    f->k33b = skey(seed, 33 + 7919);
    f->k32a = skey(seed, 32);
    f->k32b = skey(seed, 32 + 7919);
    f->sigma = (float)sigma;
    f->n = (long long)f->A.ns * f->B.ns;
}

static double fci_diag(const Fci *f, long long I)
{
    const int ia = (int)(I / f->B.ns), ib = (int)(I % f->B.ns);
    return (f->A.occ[ia] + f->B.occ[ib]) + 0.01 * (double)gauss(f->k32a, f->k32b, (uint64_t)I, 0);
}

static float fci_value(const Fci *f, long long I, long long J, float gap)
{
    const uint64_t lo = (uint64_t)(I < J ? I : J), hi = (uint64_t)(I < J ? J : I);
    const float z = sqrtf(-2.0f * f_log(unif(sm64(f->k33a ^ lo), hi))) *
                    f_cos2pi(unif(sm64(f->k33b ^ lo), hi));
    return (f->sigma * z) * f_exp(-fabsf(gap));
}

/* Connected columns of row I in the GPU enumeration order; returns the count. */
static int fci_row(const Fci *f, long long I, long long *cols, float *vals)
{
    const int nsb = f->B.ns;
    const int ia = (int)(I / nsb), ib = (int)(I % nsb);
    const float eIa = f->A.occf[ia], eIb = f->B.occf[ib];
    int c = 0;
    const int *sa = f->A.sing + (size_t)ia * f->A.nsing, *sb = f->B.sing + (size_t)ib * f->B.nsing;
    const int *da = f->A.doub + (size_t)ia * f->A.ndoub, *db = f->B.doub + (size_t)ib * f->B.ndoub;
#define PUSH(JA, JB)                                                             \
    do {                                                                         \
        const long long J_ = (long long)(JA) * nsb + (JB);                        \
        cols[c] = J_;                                                            \
        vals[c] = fci_value(f, I, J_, (f->A.occf[JA] - eIa) + (f->B.occf[JB] - eIb)); \
        ++c;                                                                     \
    } while (0)
    for (int q = 0; q < f->A.nsing; ++q) PUSH(sa[q], ib);
    for (int q = 0; q < f->B.nsing; ++q) PUSH(ia, sb[q]);
    for (int q = 0; q < f->A.ndoub; ++q) PUSH(da[q], ib);
    for (int q = 0; q < f->B.ndoub; ++q) PUSH(ia, db[q]);
    for (int a = 0; a < f->A.nsing; ++a)
        for (int b = 0; b < f->B.nsing; ++b) PUSH(sa[a], sb[b]);
#undef PUSH
    return c;
}

ORACLE_API long long oracle_fci_dimension(int norb, int na, int nb)
{
    long long a = 1, b = 1;
    for (int i = 0; i < na; ++i) a = a * (norb - i) / (i + 1);
    for (int i = 0; i < nb; ++i) b = b * (norb - i) / (i + 1);
    return a * b;
}

ORACLE_API int oracle_fci_row_length(int norb, int na, int nb)
{
    const int va = norb - na, vb = norb - nb;
    const int sA = na * va, sB = nb * vb;
    return sA + sB + na * (na - 1) / 2 * (va * (va - 1) / 2) + nb * (nb - 1) / 2 * (vb * (vb - 1) / 2) +
           sA * sB;
}

/* diag[n]; if want_csr, CSR of the off-diagonal part plus the diagonal
 * (columns sorted within rows): row_ptr[n+1], col[n*(len+1)], val[...]. */
ORACLE_API int oracle_fci_matrix(int norb, int na, int nb, unsigned long long seed, double sigma,
                                 double *diag, int *row_ptr, int *col, double *val)
{
    const int len = oracle_fci_row_length(norb, na, nb);
    if (row_ptr != NULL && len + 1 > 4096) return -1;
    Fci f;
    fci_build(norb, na, nb, seed, sigma, &f);
    long long *cols = (long long *)malloc(sizeof(long long) * (len + 1));
    float *vals = (float *)malloc(sizeof(float) * (len + 1));
    long long pos = 0;
    for (long long I = 0; I < f.n; ++I) {
        diag[I] = fci_diag(&f, I);
        if (row_ptr == NULL) continue;
        const int c = fci_row(&f, I, cols, vals);
        /* insertion of the diagonal, then sort by column */
        long long idx[4096];
        double vv[4096];
        int m = 0;
        for (int q = 0; q < c; ++q) {
            idx[m] = cols[q];
            vv[m++] = (double)vals[q];
        }
        idx[m] = I;
        vv[m++] = diag[I];
        for (int a = 1; a < m; ++a) {
            const long long ki = idx[a];
            const double kv = vv[a];
            int b = a - 1;
            while (b >= 0 && idx[b] > ki) {
                idx[b + 1] = idx[b];
                vv[b + 1] = vv[b];
                --b;
            }
            idx[b + 1] = ki;
            vv[b + 1] = kv;
        }
        row_ptr[I] = (int)pos;
        for (int q = 0; q < m; ++q) {
            col[pos] = (int)idx[q];
            val[pos] = vv[q];
            ++pos;
        }
    }
    if (row_ptr != NULL) row_ptr[f.n] = (int)pos;
    free(cols);
    free(vals);
    free_strs(&f.A);
    free_strs(&f.B);
    return 0;
}

/* Y (n x k, column-major) = H X with FP64 accumulation in the GPU's
 * enumeration order per row (diagonal first). */
ORACLE_API int oracle_fci_sigma(int norb, int na, int nb, unsigned long long seed, double sigma,
                                const double *X, int k, double *Y)
{
    Fci f;
    fci_build(norb, na, nb, seed, sigma, &f);
    const int len = oracle_fci_row_length(norb, na, nb);
    long long *cols = (long long *)malloc(sizeof(long long) * (len + 1));
    float *vals = (float *)malloc(sizeof(float) * (len + 1));
    for (long long I = 0; I < f.n; ++I) {
        const double d = fci_diag(&f, I);
        const int c = fci_row(&f, I, cols, vals);
        for (int j = 0; j < k; ++j) {
            double s = d * X[I + (long long)j * f.n];
            for (int q = 0; q < c; ++q) s += (double)vals[q] * X[cols[q] + (long long)j * f.n];
            Y[I + (long long)j * f.n] = s;
        }
    }
    free(cols);
    free(vals);
    free_strs(&f.A);
    free_strs(&f.B);
    return 0;
}
