// Checks that the two digit extractions of the FP64-accurate tensor-core
// product (block_ipt_gb300/csrc/oz.cuh: the 64-bit reference form and the
// 32-bit form the kernels run) give identical digits on random values of
// every kind (scaled, full-exponent, exact fixed-point, powers of two,
// subnormal-scale rows, zero).  Built and run by tests/test_accurate_split.py.
#include <cstdio>
#include <cstring>
#include <random>
#include <cmath>
#include "oz.cuh"
using namespace iptgb;
int main() {
    std::mt19937_64 rng(7);
    long long bad = 0, n = 0;
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    for (int trial = 0; trial < 3000000; ++trial) {
        double v; int e;
        int kind = trial % 7;
        if (kind == 0) { v = u(rng); e = 0; }
        else if (kind == 1) { v = u(rng) * std::ldexp(1.0, (int)(rng() % 120) - 60); int ex; std::frexp(std::fabs(v) * (1 + (rng() % 4)), &ex); e = ex; }
        else if (kind == 2) { uint64_t bits = rng() & 0x7FFFFFFFFFFFFFFFULL; bits = (bits & 0x800FFFFFFFFFFFFFULL) | ((uint64_t)(rng() % 2046 + 1) << 52); std::memcpy(&v, &bits, 8); if (rng() & 1) v = -v; int ex; std::frexp(v, &ex); e = ex + (int)(rng() % 3); }
        else if (kind == 3) { v = std::ldexp((double)((long long)(rng() % 2000001) - 1000000), -20); e = 0; }
        else if (kind == 4) { v = std::ldexp(0.5, -(int)(rng() % 70)); if (rng()&1) v=-v; e = 0; }
        else if (kind == 5) { uint64_t bits = rng() % 0x000FFFFFFFFFFFFFULL; std::memcpy(&v, &bits, 8); e = -1000 + (int)(rng() % 40); }
        else { v = 0.0; e = (int)(rng() % 10); }
        int a[6], b[6];
        oz_digits_of(oz_fixed(v, e), a);
        oz_digits_fast(v, e, b);
        ++n;
        if (std::memcmp(a, b, sizeof(a)) != 0) { if (bad < 5) printf("mismatch v=%.17g e=%d\n", v, e); ++bad; }
    }
    printf("checked %lld mismatches %lld\n", n, bad);
    return bad != 0;
}
