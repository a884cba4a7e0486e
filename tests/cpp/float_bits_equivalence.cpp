// Checks the integer-pipe double -> float rounding of the batched solver's
// FP32 sweeps (block_ipt_gb300/csrc/fpconv.cuh, double_to_float_bits)
// against the host's IEEE conversion (round to nearest even), bit for bit,
// wherever the helper accepts the value, on random values of every exponent
// and on exact ties of the dropped bits.  Built and run by
// tests/test_split.py.
#include <cstdio>
#include <cstring>
#include <random>
#include "fpconv.cuh"
using namespace iptgb;
int main() {
    std::mt19937_64 rng(11);
    long long bad = 0, accepted = 0, n = 0;
    for (long long trial = 0; trial < 4000000; ++trial) {
        uint64_t bits = rng();
        if (trial % 3 == 0) {
            // exponents around the float range
            bits = (bits & 0x800FFFFFFFFFFFFFULL) | ((uint64_t)(1023 - 160 + rng() % 320) << 52);
        } else if (trial % 3 == 1) {
            // exact ties of the 29 dropped bits
            bits = (bits & 0x800FFFFFE0000000ULL) | (1ULL << 28) |
                   ((uint64_t)(1023 - 126 + rng() % 254) << 52);
        }
        double v;
        std::memcpy(&v, &bits, 8);
        if (v != v) continue;
        ++n;
        uint32_t got;
        if (!double_to_float_bits(bits, &got)) continue;
        ++accepted;
        const float want = (float)v;
        uint32_t wb;
        std::memcpy(&wb, &want, 4);
        if (wb != got) {
            if (bad < 5) printf("mismatch %.17g\n", v);
            ++bad;
        }
    }
    printf("values %lld accepted %lld mismatches %lld\n", n, accepted, bad);
    return bad != 0 || accepted < n / 2;
}
