// Host check of ddla::d2f_bits against the compiler's FP64 -> FP32 conversion
// (round to nearest even): special values, the edges of the FP32 range and
// its subnormals, ties, and random bit patterns.  Prints the number of
// mismatches (NaNs compare by class and sign) and exits 1 on any.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <random>

#include "convert.cuh"

static uint64_t bits_d(double v) { uint64_t b; std::memcpy(&b, &v, 8); return b; }
static double d_bits(uint64_t b) { double v; std::memcpy(&v, &b, 8); return v; }
static uint32_t bits_f(float v) { uint32_t b; std::memcpy(&b, &v, 4); return b; }

static long long bad = 0, total = 0;

static void check(uint64_t b) {
    const double v = d_bits(b);
    const uint32_t want = bits_f((float)v), got = ddla::d2f_bits(b);
    total++;
    if (std::isnan(v)) {
        const bool ok = (got & 0x7FC00000u) == 0x7FC00000u && (got >> 31) == (want >> 31);
        if (!ok) bad++;
        return;
    }
    if (want != got) {
        if (bad < 10) std::printf("mismatch %016llx: want %08x got %08x\n", (unsigned long long)b, want, got);
        bad++;
    }
}

int main() {
    const double specials[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38,
                               3.4028235677973362e38, 3.402823567797337e38, 1e39, -1e39, 1.1754943508222875e-38,
                               1.1754942807573643e-38, 1.401298464324817e-45, 7.006492321624085e-46,
                               7.006492321624086e-46, 2.1019476964872256e-45, 1e-50, 5e-324, -5e-324,
                               2.2250738585072014e-308, INFINITY, -INFINITY, NAN, -NAN, 0.1, 1.0 / 3.0,
                               16777217.0, 16777219.0, -16777217.0};
    for (double v : specials) {
        check(bits_d(v));
        check(bits_d(v) + 1);
        check(bits_d(v) - 1);
    }
    // ties and their neighbours at every exponent of the FP32 range and below
    for (int E = 1023 - 160; E <= 1023 + 130; E++)
        for (uint64_t low : {0x10000000ull, 0x30000000ull, 0x0FFFFFFFull, 0x10000001ull, 0x1FFFFFFFull, 0ull})
            for (uint64_t top : {0ull, 1ull << 29, 3ull << 29, 0xFFFFFull << 32}) {
                const uint64_t M = (top | low) & 0xFFFFFFFFFFFFFull;
                const uint64_t b = ((uint64_t)E << 52) | M;
                check(b);
                check(b | (1ull << 63));
            }
    // subnormal FP32 results: every tie position of the shifted significand
    for (int E = 1023 - 127 - 26; E <= 1023 - 126; E++)
        for (int sh = 0; sh < 52; sh++) {
            const uint64_t b = ((uint64_t)E << 52) | (1ull << sh);
            check(b);
            check(b - 1);
            check(b + 1);
        }
    std::mt19937_64 g(12345);
    for (int i = 0; i < 4000000; i++) check(g());
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    for (int i = 0; i < 2000000; i++) check(bits_d(u(g) * std::ldexp(1.0, (int)(g() % 300) - 150)));
    std::printf("checked %lld, mismatches %lld\n", total, bad);
    return bad ? 1 : 0;
}
