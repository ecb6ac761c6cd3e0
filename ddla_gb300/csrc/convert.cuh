// FP64 -> FP32 conversion on the integer pipes.
//
// GB300 runs the FP64 -> FP32 conversion instruction at its FP64 rate
// (1/64 of FP32), which makes a pass that converts every entry of an n x n
// FP64 matrix FP64-pipe bound.  This conversion works on the IEEE 754 fields
// with 32- and 64-bit integer operations instead and gives the same result as
// a round-to-nearest-even conversion: the significand rounded to 24 bits (ties
// to even), overflow to infinity, results below half the smallest FP32
// subnormal to zero, infinities kept, NaNs kept quiet with the sign and the
// leading payload bits.  Written as plain C++ so a host test can check it bit
// for bit against the compiler's own conversion.
#pragma once

#ifdef __CUDACC__
#define DDLA_HD __host__ __device__ __forceinline__
#else
#define DDLA_HD inline
#endif

namespace ddla {

// Bits of the FP32 nearest to the FP64 value with bits b.
DDLA_HD unsigned d2f_bits(unsigned long long b) {
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int E = (int)((b >> 52) & 0x7FF);
    const unsigned long long M = b & 0xFFFFFFFFFFFFFull;
    unsigned r;
    if (E == 0x7FF) {
        r = M ? (0x7FC00000u | (unsigned)(M >> 29)) : 0x7F800000u;
    } else {
        const int e = E - 1023 + 127;   // biased FP32 exponent of a normal result
        if (e >= 255) {
            r = 0x7F800000u;
        } else if (e >= 1) {
            // keep 23 of the 52 fraction bits; a carry out of the fraction
            // steps the exponent (to infinity past the largest finite value)
            const unsigned m = (unsigned)(M >> 29);
            const unsigned rem = (unsigned)(M & 0x1FFFFFFFull);
            r = ((unsigned)e << 23) + m + ((rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u);
        } else {
            // FP32 subnormal (or zero): the significand with its leading one
            // in units of 2^-149 is sig / 2^(30 - e); a carry into bit 23
            // gives the smallest normal
            const int sh = 30 - e;
            if (sh >= 55) {
                r = 0u;   // below half of 2^-149
            } else {
                const unsigned long long sig = M | (1ull << 52);
                const unsigned m = (unsigned)(sig >> sh);
                const unsigned long long rem = sig & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
                r = m + ((rem > half || (rem == half && (m & 1u))) ? 1u : 0u);
            }
        }
    }
    return sign | r;
}

}  // namespace ddla
