// FP64 <-> FP32 conversions and FP64 comparisons in integer arithmetic on the IEEE 754 bit
// patterns, for the admission pass over the nonzeros and the per-row epilogues of the checks and
// the polish.  GB300 issues FP64 instructions (conversions and comparisons included) at 1/64 of
// the FP32 rate, so a per-nonzero F2F or DADD costs about 30 us on 15M nonzeros; these forms keep
// that work on the integer and FP32 pipes.  Host and device share them, so the host tests check
// them against the C library's conversions and comparisons.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define BQP_HD __host__ __device__ __forceinline__
#else
#define BQP_HD inline
#endif

namespace bqp {

// The bit pattern of v.  On the device it comes out of an opaque move: the compiler folds masks
// and comparisons of a plain reinterpretation back into FP64 instructions (x & ~sign becomes
// |x|, materialized by an FP64 add; exponent tests become FP64 compares), which is the work these
// forms exist to avoid.
BQP_HD uint64_t bits64(double v) {
    uint64_t b;
#ifdef __CUDA_ARCH__
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(v));
#else
    memcpy(&b, &v, sizeof b);
#endif
    return b;
}

// hi = RN32(v) and lo = RN32(v - hi), the FP32 pair with v ~= hi + lo (round to nearest, ties to
// even, as an FP32 conversion in the default mode).  Exact in integer arithmetic where both parts
// are normal floats and hi is finite: biased exponent 949..1150 of v (2^-74 <= |v| < 2^128) and
// hi below the overflow threshold.  Returns false outside that window (zero included): the caller
// converts with FP64 instructions there.
//   hi: the 52-bit fraction rounded to 23 bits by adding 2^28 - 1 plus the lowest kept bit and
//       truncating; a carry moves into the exponent field, as the rounding of the value does.
//   lo: |v| - |hi| is an integer D (|D| <= 2^28) of units 2^(e-1075) (e the biased exponent of v;
//       the bit patterns of two doubles of one sign differ by the count of steps between them,
//       and every step lies in v's binade), so lo = sign(v) sign(D) RN24(|D|) 2^(e-1075).
BQP_HD bool split_hilo_bits(uint64_t bits, uint32_t& hi, uint32_t& lo) {
    const uint64_t mag = bits & 0x7fffffffffffffffull;
    const uint32_t sign = static_cast<uint32_t>(bits >> 32) & 0x80000000u;
    const int e = static_cast<int>(mag >> 52);
    if (e < 949 || e > 1150) return false;
    const uint64_t r = (mag + 0x0fffffffull + ((mag >> 29) & 1ull)) & ~0x1fffffffull;  // |hi| as FP64 bits
    const uint32_t h = static_cast<uint32_t>(r >> 29) - (896u << 23);                     // rebias 1023 -> 127
    if ((h & 0x7f800000u) == 0x7f800000u) return false;                                 // rounds to infinity
    hi = h | sign;
    const int64_t D = static_cast<int64_t>(mag - r);
    if (D == 0) {
        lo = 0;  // v - hi = +0 in round-to-nearest
        return true;
    }
    uint32_t m = static_cast<uint32_t>(D < 0 ? -D : D);
#ifdef __CUDA_ARCH__
    const int p = 31 - __clz(m);  // leading bit, p <= 28
#else
    const int p = 31 - __builtin_clz(m);
#endif
    uint32_t mant;
    if (p <= 23) {
        mant = m << (23 - p);
    } else {
        const int sh = p - 23;
        mant = (m + ((1u << (sh - 1)) - 1u) + ((m >> sh) & 1u)) >> sh;  // in [2^23, 2^24]
    }
    // biased exponent p + e - 1075 + 127 >= 1; mant = 2^24 carries into the exponent
    lo = ((static_cast<uint32_t>(p + e - 948) << 23) + (mant - 0x00800000u)) | (sign ^ (D < 0 ? 0x80000000u : 0u));
    return true;
}

// RN32(v) (round to nearest, ties to even) in integer arithmetic where the result is a normal
// finite float: biased exponent 897..1150 of v and no overflow; returns false elsewhere (zero
// included), where the caller converts with an FP64 instruction.
BQP_HD bool round_float_bits(uint64_t bits, uint32_t& f) {
    const uint64_t mag = bits & 0x7fffffffffffffffull;
    const int e = static_cast<int>(mag >> 52);
    if (e < 897 || e > 1150) return false;
    const uint32_t h = static_cast<uint32_t>((mag + 0x0fffffffull + ((mag >> 29) & 1ull)) >> 29) - (896u << 23);
    if ((h & 0x7f800000u) == 0x7f800000u) return false;
    f = h | (static_cast<uint32_t>(bits >> 32) & 0x80000000u);
    return true;
}

// FP32 bounds of a magnitude given by its FP64 bits: rd <= |v| <= ru.  Inside the normal FP32
// range they are the nearest floats below and above (truncation, plus one unit when a dropped
// bit is set); below it 0 and 2^-126, above it FLT_MAX and infinity.
BQP_HD void abs_bounds_bits(uint64_t mag, uint32_t& rd, uint32_t& ru) {
    const int e = static_cast<int>(mag >> 52);
    if (e >= 897 && e <= 1150) {
        rd = static_cast<uint32_t>(mag >> 29) - (896u << 23);
        ru = rd + ((mag & 0x1fffffffull) != 0 ? 1u : 0u);
    } else if (e < 897) {
        rd = 0;
        ru = mag ? 0x00800000u : 0u;
    } else {
        rd = 0x7f7fffffu;
        ru = 0x7f800000u;
    }
}

// FP64 bits of a non-negative float that is 0, normal or infinite (the FP32 sums of
// abs_bounds_bits values are nothing else).
BQP_HD uint64_t widen_bits(uint32_t f) {
    if (f == 0) return 0;
    if (f >= 0x7f800000u) return 0x7ff0000000000000ull;
    return (static_cast<uint64_t>(f) + (896ull << 23)) << 29;
}

// FP64 bits of a float of either sign that is zero or normal; false for subnormals, infinities
// and NaNs, which the caller converts with an FP64 instruction.
BQP_HD bool widen_signed_bits(uint32_t f, uint64_t& d) {
    const uint32_t mag = f & 0x7fffffffu;
    const uint64_t sign = static_cast<uint64_t>(f & 0x80000000u) << 32;
    if (mag == 0) {
        d = sign;
        return true;
    }
    if (mag < 0x00800000u || mag >= 0x7f800000u) return false;
    d = ((static_cast<uint64_t>(mag) + (896ull << 23)) << 29) | sign;
    return true;
}

// IEEE 754 comparisons of two doubles given by their bit patterns, in integer arithmetic: false
// when either is a NaN, and -0 equal to +0, as the FP64 comparison instructions decide.
constexpr uint64_t kAbsMask64 = 0x7fffffffffffffffull;
constexpr uint64_t kExpMask64 = 0x7ff0000000000000ull;
BQP_HD bool nan_bits(uint64_t b) { return (b & kAbsMask64) > kExpMask64; }
BQP_HD bool finite_bits(uint64_t b) { return (b & kExpMask64) != kExpMask64; }
// a key whose unsigned order is the numeric order of non-NaN doubles (-0 just below +0)
BQP_HD uint64_t order_key(uint64_t b) { return (b >> 63) ? ~b : (b | 0x8000000000000000ull); }
BQP_HD bool less_bits(uint64_t a, uint64_t b) {
    if (nan_bits(a) || nan_bits(b) || ((a | b) & kAbsMask64) == 0) return false;
    return order_key(a) < order_key(b);
}
BQP_HD bool less_equal_bits(uint64_t a, uint64_t b) {
    if (nan_bits(a) || nan_bits(b)) return false;
    return ((a | b) & kAbsMask64) == 0 || order_key(a) <= order_key(b);
}

// FP32 conversions of a double in a given rounding direction (dir 0 to nearest even, 1 up, -1
// down), in integer arithmetic for zeros, infinities and every result that is a normal float or
// an overflow; false for results in FP32's subnormal range and for NaNs, which the caller
// converts with an FP64 instruction.  Up and down come from the magnitude's bounds
// (abs_bounds_bits): RU(x) = ru(|x|) and RD(x) = rd(|x|) for x > 0, -rd(|x|) and -ru(|x|) for x < 0.
BQP_HD bool round_dir_bits(uint64_t bits, int dir, uint32_t& f) {
    const uint64_t mag = bits & kAbsMask64;
    const uint32_t sign = static_cast<uint32_t>(bits >> 32) & 0x80000000u;
    if (mag == 0 || mag == kExpMask64) {  // zeros and infinities keep their sign
        f = sign | (mag ? 0x7f800000u : 0u);
        return true;
    }
    const int e = static_cast<int>(mag >> 52);
    if (e < 897 || mag > kExpMask64) return false;  // a subnormal result, or a NaN
    if (dir == 0) {
        if (e > 1150) {  // beyond every float: rounds to infinity
            f = sign | 0x7f800000u;
            return true;
        }
        if (round_float_bits(bits, f)) return true;
        f = sign | 0x7f800000u;  // rounds past the largest float
        return true;
    }
    uint32_t rd, ru;
    abs_bounds_bits(mag, rd, ru);
    const bool away = (dir > 0) == (sign == 0);  // rounding away from zero
    f = sign | (away ? ru : rd);
    return true;
}

BQP_HD float float_of_bits(uint32_t b) {
    float f;
    memcpy(&f, &b, sizeof f);
    return f;
}

// A lower bound of a * b for non-negative floats: the product rounded down (the host forms the
// exact product in FP64 and truncates it to FP32, flushing below the normal range to 0).
BQP_HD float mul_rd_nonneg(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rd(a, b);
#else
    uint32_t rd, ru;
    abs_bounds_bits(bits64(static_cast<double>(a) * static_cast<double>(b)), rd, ru);
    return float_of_bits(rd);
#endif
}

// Whether num / RN64(1 + |x|), rounded to FP64, can exceed m (num and m non-negative doubles,
// num finite; all three given by their bits).  No when RU32(num) <= RD32(RD32(m) * max(1,
// RD32(|x|))): then num <= m * RN64(1 + |x|), because max(1, |x|) <= RN64(1 + |x|), and the
// rounded quotient is at most m.  Integer and FP32 arithmetic only.
BQP_HD bool ratio_may_exceed(uint64_t num, uint64_t x, uint64_t m) {
    uint32_t nrd, nru, xrd, xru, mrd, mru;
    abs_bounds_bits(num, nrd, nru);
    abs_bounds_bits(x & kAbsMask64, xrd, xru);
    abs_bounds_bits(m, mrd, mru);
    const float xf = float_of_bits(xrd);
    const float den = xf > 1.0f ? xf : 1.0f;
    return float_of_bits(nru) > mul_rd_nonneg(float_of_bits(mrd), den);
}

}  // namespace bqp
