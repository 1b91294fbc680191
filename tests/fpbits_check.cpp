// Host check of the integer FP64 <-> FP32 conversions and FP64 comparisons the kernels use
// (csrc/fpbits.h) against the C library: split_hilo_bits against (float)v and (float)(v - hi),
// round_float_bits against (float)v, abs_bounds_bits against the neighbouring floats, widen_bits
// and widen_signed_bits against (double)f, less_bits / less_equal_bits against a < b and a <= b,
// ratio_may_exceed's "no" against the FP64 quotient num / (1 + |x|) <= m, and round_dir_bits
// against the conversion under the C library's rounding modes (compiled with -frounding-math).
// Prints "checked split S bounds B round R widen W compare C ratio Q (skipped K) directed D
// failures F" and exits non-zero on a failure.
#include "fpbits.h"

#include <cfenv>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

using bqp::abs_bounds_bits;
using bqp::split_hilo_bits;
using bqp::widen_bits;

static uint32_t fbits(float f) {
    uint32_t b;
    std::memcpy(&b, &f, sizeof b);
    return b;
}
static float ffrom(uint32_t b) {
    float f;
    std::memcpy(&f, &b, sizeof f);
    return f;
}
static double dfrom(uint64_t b) {
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
}

static long failures = 0, n_split = 0, n_bounds = 0, n_round = 0, n_widen = 0, n_compare = 0, n_ratio = 0,
            n_skipped = 0, n_directed = 0;

static void fail(const char* what, double v) {
    if (failures++ < 20) std::printf("FAIL %s at %.17g (bits %016llx)\n", what, v, (unsigned long long)bqp::bits64(v));
}

static void check(double v) {
    const uint64_t bits = bqp::bits64(v);
    uint32_t h, l;
    if (split_hilo_bits(bits, h, l)) {
        ++n_split;
        const float hf = static_cast<float>(v);
        const float lf = static_cast<float>(v - static_cast<double>(hf));
        if (h != fbits(hf)) fail("split hi", v);
        if (l != fbits(lf)) fail("split lo", v);
    }
    uint32_t f;
    if (bqp::round_float_bits(bits, f)) {
        ++n_round;
        if (f != fbits(static_cast<float>(v))) fail("round", v);
    }
    if (!std::isfinite(v)) return;
    const uint64_t mag = bits & 0x7fffffffffffffffull;
    const double a = std::fabs(v);
    uint32_t rd, ru;
    abs_bounds_bits(mag, rd, ru);
    ++n_bounds;
    const float frd = ffrom(rd), fru = ffrom(ru);
    if (!(static_cast<double>(frd) <= a)) fail("bounds rd above", v);
    if (!(static_cast<double>(fru) >= a)) fail("bounds ru below", v);
    if (a >= FLT_MIN && a <= FLT_MAX) {  // nearest floats inside the normal range
        if (static_cast<double>(std::nextafter(frd, INFINITY)) <= a && static_cast<double>(frd) != a) fail("rd not nearest", v);
        if (static_cast<double>(std::nextafter(fru, 0.0f)) >= a && static_cast<double>(fru) != a) fail("ru not nearest", v);
    }
    for (uint32_t f : {rd, ru}) {
        if (f != 0 && f < 0x00800000u) continue;  // subnormal: never produced by a sum of these bounds
        if (widen_bits(f) != bqp::bits64(static_cast<double>(ffrom(f)))) fail("widen", v);
    }
}

// widen_signed_bits against the C conversion, for one float pattern
static void check_widen(uint32_t f) {
    uint64_t d;
    const float v = ffrom(f);
    const uint32_t mag = f & 0x7fffffffu;
    const bool expect = mag == 0 || (mag >= 0x00800000u && mag < 0x7f800000u);
    if (bqp::widen_signed_bits(f, d) != expect) {
        fail("widen_signed accepts", static_cast<double>(v));
        return;
    }
    ++n_widen;
    if (expect && d != bqp::bits64(static_cast<double>(v))) fail("widen_signed", static_cast<double>(v));
}

static void check_compare(double a, double b) {
    ++n_compare;
    const uint64_t x = bqp::bits64(a), y = bqp::bits64(b);
    if (bqp::less_bits(x, y) != (a < b)) fail("less", a);
    if (bqp::less_equal_bits(x, y) != (a <= b)) fail("less_equal", a);
    if (bqp::finite_bits(x) != static_cast<bool>(std::isfinite(a))) fail("finite", a);
    if (bqp::nan_bits(x) != static_cast<bool>(std::isnan(a))) fail("nan", a);
}

// ratio_may_exceed(num, x, m) false must mean RN64(num / RN64(1 + |x|)) <= m
static void check_ratio(double num, double x, double m) {
    ++n_ratio;
    if (bqp::ratio_may_exceed(bqp::bits64(num), bqp::bits64(x), bqp::bits64(m))) return;
    ++n_skipped;
    const volatile double den = 1.0 + std::fabs(x);
    const volatile double q = num / den;
    if (!(q <= m)) fail("ratio skipped above the maximum", num);
}

// round_dir_bits in the three directions against (float)v under the matching rounding mode
static void check_directed(double v) {
    static const int modes[3] = {FE_TONEAREST, FE_UPWARD, FE_DOWNWARD};
    static const int dirs[3] = {0, 1, -1};
    for (int i = 0; i < 3; ++i) {
        uint32_t f;
        if (!bqp::round_dir_bits(bqp::bits64(v), dirs[i], f)) {
            // only NaNs and results in the subnormal range fall back
            const double a = std::fabs(v);
            if (!(std::isnan(v) || (a != 0 && a < FLT_MIN))) fail("directed refused", v);
            continue;
        }
        std::fesetround(modes[i]);
        volatile double in = v;
        volatile float out = static_cast<float>(in);
        std::fesetround(FE_TONEAREST);
        ++n_directed;
        if (f != fbits(out)) fail(i == 0 ? "directed RN" : (i == 1 ? "directed RU" : "directed RD"), v);
    }
}

int main() {
    std::mt19937_64 rng(20261204);
    // directed conversions: random patterns over every exponent, the float range's edges, zeros
    // and infinities of both signs
    for (int i = 0; i < 1000000; ++i) {
        const uint64_t e = (i & 1) ? rng() % 2047 : 890 + rng() % 270;
        check_directed(dfrom((rng() & 0x800fffffffffffffull) | (e << 52)));
    }
    for (double v : {0.0, -0.0, static_cast<double>(INFINITY), -static_cast<double>(INFINITY), 1.0, -1.0,
                     static_cast<double>(FLT_MAX), -static_cast<double>(FLT_MAX), static_cast<double>(FLT_MIN),
                     -static_cast<double>(FLT_MIN), 1e300, -1e300, 1e-300, -1e-300, 0.1, -0.1})
        check_directed(v);
    for (int k = -3; k <= 3; ++k) {
        check_directed(std::nextafter(static_cast<double>(FLT_MAX), k < 0 ? 0.0 : 1e300) * (1.0 + k * 1e-10));
        check_directed(-std::nextafter(static_cast<double>(FLT_MAX), k < 0 ? 0.0 : 1e300) * (1.0 + k * 1e-10));
        check_directed(static_cast<double>(FLT_MIN) * (1.0 + k * 1e-9));
    }
    // signed widening: random patterns over every exponent, and the range edges
    for (int i = 0; i < 1000000; ++i) check_widen(static_cast<uint32_t>(rng()));
    for (uint32_t f : {0u, 0x80000000u, 1u, 0x007fffffu, 0x00800000u, 0x80800000u, 0x7f7fffffu, 0xff7fffffu,
                       0x7f800000u, 0xff800000u, 0x7fc00000u, 0x3f800000u, 0xbf800000u})
        check_widen(f);
    // comparisons: special values against each other, random pairs, equal and adjacent pairs
    const double specials[] = {0.0, -0.0, 1.0, -1.0, INFINITY, -INFINITY, NAN, -NAN, DBL_MIN, -DBL_MIN,
                               DBL_TRUE_MIN, -DBL_TRUE_MIN, DBL_MAX, -DBL_MAX, 1e-300, -1e300, 3.0, -3.0};
    for (double a : specials)
        for (double b : specials) check_compare(a, b);
    for (int i = 0; i < 1000000; ++i) {
        const double a = dfrom(rng()), b = (i & 3) == 0 ? a : dfrom(rng());
        check_compare(a, b);
        check_compare(a, std::nextafter(a, INFINITY));
        check_compare(std::nextafter(a, -INFINITY), a);
        check_compare(-a, b);
    }
    // the division filter: quotients near the maximum (within a few ulps either side), tiny and
    // huge magnitudes, |x| around 1 where max(1, |x|) is loosest
    std::uniform_real_distribution<double> unit(0.0, 1.0);
    for (int i = 0; i < 2000000; ++i) {
        const double x = (i & 1 ? 1.0 : -1.0) * std::ldexp(unit(rng), static_cast<int>(rng() % 80) - 40);
        const double m = std::ldexp(unit(rng), static_cast<int>(rng() % 200) - 150);
        const double q0 = m * (1.0 + std::fabs(x));
        double num = q0;
        const int steps = static_cast<int>(rng() % 9) - 4;
        for (int k = 0; k < (steps < 0 ? -steps : steps); ++k) num = std::nextafter(num, steps < 0 ? 0.0 : INFINITY);
        if (i % 5 == 0) num *= unit(rng);
        check_ratio(num, x, m);
        check_ratio(num, x, std::nextafter(m, 0.0));
    }
    for (double num : {0.0, DBL_TRUE_MIN, 1e-300, 1e-40, 1.0, 3e38, 1e300}) {
        for (double x : {0.0, -0.0, 1e-30, 0.5, 1.0, -1.0, 2.0, 1e30, 1e300, -1e300}) {
            for (double m : {0.0, DBL_TRUE_MIN, 1e-300, 1e-40, 1e-7, 1.0, 3e38, 1e300, static_cast<double>(INFINITY)}) check_ratio(num, x, m);
        }
    }
    // random bit patterns over the whole exponent range, both signs
    for (int i = 0; i < 2000000; ++i) {
        const uint64_t e = (i & 1) ? rng() % 2047 : 890 + rng() % 270;  // half of them around the window
        const uint64_t b = (rng() & 0x800fffffffffffffull) | (e << 52);
        check(dfrom(b));
    }
    // the exponent window's edges and rounding ties: fractions with the dropped 29 bits at, just
    // below and just above half a unit, kept lsb even and odd, and the carries into the exponent
    const uint64_t lows[] = {0, 1, 0x0fffffffull, 0x10000000ull, 0x10000001ull, 0x1fffffffull, 0x0ffffffeull};
    for (uint64_t e : {896ull, 897ull, 948ull, 949ull, 950ull, 1022ull, 1023ull, 1149ull, 1150ull, 1151ull, 1152ull}) {
        for (uint64_t hi23 : {0ull, 1ull, 2ull, 0x7ffffeull, 0x7fffffull, 0x400000ull}) {
            for (uint64_t lo : lows) {
                for (uint64_t s : {0ull, 1ull}) {
                    const uint64_t b = (s << 63) | (e << 52) | (hi23 << 29) | lo;
                    check(dfrom(b));
                }
            }
        }
    }
    // values near FLT_MAX (the overflow threshold of the nearest float) and near 2^-74
    for (int k = -4; k <= 4; ++k) {
        check(std::nextafter(static_cast<double>(FLT_MAX), k < 0 ? 0.0 : INFINITY) * (1.0 + k * 1e-9));
        check(std::ldexp(1.0, -74) * (1.0 + k * 1e-12));
    }
    check(0.0);
    check(-0.0);
    check(1.0);
    check(-2.0);
    check(1.0 / 3.0);
    check(3.4028235677973366e38);  // rounds to infinity in FP32
    std::printf("checked split %ld bounds %ld round %ld widen %ld compare %ld ratio %ld (skipped %ld) directed %ld "
                "failures %ld\n",
                n_split, n_bounds, n_round, n_widen, n_compare, n_ratio, n_skipped, n_directed, failures);
    return failures ? 1 : 0;
}
