// Host check of the integer FP64 -> FP32 conversions the kernels use (csrc/fpbits.h) against the
// C library's conversions: split_hilo_bits against (float)v and (float)(v - hi), round_float_bits
// against (float)v, abs_bounds_bits against the neighbouring floats, widen_bits against
// (double)f.  Prints "checked split S bounds B round R failures F" and exits non-zero on a failure.
#include "fpbits.h"

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

static long failures = 0, n_split = 0, n_bounds = 0, n_round = 0;

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

int main() {
    std::mt19937_64 rng(20261204);
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
    std::printf("checked split %ld bounds %ld round %ld failures %ld\n", n_split, n_bounds, n_round, failures);
    return failures ? 1 : 0;
}
