// java_random.h -- java.util.Random on the host, bit-exact with Java.
//
// The generator the Java SE API documentation specifies: a 48-bit linear
// congruential generator (multiplier 0x5DEECE66D, addend 0xB); nextDouble
// takes 26 + 27 bits; nextGaussian is the polar method with one cached
// deviate and uses StrictMath.log, i.e. the fdlibm logarithm, restated here:
// x = 2^k (1+f) with sqrt(2)/2 < 1+f < sqrt(2), s = f/(2+f),
// log(1+f) = f - s (f - R(s^2)) with fdlibm's minimax polynomial R, and k ln2
// split into a high and a low part.  Compile without floating-point
// contraction (-ffp-contract=off) so that every host gives the same bits.
//
// fdlibm_log restates fdlibm's e_log.c (its constants and reduction steps),
// which carries this notice:
// ====================================================
// Copyright (C) 1993 by Sun Microsystems, Inc. All rights reserved.
//
// Developed at SunSoft, a Sun Microsystems, Inc. business.
// Permission to use, copy, modify, and distribute this
// software is freely granted, provided that this notice
// is preserved.
// ====================================================
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace opx {

inline double fdlibm_log(double x) {
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10,
                 two54 = 1.80143985094819840000e+16;
    const double Lg1 = 6.666666666666735130e-01, Lg2 = 3.999999999940941908e-01, Lg3 = 2.857142874366239149e-01,
                 Lg4 = 2.222219843214978396e-01, Lg5 = 1.818357216161805012e-01, Lg6 = 1.531383769920937332e-01,
                 Lg7 = 1.479819860511658591e-01;
    uint64_t bits;
    std::memcpy(&bits, &x, 8);
    int32_t hx = (int32_t)(bits >> 32);
    int32_t k = 0;
    if (hx < 0x00100000) {  // subnormal argument
        k -= 54;
        x *= two54;
        std::memcpy(&bits, &x, 8);
        hx = (int32_t)(bits >> 32);
    }
    k += (hx >> 20) - 1023;
    hx &= 0x000fffff;
    int32_t i = (hx + 0x95f64) & 0x100000;
    bits = ((uint64_t)(uint32_t)(hx | (i ^ 0x3ff00000)) << 32) | (bits & 0xffffffffULL);
    std::memcpy(&x, &bits, 8);
    k += i >> 20;
    const double f = x - 1.0;
    const double dk = (double)k;
    if ((0x000fffff & (2 + hx)) < 3) {  // |f| < 2^-20
        if (f == 0.0) return k == 0 ? 0.0 : dk * ln2_hi + dk * ln2_lo;
        const double R = f * f * (0.5 - 0.33333333333333333 * f);
        return k == 0 ? f - R : dk * ln2_hi - ((R - dk * ln2_lo) - f);
    }
    const double s = f / (2.0 + f);
    const double z = s * s, w = z * z;
    const int32_t sel = (hx - 0x6147a) | (0x6b851 - hx);
    const double t1 = w * (Lg2 + w * (Lg4 + w * Lg6));
    const double t2 = z * (Lg1 + w * (Lg3 + w * (Lg5 + w * Lg7)));
    const double R = t2 + t1;
    if (sel > 0) {
        const double hfsq = 0.5 * f * f;
        return k == 0 ? f - (hfsq - s * (hfsq + R)) : dk * ln2_hi - ((hfsq - (s * (hfsq + R) + dk * ln2_lo)) - f);
    }
    return k == 0 ? f - s * (f - R) : dk * ln2_hi - ((s * (f - R) - dk * ln2_lo) - f);
}

struct JavaRandom {
    uint64_t seed;
    bool have = false;
    double next_g = 0;
    explicit JavaRandom(int64_t s) { seed = ((uint64_t)s ^ 0x5DEECE66DULL) & ((1ULL << 48) - 1); }
    int32_t next(int bits) {
        seed = (seed * 0x5DEECE66DULL + 0xBULL) & ((1ULL << 48) - 1);
        return (int32_t)(int64_t)(seed >> (48 - bits));
    }
    double next_double() { return (double)(((int64_t)next(26) << 27) + next(27)) * 0x1.0p-53; }
    double next_gaussian() {
        if (have) { have = false; return next_g; }
        double v1, v2, s;
        do {
            v1 = 2 * next_double() - 1;
            v2 = 2 * next_double() - 1;
            s = v1 * v1 + v2 * v2;
        } while (s >= 1 || s == 0);
        const double mul = std::sqrt(-2 * fdlibm_log(s) / s);
        next_g = v2 * mul;
        have = true;
        return v1 * mul;
    }
};

}  // namespace opx
