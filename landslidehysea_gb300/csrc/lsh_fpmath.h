// lsh_fpmath.h -- the few elementary functions the scheme needs beyond
// +, -, *, /, sqrt and fma, written so the host (CPU oracle) and the device
// (CUDA kernels) produce bit-identical results: each one uses only IEEE-754
// basic operations in a fixed order, never a vendor libm.
//
//   exp_neg(x) = e^-x, x >= 0.  Cody & Waite argument reduction
//       (-x = k ln2 + r, ln2 split in a 32-bit-exact high part and a low
//       part), e^r by its Taylor series to r^13/13! in Horner form, then a
//       scaling by 2^k built from the exponent bits (two steps below 2^-1021
//       so subnormal results round once).  Exactly 1 for x < 2^-54 and
//       exactly 0 for x > 746 (what a correctly rounded exp returns there).
//   cbrt_pos(x) = x^(1/3), x >= 0.  x = a 2^(3q) with a in [1, 8) (integer
//       ops); z ~ a^(-1/3) by Newton's method on f(z) = z^-3 - a, written
//       without division as z <- z + (z / 3)(1 - a z^3): a quadratic first
//       guess (4.4% error) and three steps in FP32 on a's leading 24 bits
//       (to about 1e-7: FP32 rounding), then two FP64 steps (the error
//       squares each step); a^(1/3) = a z^2, and 2^q is added to the
//       exponent bits.  Within a few ulp; about 12 FP64 operations, the rest
//       on the FP32 and integer pipes.  FP32 basic operations and fmaf are
//       IEEE on host and device alike, so both give the same bits.
//   log_pos(x) = ln x, x > 0.  x = m 2^e with m in [sqrt(1/2), sqrt(2)),
//       ln m = 2 atanh(s), s = (m - 1)/(m + 1), by its odd series to s^23.
// Accuracy: a few ulp (tests/test_fpmath.py checks them against the C
// library); what matters here is that both sides compute the same bits.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define LSH_HD __host__ __device__ __forceinline__
#else
#define LSH_HD inline
#endif

namespace lshm {

LSH_HD uint64_t bits_of(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    std::memcpy(&u, &x, sizeof(u));
    return u;
#endif
}

LSH_HD double from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    std::memcpy(&x, &u, sizeof(x));
    return x;
#endif
}

LSH_HD double fmad(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
    return fma(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

LSH_HD float fmadf(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return fmaf(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}

LSH_HD uint32_t fbits_of(float x) {
#if defined(__CUDA_ARCH__)
    return (uint32_t)__float_as_uint(x);
#else
    uint32_t u;
    std::memcpy(&u, &x, sizeof(u));
    return u;
#endif
}

LSH_HD float ffrom_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, sizeof(x));
    return x;
#endif
}

LSH_HD double rint_even(double x) {
#if defined(__CUDA_ARCH__)
    return rint(x);
#else
    return std::nearbyint(x);  // default rounding mode: to nearest, ties to even
#endif
}

// The two 32-bit halves of x.  On the device through a PTX move, which the
// compiler cannot see through: an integer test on the bits that is
// equivalent to a floating-point compare (x == 0, !isfinite(x)) would
// otherwise be folded back into an FP64 compare.
LSH_HD void halves(double x, uint32_t& lo, uint32_t& hi) {
#if defined(__CUDA_ARCH__)
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
#else
    const uint64_t u = bits_of(x);
    lo = (uint32_t)u;
    hi = (uint32_t)(u >> 32);
#endif
}

LSH_HD double from_halves(uint32_t lo, uint32_t hi) {
#if defined(__CUDA_ARCH__)
    double x;
    asm("mov.b64 %0, {%1, %2};" : "=d"(x) : "r"(lo), "r"(hi));
    return x;
#else
    return from_bits(((uint64_t)hi << 32) | lo);
#endif
}

// c ? -x : x by flipping the sign bit (integer pipe): the bits of -x
LSH_HD double neg_if(double x, bool c) {
    uint32_t lo, hi;
    halves(x, lo, hi);
    return from_halves(lo, hi ^ ((uint32_t)c << 31));
}

// 2^k for -1022 <= k <= 1023
LSH_HD double pow2i(int k) { return from_bits((uint64_t)(k + 1023) << 52); }

// ---- comparisons on the integer pipe
//
// The GPU's FP64 unit takes one warp instruction per 16 cycles per SM, and a
// double compare occupies it like an add.  These forms compare bit patterns
// on the integer ALUs instead.  For operands that are not NaN each returns
// exactly what the IEEE comparison returns (-0 == +0), so they are exact
// restatements of the compares they replace.

constexpr uint64_t kMag = 0x7fffffffffffffffULL;

// x > 0
LSH_HD bool gt0(double x) { return (int64_t)bits_of(x) > 0; }
// x < 0
LSH_HD bool lt0(double x) {
    const uint64_t u = bits_of(x);
    return (int64_t)u < 0 && (u << 1) != 0;
}
// x < c and x > c for a constant c > 0: doubles >= -0 order like their
// patterns, and every negative pattern (-0 included) is below c's
LSH_HD bool lt_pos(double x, double c) { return (int64_t)bits_of(x) < (int64_t)bits_of(c); }
LSH_HD bool gt_pos(double x, double c) { return (int64_t)bits_of(x) > (int64_t)bits_of(c); }
// |x| by clearing the sign bit (integer pipe): the bits fabs gives.  A
// fabs whose result feeds an integer-pipe compare would otherwise be
// materialised by an FP64 instruction.
LSH_HD double abs_bits(double x) { return from_bits(bits_of(x) & kMag); }
// |a| < |b|
LSH_HD bool abs_lt(double a, double b) { return (bits_of(a) & kMag) < (bits_of(b) & kMag); }
// a key ordered like the doubles, -0 and +0 both 0: the magnitude, negated
// for a negative value
LSH_HD int64_t okey(double x) {
    const int64_t k = (int64_t)bits_of(x);
    return (k < 0) ? -(k & (int64_t)kMag) : k;
}
// a < b, any non-NaN a and b
LSH_HD bool lt(double a, double b) { return okey(a) < okey(b); }

constexpr int64_t kInfBits = 0x7ff0000000000000LL;  // +inf; positive NaNs lie above

LSH_HD double exp_neg(double x) {
    // the range tests on the integer pipe: x < 2^-54 (negative x, -0 and
    // negative NaNs included), then 746 < x <= +inf; NaN stays NaN
    const int64_t k0 = (int64_t)bits_of(x);
    if (k0 < (int64_t)bits_of(0x1p-54)) return (k0 & (int64_t)kMag) > kInfBits ? x : 1.0;
    if (k0 > (int64_t)bits_of(746.0) && k0 <= kInfBits) return 0.0;
    const double inv_ln2 = 1.4426950408889634074;
    const double ln2_hi = 6.93147180369123816490e-01;  // 0x3fe62e42fee00000: low 32 bits zero
    const double ln2_lo = 1.90821492927058770002e-10;
    const double kd = rint_even(-x * inv_ln2);
    double r = fmad(kd, -ln2_hi, -x);
    r = fmad(kd, -ln2_lo, r);
    // Taylor coefficients 1/n!, n = 13 .. 2
    double p = 1.6059043836821614599e-10;
    p = fmad(p, r, 2.0876756987868098979e-09);
    p = fmad(p, r, 2.5052108385441718775e-08);
    p = fmad(p, r, 2.7557319223985890653e-07);
    p = fmad(p, r, 2.7557319223985890653e-06);
    p = fmad(p, r, 2.4801587301587301587e-05);
    p = fmad(p, r, 1.9841269841269841270e-04);
    p = fmad(p, r, 1.3888888888888888889e-03);
    p = fmad(p, r, 8.3333333333333333333e-03);
    p = fmad(p, r, 4.1666666666666666667e-02);
    p = fmad(p, r, 1.6666666666666666667e-01);
    p = fmad(p, r, 0.5);
    p = fmad(p, r, 1.0);
    p = fmad(p, r, 1.0);
    const int k = (int)kd;
    if (k >= -1021) return p * pow2i(k);
    return (p * pow2i(k + 600)) * pow2i(-600);
}

LSH_HD double cbrt_pos(double x) {
    // the range tests on the integer pipe: 0 < x < +inf goes on, anything
    // else (0, +inf, NaN, negative) comes back as it is
    const int64_t kx = (int64_t)bits_of(x);
    if (!(kx > 0 && kx < kInfBits)) return x;
    int scale = 0;
    if (kx < (int64_t)bits_of(0x1p-1000)) { x *= 0x1p300; scale = -100; }  // keep the exponent normal
    const uint64_t u = bits_of(x);
    const int e = (int)((u >> 52) & 0x7ff) - 1023;
    int q = e / 3, rem = e - 3 * q;
    if (rem < 0) { rem += 3; q -= 1; }
    // a = m 2^rem in [1, 8): x's mantissa with the exponent field set to rem
    const uint64_t ua = (u & 0x000fffffffffffffULL) | ((uint64_t)(rem + 1023) << 52);
    const double a = from_bits(ua);
    // FP32: a's leading 24 bits (truncated), a quadratic guess, three steps
    const float af = ffrom_bits(((uint32_t)(rem + 127) << 23) | (uint32_t)((ua >> 29) & 0x7fffffu));
    float zf = fmadf(fmadf(0.0115f, af, -0.1656f), af, 1.1098f);
    const float thirdf = 1.0f / 3.0f;
    for (int i = 0; i < 3; ++i) {
        const float t = (af * zf) * zf;
        zf = fmadf(zf * thirdf, fmadf(-t, zf, 1.0f), zf);
    }
    // widen exactly (zf in [1/2, 1], normal): sign 0, exponent rebased, mantissa shifted
    const uint32_t zb = fbits_of(zf);
    double z = from_bits(((uint64_t)(((zb >> 23) & 0xffu) - 127 + 1023) << 52) | ((uint64_t)(zb & 0x7fffffu) << 29));
    const double third = 1.0 / 3.0;
    for (int i = 0; i < 2; ++i) {
        const double t = (a * z) * z;
        z = fmad(z * third, fmad(-t, z, 1.0), z);
    }
    // a z^2 is in [1, 2]; times 2^(q + scale) by the exponent bits (the result
    // of a positive normal or subnormal x is normal)
    const double r = (a * z) * z;
    return from_bits(bits_of(r) + ((uint64_t)(int64_t)(q + scale) << 52));
}

LSH_HD double log_pos(double x) {
    if (!(x > 0.0)) return (x == 0.0) ? -INFINITY : (x - x) / (x - x);
    if (x == INFINITY) return x;
    int scale = 0;
    if (x < 0x1p-1000) { x *= 0x1p300; scale = -300; }
    const uint64_t u = bits_of(x);
    int e = (int)((u >> 52) & 0x7ff) - 1023;
    double m = from_bits((u & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);  // [1, 2)
    if (m > 1.4142135623730950488) { m *= 0.5; e += 1; }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double p = 1.0 / 23.0;
    p = fmad(p, s2, 1.0 / 21.0);
    p = fmad(p, s2, 1.0 / 19.0);
    p = fmad(p, s2, 1.0 / 17.0);
    p = fmad(p, s2, 1.0 / 15.0);
    p = fmad(p, s2, 1.0 / 13.0);
    p = fmad(p, s2, 1.0 / 11.0);
    p = fmad(p, s2, 1.0 / 9.0);
    p = fmad(p, s2, 1.0 / 7.0);
    p = fmad(p, s2, 1.0 / 5.0);
    p = fmad(p, s2, 1.0 / 3.0);
    p = fmad(p, s2, 1.0);
    const double lnm = 2.0 * s * p;
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    const double ed = (double)(e + scale);
    return fmad(ed, ln2_hi, fmad(ed, ln2_lo, lnm));
}

// a^b for a > 0 (Pouliquen's (Fr/beta)^chi)
LSH_HD double pow_pos(double a, double b) {
    const double y = b * log_pos(a);
    if (y <= 0.0) return exp_neg(-y);
    return 1.0 / exp_neg(y);
}

}  // namespace lshm
