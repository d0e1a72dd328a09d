// TEST INFRASTRUCTURE: the integer-pipe compares, selections and sign flips
// of lsh_fpmath.h / lsh_scheme.cuh / lsh_passes.cuh against the
// floating-point expressions they restate, over every pair of a set of
// special values.  Compiled for the host (cmp_check.cpp) and the device
// (cmp_check_gpu.cu): each returns the number of mismatching pairs.
#pragma once

#include <cmath>
#include <cstdint>

#include "../../landslidehysea_gb300/csrc/lsh_passes.cuh"

namespace cmpcheck {

using lshm::bits_of;

LSH_HD bool same_bits(double a, double b) { return bits_of(a) == bits_of(b); }

// The compares as the oracle writes them.
LSH_HD double f_tmin(double a, double b) { return (b < a) ? b : a; }
LSH_HD double f_tmax(double a, double b) { return (b > a) ? b : a; }
LSH_HD double f_max0(double a) { return (a > 0.0) ? a : 0.0; }
LSH_HD int f_sgn(double x) { return (fabs(x) < lsh::kEps) ? 0 : ((x > 0) ? 1 : -1); }
LSH_HD double f_minmod(double a, double b) {
    if (a > 0.0 && b > 0.0) return (a < b) ? a : b;
    if (a < 0.0 && b < 0.0) return (a > b) ? a : b;
    return 0.0;
}

// Pairs (a, b) of non-NaN values: returns the count of mismatches.
LSH_HD long long check_pair(double a, double b) {
    long long bad = 0;
    bad += lshm::lt(a, b) != (a < b);
    bad += (lshm::okey(a) == lshm::okey(b)) != (a == b);
    bad += lshm::abs_lt(a, b) != (fabs(a) < fabs(b));
    bad += !same_bits(lsh::tmin(a, b), f_tmin(a, b));
    bad += !same_bits(lsh::tmax(a, b), f_tmax(a, b));
    bad += !same_bits(lsh::minmod(a, b), f_minmod(a, b));
    if (b > 0.0) {  // the positive-threshold forms
        bad += lshm::lt_pos(a, b) != (a < b);
        bad += lshm::gt_pos(a, b) != (a > b);
    }
    return bad;
}

// Single values, NaN included where the form keeps NaN semantics.
LSH_HD long long check_one(double x) {
    long long bad = 0;
    const bool nan = x != x;
    if (!nan) {
        bad += lshm::gt0(x) != (x > 0.0);
        bad += lshm::lt0(x) != (x < 0.0);
        bad += !same_bits(lsh::max0(x), f_max0(x));
        bad += lsh::sgn(x) != f_sgn(x);
    }
    bad += lsh::is_zero(x) != (x == 0.0);
    bad += lsh::is_bad(x) != !(fabs(x) <= 1.79769313486231570815e308);
    bad += !same_bits(lshm::neg_if(x, false), x);
    if (!nan) {
        bad += !same_bits(lshm::neg_if(x, true), -x);
        bad += !same_bits(lshm::abs_bits(x), fabs(x));
    } else {
        // IEEE negate and abs change only the sign bit, NaN included (the
        // device's -x and fabs may return another NaN payload)
        bad += (bits_of(lshm::neg_if(x, true)) ^ bits_of(x)) != 0x8000000000000000ULL;
        bad += bits_of(lshm::abs_bits(x)) != (bits_of(x) & lshm::kMag);
    }
    // exp_neg and cbrt_pos: NaN stays NaN, the ends as before
    const double e = lshm::exp_neg(x), c = lshm::cbrt_pos(x);
    if (nan) {
        bad += (e == e);
        bad += (c == c);
    } else {
        if (x < 0x1p-54) bad += !(e == 1.0);
        else if (x > 746.0) bad += !(e == 0.0);
        else bad += !(e >= 0.0 && e <= 1.0);
        if (!(x > 0.0) || x == INFINITY) bad += !same_bits(c, x);
        else bad += !(c > 0.0);
    }
    return bad;
}

}  // namespace cmpcheck
