// dual.h -- TEST INFRASTRUCTURE: forward-mode dual numbers for the oracle's
// tangent-linear model (lsh_oracle.cpp instantiated on Dual instead of
// double).  The value part of every operation is the same IEEE operation as
// the double code (same fma placement, same elementary functions), so a
// Dual run reproduces the double run's values bit for bit and carries the
// exact directional derivative of that piecewise-smooth computation:
// comparisons act on values, so every branch follows the primal run.
// Derivative conventions at the points where a function is not
// differentiable (shared with the CUDA adjoint, which makes the same choice):
//   sqrt'(0) = 0;  |x|' = -1 for x < 0 and +1 otherwise;
//   cbrt'(0) = 0;  min / max / minmod follow the operand the primal selected.
#pragma once

#include <cmath>

#include "../landslidehysea_gb300/csrc/lsh_fpmath.h"

namespace orc {

struct Dual {
    double v, d;
    Dual() : v(0.0), d(0.0) {}
    Dual(double x) : v(x), d(0.0) {}  // NOLINT: implicit on purpose (constants)
    Dual(double x, double dx) : v(x), d(dx) {}
    Dual& operator+=(const Dual& b) { v = v + b.v; d = d + b.d; return *this; }
    Dual& operator-=(const Dual& b) { v = v - b.v; d = d - b.d; return *this; }
};

inline Dual operator+(const Dual& a, const Dual& b) { return Dual(a.v + b.v, a.d + b.d); }
inline Dual operator-(const Dual& a, const Dual& b) { return Dual(a.v - b.v, a.d - b.d); }
inline Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
inline Dual operator*(const Dual& a, const Dual& b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Dual operator/(const Dual& a, const Dual& b) {
    const double q = a.v / b.v;
    return Dual(q, (a.d - q * b.d) / b.v);
}
inline bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
inline bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
inline bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
inline bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
inline bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
inline bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }

inline Dual sqrt(const Dual& a) {
    const double s = std::sqrt(a.v);
    return Dual(s, (s > 0.0) ? a.d / (2.0 * s) : 0.0);
}
inline Dual fabs(const Dual& a) { return (a.v < 0.0) ? Dual(-a.v, -a.d) : Dual(std::fabs(a.v), a.d); }
inline Dual fmad(const Dual& a, const Dual& b, const Dual& c) {
    return Dual(lshm::fmad(a.v, b.v, c.v), a.d * b.v + a.v * b.d + c.d);
}
inline Dual exp_neg(const Dual& x) {
    const double e = lshm::exp_neg(x.v);
    return Dual(e, -e * x.d);
}
inline Dual cbrt_pos(const Dual& x) {
    const double c = lshm::cbrt_pos(x.v);
    return Dual(c, (x.v > 0.0) ? (c / (3.0 * x.v)) * x.d : 0.0);
}
inline Dual pow_pos(const Dual& x, double e) {
    const double p = lshm::pow_pos(x.v, e);
    return Dual(p, (x.v > 0.0) ? ((e * p) / x.v) * x.d : 0.0);
}

inline double value(double x) { return x; }
inline double value(const Dual& x) { return x.v; }

}  // namespace orc
