// count.h -- TEST INFRASTRUCTURE: an operation-counting scalar for the
// oracle (lsh_oracle.cpp instantiated on Cnt): every FP64 operation of the
// scheme, as the oracle performs it, increments a per-thread counter by
// kind.  Values are computed exactly as the double code does.
#pragma once

#include <cmath>

#include "../landslidehysea_gb300/csrc/lsh_fpmath.h"
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

enum CntKind { kAdd = 0, kMul, kFma, kDiv, kSqrt, kExp, kCbrt, kPow, kCmp, kAbs, kNumCnt };

constexpr int kCntThreads = 256;
extern long long g_cnt[kCntThreads][16];

inline void bump(int k) {
#ifdef _OPENMP
    g_cnt[omp_get_thread_num() & (kCntThreads - 1)][k] += 1;
#else
    g_cnt[0][k] += 1;
#endif
}

struct Cnt {
    double v;
    Cnt() : v(0.0) {}
    Cnt(double x) : v(x) {}  // NOLINT: implicit on purpose (constants)
    Cnt& operator+=(const Cnt& b) { bump(kAdd); v = v + b.v; return *this; }
    Cnt& operator-=(const Cnt& b) { bump(kAdd); v = v - b.v; return *this; }
};

inline Cnt operator+(const Cnt& a, const Cnt& b) { bump(kAdd); return Cnt(a.v + b.v); }
inline Cnt operator-(const Cnt& a, const Cnt& b) { bump(kAdd); return Cnt(a.v - b.v); }
inline Cnt operator-(const Cnt& a) { return Cnt(-a.v); }  // a sign flip, no FP64 operation
inline Cnt operator*(const Cnt& a, const Cnt& b) { bump(kMul); return Cnt(a.v * b.v); }
inline Cnt operator/(const Cnt& a, const Cnt& b) { bump(kDiv); return Cnt(a.v / b.v); }
inline bool operator<(const Cnt& a, const Cnt& b) { bump(kCmp); return a.v < b.v; }
inline bool operator>(const Cnt& a, const Cnt& b) { bump(kCmp); return a.v > b.v; }
inline bool operator<=(const Cnt& a, const Cnt& b) { bump(kCmp); return a.v <= b.v; }
inline bool operator>=(const Cnt& a, const Cnt& b) { bump(kCmp); return a.v >= b.v; }
inline bool operator==(const Cnt& a, const Cnt& b) { bump(kCmp); return a.v == b.v; }
inline bool operator!=(const Cnt& a, const Cnt& b) { bump(kCmp); return a.v != b.v; }

inline Cnt sqrt(const Cnt& a) { bump(kSqrt); return Cnt(std::sqrt(a.v)); }
inline Cnt fabs(const Cnt& a) { bump(kAbs); return Cnt(std::fabs(a.v)); }
inline Cnt fmad(const Cnt& a, const Cnt& b, const Cnt& c) { bump(kFma); return Cnt(lshm::fmad(a.v, b.v, c.v)); }
inline Cnt exp_neg(const Cnt& x) { bump(kExp); return Cnt(lshm::exp_neg(x.v)); }
inline Cnt cbrt_pos(const Cnt& x) { bump(kCbrt); return Cnt(lshm::cbrt_pos(x.v)); }
inline Cnt pow_pos(const Cnt& x, double e) { bump(kPow); return Cnt(lshm::pow_pos(x.v, e)); }
inline double value(const Cnt& x) { return x.v; }

}  // namespace orc
