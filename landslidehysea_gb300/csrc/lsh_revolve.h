// lsh_revolve.h -- binomial checkpointing (Griewank & Walther, "Algorithm
// 799: revolve", ACM TOMS 26(1), 2000) for reversing a time loop of n steps
// with s state slots.  With the minimal repetition number r such that
// beta(s, r) = C(s + r, s) >= n, the fewest forward steps any schedule
// needs is r n - beta(s + 1, r - 1); the recursive split below attains it:
// the first checkpoint after the one holding the start goes j steps ahead,
//   j in [max(beta(s, r-2), n - beta(s-1, r)), min(beta(s, r-1), n - beta(s-1, r-1))]
// (the upper end is used).  The test suite checks the schedule against a
// brute-force dynamic program on small n and s.
#pragma once

#include <cstdint>

namespace lsh {

// C(s + t, s), saturating at 2^62; 0 for t < 0
inline long long revolve_beta(int s, int t) {
    if (t < 0 || s < 0) return 0;
    long long b = 1;
    const long long cap = 1LL << 62;
    for (int k = 1; k <= t; ++k) {
        // b = C(s + k, k) = C(s + k - 1, k - 1) (s + k) / k
        const long long m = (long long)s + k;
        if (b > cap / m) return cap;
        b = (b * m) / k;
    }
    return b;
}

// minimal r with beta(s, r) >= n
inline int revolve_repetitions(long long n, int s) {
    int r = 0;
    while (revolve_beta(s, r) < n) ++r;
    return r;
}

// Steps between the start of a segment of n > 1 steps and the next
// checkpoint, with s >= 2 slots (the start's included).
inline long long revolve_split(long long n, int s) {
    const int r = revolve_repetitions(n, s);
    long long j = revolve_beta(s, r - 1);
    const long long alt = n - revolve_beta(s - 1, r - 1);
    if (alt < j) j = alt;
    if (j > n - 1) j = n - 1;
    if (j < 1) j = 1;
    return j;
}

// Fewest forward steps to reverse n steps with s slots: r n - beta(s + 1, r - 1).
inline long long revolve_cost(long long n, int s) {
    if (n <= 1) return 0;
    if (s <= 1) return n * (n - 1) / 2;
    const int r = revolve_repetitions(n, s);
    return r * n - revolve_beta(s + 1, r - 1);
}

// The schedule's operations; each returns 0 or an error status.
struct RevolveOps {
    virtual ~RevolveOps() {}
    virtual int advance(int from, int to) = 0;  // current state X_from -> X_to
    virtual int store(int slot) = 0;            // current state -> slot
    virtual int restore(int slot, int step) = 0;  // slot (holding X_step) -> current state
    virtual int reverse_step(int step) = 0;     // current state is X_step
    int cur = -1;                               // step of the current state
};

// Reverse steps [a, b): slot s0 holds X_a, slots s0+1 .. s0+free are free.
// `prestored`: the forward sweep already stored this segment's right spine
// (the checkpoints this recursion would store first, in slots s0+1, ...).
inline int revolve_reverse(RevolveOps& ops, int a, int b, int s0, int free, bool prestored) {
    auto ensure = [&](int step, int slot) -> int {
        if (ops.cur == step) return 0;
        int st = ops.restore(slot, step);
        if (!st) ops.cur = step;
        return st;
    };
    if (b - a == 1) {
        if (int st = ensure(a, s0)) return st;
        return ops.reverse_step(a);
    }
    if (free == 0) {
        for (int k = b - 1; k >= a; --k) {
            if (int st = ensure(a, s0)) return st;
            if (k > a) {
                if (int st = ops.advance(a, k)) return st;
                ops.cur = k;
            }
            if (int st = ops.reverse_step(k)) return st;
        }
        return 0;
    }
    const int m = a + (int)revolve_split(b - a, free + 1);
    if (!prestored) {
        if (int st = ensure(a, s0)) return st;
        if (int st = ops.advance(a, m)) return st;
        ops.cur = m;
        if (int st = ops.store(s0 + 1)) return st;
    }
    if (int st = revolve_reverse(ops, m, b, s0 + 1, free - 1, prestored)) return st;
    return revolve_reverse(ops, a, m, s0, free, false);
}

}  // namespace lsh
