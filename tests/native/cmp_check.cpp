// TEST INFRASTRUCTURE: the host side of cmp_cases.h.
#include "cmp_cases.h"

extern "C" long long cmpc_check(const double* v, long long n) {
    long long bad = 0;
    for (long long i = 0; i < n; ++i) {
        bad += cmpcheck::check_one(v[i]);
        if (v[i] != v[i]) continue;
        for (long long j = 0; j < n; ++j)
            if (v[j] == v[j]) bad += cmpcheck::check_pair(v[i], v[j]);
    }
    return bad;
}
