/* Test-oracle stand-in for vecmathlib (an absent SuperDCA submodule): the
 * only function the solve path calls is the 4-lane double exp
 * (SuperDCA/include/Vector_operations.hpp:55-59).  Each lane goes through the
 * C library's exp, the same function the C oracle uses. */
#pragma once
#include <cmath>
#include <immintrin.h>

namespace vecmathlib {
template <typename T, int N> struct realvec {
    __m256d v;
};
template <typename V> struct mathfuncs {
    static V vml_exp(__m256d a)
    {
        alignas(32) double t[4];
        _mm256_store_pd(t, a);
        for (int i = 0; i < 4; ++i) t[i] = std::exp(t[i]);
        V r;
        r.v = _mm256_load_pd(t);
        return r;
    }
};
} // namespace vecmathlib
