// Prelude included before the reference's Mat.h when compiling it as the
// validation oracle (oracle/_ref).  Mat-8.3.1 relies on names it does not
// define itself: std math/min/max, a complex<T> template and the copy/zero
// helpers that older snapshots defined in Base/Base.h.  The SIMD vector types
// are switched to their unaligned variants because Mat dereferences
// (__m512d*) on pointers that are not 64-byte aligned.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdarg>
#include <cstring>
#include <utility>
#include <immintrin.h>

using std::abs;
using std::max;
using std::min;
using std::sqrt;

template <typename T>
struct complex {
    T real, imag;
    complex() : real(0), imag(0) {}
    complex(T r) : real(r), imag(0) {}
    complex(T r, T i) : real(r), imag(i) {}
    complex conj() const { return complex(real, -imag); }
};

// Element-wise copy with conversion.
template <typename T, typename S>
inline void __copy(T* dst, const S* src, int len) {
    for (int i = 0; i < len; ++i) dst[i] = (T)src[i];
}
// Zero fill (the length may arrive as size_t, long long or a floating value).
template <typename T, typename L>
inline void __set0(T* dst, L len) {
    const long long n = (long long)len;
    for (long long i = 0; i < n; ++i) dst[i] = T(0);
}

#define __m512d __m512d_u
#define __m256d __m256d_u
