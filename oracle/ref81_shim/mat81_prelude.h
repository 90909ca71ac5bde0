// Prelude included before the Mat-8.1 headers when compiling the snapshot's
// EVD_Q tridiagonalisation as a validation oracle (oracle/_ref).  Mat-8.1's
// Mat.h pulls in a Windows-only include, so only the headers the path needs
// are included by the wrapper; this prelude provides the standard names they
// expect and switches the SIMD vector types to their unaligned variants
// (Mat dereferences (__m512d*) on pointers that are not 64-byte aligned).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cstdarg>
#include <iostream>
#include <utility>
#include <immintrin.h>

using std::abs;
using std::max;
using std::min;
using std::sqrt;
using std::cout;
using std::endl;

enum EVD_type { EVD_QR, EVD_Jacobi, EVD_CDC, EVD_ADC };

#define __m512d __m512d_u
#define __m256d __m256d_u
#define __m512 __m512_u
#define __m256 __m256_u
