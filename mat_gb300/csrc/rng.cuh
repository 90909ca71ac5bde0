// Counter-based seeded generator shared by the host and the device.
//
// Every value depends only on (seed, index), so a matrix can be filled in
// parallel on the GPU or on the host with bit-identical results.  To keep the
// two sides identical the arithmetic avoids libm and fused operations: the
// device side uses the explicitly-rounded intrinsics, the host side is
// compiled with -ffp-contract=off, sqrt and division are IEEE correctly
// rounded on both, and the logarithm below is written out from its series.
#pragma once
#include <cstdint>
#include <cmath>

#if defined(__CUDACC__)
#define MG_HD __host__ __device__ __forceinline__
#else
#define MG_HD inline
#endif

namespace mgrng {

// splitmix64 finaliser (Steele, Lea & Flood 2014) used as a counter hash.
MG_HD uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

MG_HD double rmul(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
MG_HD double radd(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
MG_HD double rdiv(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}
MG_HD double rsqrt_cr(double a) {
#if defined(__CUDA_ARCH__)
    return __dsqrt_rn(a);
#else
    return std::sqrt(a);
#endif
}

// Uniform in [0,1) from the top 53 bits (exact).
MG_HD double u01(uint64_t bits) { return (double)(bits >> 11) * 0x1.0p-53; }

// Natural logarithm of x in (0, 1]: x = m * 2^e with m in [sqrt(1/2), sqrt(2)),
// log m = 2 atanh(t), t = (m-1)/(m+1), summed as 2 t * sum_k t^(2k)/(2k+1).
MG_HD double log_series(double x) {
    int e = 0;
    double m = frexp(x, &e);  // exact
    if (m < 0.70710678118654752440) {
        m = rmul(m, 2.0);
        e -= 1;
    }
    const double f = radd(m, -1.0);  // exact (Sterbenz)
    const double t = rdiv(f, radd(2.0, f));
    const double z = rmul(t, t);
    double p = 1.0 / 23.0;
    p = radd(rmul(p, z), 1.0 / 21.0);
    p = radd(rmul(p, z), 1.0 / 19.0);
    p = radd(rmul(p, z), 1.0 / 17.0);
    p = radd(rmul(p, z), 1.0 / 15.0);
    p = radd(rmul(p, z), 1.0 / 13.0);
    p = radd(rmul(p, z), 1.0 / 11.0);
    p = radd(rmul(p, z), 1.0 / 9.0);
    p = radd(rmul(p, z), 1.0 / 7.0);
    p = radd(rmul(p, z), 1.0 / 5.0);
    p = radd(rmul(p, z), 1.0 / 3.0);
    p = radd(rmul(p, z), 1.0);
    const double lnm = rmul(rmul(2.0, t), p);
    const double de = (double)e;
    const double ln2_hi = 6.93147180369123816490e-01;  // high 32 bits of ln 2
    const double ln2_lo = 1.90821492927058770002e-10;  // ln 2 - ln2_hi
    return radd(rmul(de, ln2_hi), radd(lnm, rmul(de, ln2_lo)));
}

// e^x for x <= 0 of moderate size: x = k ln 2 + f with k the integer nearest
// x / ln 2 (|f| <= ln 2 / 2), e^f by its Taylor series to degree 17 (the
// dropped terms are below 1e-21 relative), then the exact scaling by 2^k.
MG_HD double exp_series(double x) {
    const double kd = floor(radd(rmul(x, 1.44269504088896340736), 0.5));
    const double ln2_hi = 6.93147180369123816490e-01;  // 32 significant bits: kd * ln2_hi is exact
    const double ln2_lo = 1.90821492927058770002e-10;
    const double f = radd(radd(x, -rmul(kd, ln2_hi)), -rmul(kd, ln2_lo));
    double p = rdiv(1.0, 355687428096000.0);  // 1/17!
    double fact = 355687428096000.0;
    for (int i = 17; i >= 1; --i) {
        fact = rdiv(fact, (double)i);  // (i-1)! exactly
        p = radd(rmul(p, f), rdiv(1.0, fact));
    }
    return ldexp(p, (int)kd);
}

// sigma_r = sigma_min^(r / (n-1)), r = 0..n-1, sigma_min in (0, 1]: the
// geometric singular values of the Q1 diag(sigma) Q2 test matrices, from
// the series above so that the host and the device agree bit for bit.
MG_HD double geometric_at(int r, int n, double sigma_min) {
    if (n <= 1) return 1.0;
    return exp_series(rmul(rdiv((double)r, (double)(n - 1)), log_series(sigma_min)));
}

MG_HD uint64_t stream_key(uint64_t seed, uint64_t salt) { return mix64(seed * 0xD1B54A32D192ED03ull + salt); }

MG_HD double uniform_at(uint64_t key, uint64_t idx, double lo, double hi) {
    const double u = u01(mix64(key + idx));
    return radd(lo, rmul(radd(hi, -lo), u));
}

// Standard normal by Marsaglia's polar method; attempt a of element idx
// draws the pair of counters 2*(64*idx + a) and 2*(64*idx + a) + 1.
MG_HD double normal_at(uint64_t key, uint64_t idx) {
    for (uint64_t a = 0; a < 64; ++a) {
        const uint64_t c = (idx * 64u + a) * 2u;
        const double u = radd(rmul(2.0, u01(mix64(key + c))), -1.0);
        const double v = radd(rmul(2.0, u01(mix64(key + c + 1))), -1.0);
        const double s = radd(rmul(u, u), rmul(v, v));
        if (s > 0.0 && s < 1.0) {
            const double r = rsqrt_cr(rdiv(rmul(-2.0, log_series(s)), s));
            return rmul(u, r);
        }
    }
    return 0.0;
}

// Salts separating the uniform and normal families for one seed.
constexpr uint64_t kSaltUniform = 0x55u;
constexpr uint64_t kSaltNormal = 0x4Eu;

}  // namespace mgrng
