// Mixed-precision LU solve with FP64 iterative refinement.
//
// There is no mixed precision in Mat; this is the fast form of Mat's
// Solve_direct (Mat-8.3.1/LU/__Solve_direct.h:146-220) for the n = 16384,
// 4-RHS benchmark configuration: factor in fp32 (fp32 panels, split-BF16
// tensor-core trailing updates with fp32 accumulation), then refine in fp64:
//     r = b - A x                 (fp64 A, fp64 FMA)
//     eta = ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf)   per column
//     d = U^{-1} L^{-1} P (r/s)   (fp32, s = ||r||_inf per column)
//     x = x + s d                 (fp64)
// until every column's normwise backward error eta <= tol.  If refinement
// stalls (eta not halving twice in a row, or max_iter reached) the solve
// falls back to the plain FP64 GPU path (mg_dgesv) and reports it.
//
// The triangular solves use precomputed inverses of the 128x128 diagonal
// blocks, so each block step is one kernel with no intra-kernel dependency:
// every CTA applies the block inverse to the (already final) block of the
// right-hand side and updates its share of the rows below.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <optional>
#include <type_traits>
#include <vector>

#include "grid_sync.cuh"
#include "mg_internal.cuh"

namespace {

constexpr int IR_BLOCK = 128;      // fp32 LU block / diagonal-inverse block
constexpr int MAX_RHS = 8;
constexpr int RES_ROWS = 256;      // rows per residual CTA
constexpr int RES_KCHUNK = 2048;   // columns per residual CTA (k split)

__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v);

// The fp32 copy of A and the row sums of |A| in one pass over A (one read
// of the FP64 matrix): S(i,k) = fp32(A(i,k)), partial[kc][i] = sum over the
// column chunk kc (D2S_KCHUNK columns) of |A(i,k)|, *amax = max |A(i,k)|.
// Each thread takes four consecutive rows (two 16-byte loads and one
// 16-byte store per column; a CTA covers 1024 rows, 8 KB of a column), eight
// columns' loads in flight.  Nothing runs on the FP64 pipe: the conversion
// is d2f_rn, the maximum and the chunk sums use the fp32 values (relative
// error ~1e-5 at most in ||A||_inf, which only scales the backward error;
// max |A| feeds the pivot-growth report).  Needs lda and n multiples of 4
// (checked by the caller, else d2s_absrow_scalar_kernel).
constexpr int D2S_KCHUNK = 256;
constexpr int D2S_ROWS = 1024;  // rows per CTA (256 threads x 4)

// double -> float, round to nearest even, with 32-bit integer operations
// for values in the normal float range (on GB300 the conversion instruction,
// and 64-bit integer arithmetic, run on the FP64 pipe, which limited this
// pass): the exponent is rebased by 1023 - 127, the top 23 mantissa bits
// are kept, and the 29 dropped ones round up when above half an ulp or at
// half with an odd kept part (ties to even); a carry out of the mantissa
// moves into the exponent, up to +inf.  Zeros, subnormal results,
// infinities and NaNs take the hardware conversion.
__device__ __forceinline__ float d2f_rn(double d) {
    const unsigned int hi = (unsigned int)__double2hiint(d), lo = (unsigned int)__double2loint(d);
    const unsigned int e = (hi >> 20) & 0x7ffu;
    if (e - 897u <= 1150u - 897u) {
        unsigned int f = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
        const unsigned int rnd = (lo >> 28) & 1u, sticky = (lo & 0x0fffffffu) != 0u;
        f += rnd & (sticky | (f & 1u));
        return __uint_as_float(f | (hi & 0x80000000u));
    }
    return (float)d;
}

// The biased exponent field of a double (0 for zeros and subnormals, 0x7ff
// for infinities and NaNs).
__device__ __forceinline__ int exp_field(double d) { return (__double2hiint(d) >> 20) & 0x7ff; }

// Also: rexp[i] = the largest exponent field of row i (atomicMax over the
// column chunks; rexp zeroed by the caller), and *nonfinite = 1 if A holds
// an infinity or a NaN (the scale of the integer residual below).
__global__ void __launch_bounds__(256) d2s_absrow_kernel(const double* __restrict__ A, int lda, int n,
                                                         float* __restrict__ S, int lds, double* __restrict__ partial,
                                                         double* __restrict__ amax, int* __restrict__ rexp,
                                                         int* __restrict__ nonfinite) {
    const int i0 = blockIdx.x * D2S_ROWS + 4 * threadIdx.x;
    const int k0 = blockIdx.y * D2S_KCHUNK, k1 = min(n, k0 + D2S_KCHUNK);
    float s[4] = {0.f, 0.f, 0.f, 0.f};
    int em[4] = {0, 0, 0, 0};
    float mx = 0.f;
    if (i0 < n) {  // n is a multiple of 4 here
        int k = k0;
        for (; k + 8 <= k1; k += 8) {
            double2 a[8][2];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const double2* p = reinterpret_cast<const double2*>(A + i0 + (size_t)(k + u) * lda);
                a[u][0] = p[0];
                a[u][1] = p[1];
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const float4 f = make_float4(d2f_rn(a[u][0].x), d2f_rn(a[u][0].y), d2f_rn(a[u][1].x), d2f_rn(a[u][1].y));
                *reinterpret_cast<float4*>(S + i0 + (size_t)(k + u) * lds) = f;
                s[0] += fabsf(f.x);
                s[1] += fabsf(f.y);
                s[2] += fabsf(f.z);
                s[3] += fabsf(f.w);
                mx = fmaxf(mx, fmaxf(fmaxf(fabsf(f.x), fabsf(f.y)), fmaxf(fabsf(f.z), fabsf(f.w))));
                em[0] = max(em[0], exp_field(a[u][0].x));
                em[1] = max(em[1], exp_field(a[u][0].y));
                em[2] = max(em[2], exp_field(a[u][1].x));
                em[3] = max(em[3], exp_field(a[u][1].y));
            }
        }
        for (; k < k1; ++k)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const double d = A[i0 + r + (size_t)k * lda];
                const float f = d2f_rn(d);
                S[i0 + r + (size_t)k * lds] = f;
                s[r] += fabsf(f);
                mx = fmaxf(mx, fabsf(f));
                em[r] = max(em[r], exp_field(d));
            }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            partial[(size_t)blockIdx.y * n + i0 + r] = (double)s[r];
            atomicMax(rexp + i0 + r, em[r]);
            if (em[r] == 0x7ff) atomicExch(nonfinite, 1);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, off));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(amax, (double)mx);
}

// The same for any lda / lds (one row per thread, scalar accesses).
__global__ void d2s_absrow_scalar_kernel(const double* __restrict__ A, int lda, int n, float* __restrict__ S, int lds,
                                         double* __restrict__ partial, double* __restrict__ amax,
                                         int* __restrict__ rexp, int* __restrict__ nonfinite) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int k0 = blockIdx.y * D2S_KCHUNK, k1 = min(n, k0 + D2S_KCHUNK);
    float s = 0.f, mx = 0.f;
    int em = 0;
    if (i < n) {
        for (int k = k0; k < k1; ++k) {
            const double d = A[i + (size_t)k * lda];
            const float f = d2f_rn(d);
            S[i + (size_t)k * lds] = f;
            s += fabsf(f);
            mx = fmaxf(mx, fabsf(f));
            em = max(em, exp_field(d));
        }
        partial[(size_t)blockIdx.y * n + i] = (double)s;
        atomicMax(rexp + i, em);
        if (em == 0x7ff) atomicExch(nonfinite, 1);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, off));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(amax, (double)mx);
}

// *umax = max |U(i,j)| over the upper triangle of the packed fp32 LU (one CTA
// per column), reduced in fp64
__global__ void absmax_upper_kernel(const float* __restrict__ LU, int n, double* __restrict__ umax) {
    const int c = blockIdx.x;
    float mx = 0.f;
    for (int r = threadIdx.x; r <= c; r += blockDim.x) mx = fmaxf(mx, fabsf(LU[r + (size_t)c * n]));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, off));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(umax, (double)mx);
}

__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
    // for non-negative doubles the bit patterns order like the values (NaN: skipped)
    if (!(v >= 0.0)) return;
    atomicMax((unsigned long long*)addr, (unsigned long long)__double_as_longlong(v));
}

__global__ void absrow_reduce_kernel(const double* __restrict__ partial, int nchunks, int n, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int c = 0; c < nchunks; ++c) s += partial[(size_t)c * n + i];
    atomic_max_nonneg(out, s);
}

// partial[kc][j][i] = sum_{k in chunk} A(i,k) X(k,j)   (fp64 FMA)
template <int NR>
__global__ void __launch_bounds__(RES_ROWS) residual_partial_kernel(const double* __restrict__ A, int lda, int n,
                                                                    const double* __restrict__ X, int ldx,
                                                                    double* __restrict__ partial) {
    constexpr int nrhs = NR;
    __shared__ double xs[MAX_RHS][256];
    const int i = blockIdx.x * RES_ROWS + threadIdx.x;
    const int k0 = blockIdx.y * RES_KCHUNK, k1 = min(n, k0 + RES_KCHUNK);
    double acc[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) acc[j] = 0.0;
    for (int kb = k0; kb < k1; kb += 256) {
        const int kn = min(256, k1 - kb);
        __syncthreads();
        for (int q = threadIdx.x; q < kn * nrhs; q += blockDim.x) xs[q / kn][q % kn] = X[kb + q % kn + (size_t)(q / kn) * ldx];
        __syncthreads();
        if (i < n) {
            const double* ap = A + i + (size_t)kb * lda;
#pragma unroll 8
            for (int k = 0; k < kn; ++k) {
                const double a = ap[(size_t)k * lda];
#pragma unroll
                for (int j = 0; j < NR; ++j) acc[j] = fma(a, xs[j][k], acc[j]);
            }
        }
    }
    if (i < n)
#pragma unroll
        for (int j = 0; j < NR; ++j) partial[((size_t)blockIdx.y * nrhs + j) * n + i] = acc[j];
}

// r = b - sum_c partial[c]; rnorm[j] = max |r(:,j)|, xnorm[j] = max |x(:,j)|
__global__ void residual_reduce_kernel(const double* __restrict__ partial, int nchunks, int n, int nrhs,
                                       const double* __restrict__ B, int ldb, const double* __restrict__ X, int ldx,
                                       double* __restrict__ R, int ldr, double* __restrict__ norms) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int j = 0; j < nrhs; ++j) {
        double s = 0.0;
        for (int c = 0; c < nchunks; ++c) s += partial[((size_t)c * nrhs + j) * n + i];
        const double r = B[i + (size_t)j * ldb] - s;
        R[i + (size_t)j * ldr] = r;
        atomic_max_nonneg(norms + j, fabs(r));
        atomic_max_nonneg(norms + MAX_RHS + j, fabs(X[i + (size_t)j * ldx]));
    }
}

// ---------------------------------------------------------------- integer residual
// A X (and r = b - A X) in exact fixed-point integer arithmetic on the
// integer multiply-add pipe, which on this part issues about 62 lane
// operations per clock per SM against 2 for FP64 FMA (measured: the FP64
// kernel above is bound by that pipe).
//
// Every A(i,k) becomes a 63-bit integer in units of 2^(ea_i - 1084), ea_i the
// largest exponent field of row i (the row's largest element maps below
// 2^62; the others are rounded to the unit, half away from zero), and every
// X(k,j) likewise with ex_j, the largest exponent field of column j.  Each
// integer is split into three 21-bit digits (magnitude digits with the
// value's sign), so that a digit product is below 2^42 and up to 2^20 of
// them sum exactly in an int64.  The products are kept by weight class
// c = p + q of their digits (2^(21c)): classes 4 .. 1 (8 products per
// element and right-hand side); class 0 (the two lowest digits, below
// 2^-82 of the leading products) is dropped.  Summed exactly over k,
//   (A X)(i,j) = 2^(ea_i + ex_j - 2147) (acc4 2^63 + acc3 2^42 + acc2 2^21 + acc1),
// combined once per entry in 128-bit integers and rounded to double.  The
// error is the rounding of the entries to their units (2^-63 of the row's
// and the column's largest element), not a rounding per operation.
constexpr int RI_CLASSES = 5;

// The integer of d in units of 2^(e - 1084), e >= d's exponent field: its
// magnitude (ah:al, below 2^62) and sign mask sm (0 or -1).
__device__ __forceinline__ void fx_int(double d, int e, unsigned& ah, unsigned& al, int& sm) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const int eb = (int)((hi >> 20) & 0x7ffu);
    const unsigned mh = (hi & 0xfffffu) | (eb ? 0x100000u : 0u);  // the 53-bit significand: mh:lo
    const int t = 9 + (eb ? eb : 1) - e;                          // its shift to the unit, <= 9
    if (t >= 0) {
        ah = __funnelshift_l(lo, mh, t);
        al = lo << t;
    } else if (t > -54) {  // right shift by s, adding half a unit first
        const int s = -t;
        const unsigned addl = s <= 32 ? 1u << (s - 1) : 0u, addh = s > 32 ? 1u << (s - 33) : 0u;
        unsigned rl, rh;
        asm("add.cc.u32 %0, %2, %3;\n\taddc.u32 %1, %4, %5;" : "=r"(rl), "=r"(rh) : "r"(lo), "r"(addl), "r"(mh),
            "r"(addh));
        if (s < 32) {
            al = __funnelshift_r(rl, rh, s);
            ah = rh >> s;
        } else {
            al = rh >> (s - 32);
            ah = 0u;
        }
    } else {
        ah = al = 0u;
    }
    sm = (int)hi >> 31;
}

// The three 21-bit digits (magnitude digits carrying the sign) of the
// magnitude ah:al (below 2^62) with sign mask sm.  32-bit operations only:
// on this part 64-bit integer shifts issue to the FP64 pipe.
__device__ __forceinline__ void mag_digits(unsigned ah, unsigned al, int sm, int& d0, int& d1, int& d2) {
    const int u0 = (int)(al & 0x1fffffu), u1 = (int)(__funnelshift_r(al, ah, 21) & 0x1fffffu), u2 = (int)(ah >> 10);
    d0 = (u0 ^ sm) - sm;
    d1 = (u1 ^ sm) - sm;
    d2 = (u2 ^ sm) - sm;
}

// The digits of d in units of 2^(e - 1084).
__device__ __forceinline__ void fx_digits(double d, int e, int& d0, int& d1, int& d2) {
    unsigned ah, al;
    int sm;
    fx_int(d, e, ah, al, sm);
    mag_digits(ah, al, sm, d0, d1, d2);
}

// The stored form of A's integers: sign and magnitude (the magnitude in bits
// 0..61, the sign in bit 63), packed and unpacked by register halves.
__device__ __forceinline__ long long fx_pack(unsigned ah, unsigned al, int sm) {
    return (long long)(((unsigned long long)(ah | ((unsigned)sm & 0x80000000u)) << 32) | al);
}

// cexp[j] = the largest exponent field of column j of V (n x nrhs, ld ldv;
// cexp zeroed by the caller); *nonfinite = 1 if V holds an infinity or NaN.
__global__ void colexp_kernel(const double* __restrict__ V, int ldv, int n, int nrhs, int* __restrict__ cexp,
                              int* __restrict__ nonfinite) {
    const int j = blockIdx.y;
    int em = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        em = max(em, exp_field(V[i + (size_t)j * ldv]));
    em = __reduce_max_sync(0xffffffffu, em);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(cexp + j, em);
        if (em == 0x7ff) atomicExch(nonfinite, 1);
    }
}

// rexp[i] = the largest exponent field of row i of A (n x n, ld lda; rexp
// zeroed by the caller), a thread per row over a chunk of 256 columns;
// *nonfinite = 1 if A holds an infinity or NaN.
__global__ void rowexp_kernel(const double* __restrict__ A, int lda, int n, int* __restrict__ rexp,
                              int* __restrict__ nonfinite) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k0 = blockIdx.y * 256, k1 = min(n, k0 + 256);
    int em = 0;
    for (int k = k0; k < k1; ++k) em = max(em, exp_field(A[i + (size_t)k * lda]));
    atomicMax(rexp + i, em);
    if (em == 0x7ff) atomicExch(nonfinite, 1);
}

// xdig[(k * nrhs + j) * 4 + p] = digit p of V(k,j) in units of 2^(cexp[j] -
// 1084) (p < 3; the fourth int pads the entry to 16 bytes).
__global__ void xdigits_kernel(const double* __restrict__ V, int ldv, int n, int nrhs, const int* __restrict__ cexp,
                               int* __restrict__ xdig) {
    const int total = n * nrhs;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int k = e / nrhs, j = e - k * nrhs;
        int d0, d1, d2;
        fx_digits(V[k + (size_t)j * ldv], cexp[j], d0, d1, d2);
        reinterpret_cast<int4*>(xdig)[e] = make_int4(d0, d1, d2, 0);
    }
}

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem));
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

constexpr int RI_ROWS = 256;  // rows per CTA (a thread per row)
constexpr int RI_KT = 8;      // columns per pipeline stage
constexpr int RI_NST = 4;     // stages
template <int NR>
constexpr size_t ri_stage_bytes() {
    return (size_t)RI_KT * RI_ROWS * 8 + (size_t)RI_KT * NR * 16;
}

// The two 31-bit digits (carrying the sign) of the magnitude ah:al (below
// 2^62) with sign mask sm.
__device__ __forceinline__ void mag_digits31(unsigned ah, unsigned al, int sm, int& a1, int& a0) {
    const int u0 = (int)(al & 0x7fffffffu), u1 = (int)((ah << 1) | (al >> 31));
    a0 = (u0 ^ sm) - sm;
    a1 = (u1 ^ sm) - sm;
}

// acc += a * b, 32 x 32 -> 64-bit signed (one wide integer multiply-add;
// written in C++ so that the compiler schedules it: as inline PTX the
// accumulators spilled).
__device__ __forceinline__ void imad_wide(long long& acc, int a, int b) { acc += (long long)a * b; }

// part[((kc * RI_CLASSES + c) * n + i) * NR + j] = class c of sum over the
// column chunk kc (kchunk <= 1024 columns, a multiple of RI_KT) of
// A(i,k) V(k,j), exact int64.  A's integer in two 31-bit digits a1 a0, V's
// in three 21-bit digits x2 x1 x0; the five kept products each have a
// weight of their own (a1 x2: 2^73, a1 x1: 2^52, a0 x2: 2^42, a1 x0: 2^31,
// a0 x1: 2^21; a0 x0, below 2^-72 of the leading one, is dropped), so every
// accumulator takes one product per entry, and a product below 2^52 lets
// 1024 of them sum exactly.  A thread per row with every right-hand side
// (the row's digits made once; a thread per right-hand side or pair of them
// repeated that and ran 1.3-1.8x slower).  SRC: A from its FP64 entries (0),
// the same and its integers stored to Ai (1, for the residuals to come), or
// from those integers (2: no exponent arithmetic per entry, ld ldi).  Tiles
// of RI_KT columns x RI_ROWS rows of A (8-byte cp.async, a thread per row)
// and the matching digits of V (xdig) stream through RI_NST shared-memory
// stages, so that the loads in flight are bounded by shared memory, not
// registers.
template <int NR, int SRC>
__global__ void __launch_bounds__(RI_ROWS, NR <= 4 ? 3 : 1)
    residual_int_kernel(const double* __restrict__ A, int lda, long long* __restrict__ Ai, int ldi, int n,
                        const int* __restrict__ xdig, int kchunk, const int* __restrict__ rexp,
                        long long* __restrict__ part) {
    extern __shared__ __align__(16) unsigned char ri_smem[];
    constexpr size_t SB = ri_stage_bytes<NR>();
    constexpr int XCH = RI_KT * NR;  // 16-byte digit entries of a stage
    const int tid = threadIdx.x, i = blockIdx.x * RI_ROWS + tid;
    const int k0 = blockIdx.y * kchunk, k1 = min(n, k0 + kchunk);
    const int nt = (k1 - k0 + RI_KT - 1) / RI_KT;
    const bool row_ok = i < n;
    const int ea = row_ok ? rexp[i] : 0;
    const char* const src = SRC == 2 ? (const char*)(Ai + i) : (const char*)(A + i);
    const size_t ldb = (SRC == 2 ? (size_t)ldi : (size_t)lda) * 8;  // bytes between columns
    auto issue = [&](int t) {  // tile t of the chunk into stage t % RI_NST
        if (t < nt) {
            unsigned char* const st = ri_smem + (size_t)(t % RI_NST) * SB;
            const int kt = k0 + t * RI_KT, kn = min(RI_KT, k1 - kt);
            if (row_ok)
                for (int k = 0; k < kn; ++k) cp_async8(st + ((size_t)k * RI_ROWS + tid) * 8, src + (size_t)(kt + k) * ldb);
            if (tid < XCH && tid < kn * NR)
                cp_async16(st + (size_t)RI_KT * RI_ROWS * 8 + (size_t)tid * 16, xdig + ((size_t)kt * NR + tid) * 4);
        }
        cp_async_commit();
    };
    long long acc[NR][RI_CLASSES];
#pragma unroll
    for (int j = 0; j < NR; ++j)
#pragma unroll
        for (int c = 0; c < RI_CLASSES; ++c) acc[j][c] = 0;
#pragma unroll
    for (int t = 0; t < RI_NST - 1; ++t) issue(t);
    for (int t = 0; t < nt; ++t) {
        cp_async_wait<RI_NST - 2>();
        __syncthreads();  // tile t in every thread's view; stage (t - 1) % RI_NST free
        issue(t + RI_NST - 1);
        const unsigned char* const st = ri_smem + (size_t)(t % RI_NST) * SB;
        const int4* const xs = reinterpret_cast<const int4*>(st + (size_t)RI_KT * RI_ROWS * 8);
        const int kt = k0 + t * RI_KT, kn = min(RI_KT, k1 - kt);
        if (row_ok) {
            auto mac = [&](int k) {
                const unsigned long long raw = reinterpret_cast<const unsigned long long*>(st)[k * RI_ROWS + tid];
                unsigned ah, al;
                int sm;
                if constexpr (SRC == 2) {
                    al = (unsigned)raw;
                    const unsigned hw = (unsigned)(raw >> 32);
                    ah = hw & 0x7fffffffu;
                    sm = (int)hw >> 31;
                } else {
                    fx_int(__longlong_as_double((long long)raw), ea, ah, al, sm);
                    if constexpr (SRC == 1) __stcs(Ai + i + (size_t)(kt + k) * ldi, fx_pack(ah, al, sm));
                }
                int a1, a0;
                mag_digits31(ah, al, sm, a1, a0);
#pragma unroll
                for (int j = 0; j < NR; ++j) {
                    const int4 x = xs[k * NR + j];  // x.x = x0, x.y = x1, x.z = x2
                    imad_wide(acc[j][4], a1, x.z);
                    imad_wide(acc[j][3], a1, x.y);
                    imad_wide(acc[j][2], a0, x.z);
                    imad_wide(acc[j][1], a1, x.x);
                    imad_wide(acc[j][0], a0, x.y);
                }
            };
            if (kn == RI_KT) {
#pragma unroll
                for (int k = 0; k < RI_KT; ++k) mac(k);
            } else {
                for (int k = 0; k < kn; ++k) mac(k);
            }
        }
    }
    cp_async_wait<0>();
    if (row_ok)
#pragma unroll
        for (int c = 0; c < RI_CLASSES; ++c)
#pragma unroll
            for (int j = 0; j < NR; ++j)
                part[(((size_t)blockIdx.y * RI_CLASSES + c) * n + i) * NR + j] = acc[j][c];
}

// Launch residual_int_kernel<nrhs, src> (its shared memory set once per variant).
template <int NR, int S>
cudaError_t launch_resint_t(dim3 g, cudaStream_t st, const double* A, int lda, long long* Ai, int ldi, int n,
                            const int* xdig, int kchunk, const int* rexp, long long* part) {
    static bool attr_set = false;  // benign race: every thread sets the same value
    const size_t smem = RI_NST * ri_stage_bytes<NR>();
    if (!attr_set) {
        const cudaError_t e =
            cudaFuncSetAttribute(residual_int_kernel<NR, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    residual_int_kernel<NR, S><<<g, RI_ROWS, smem, st>>>(A, lda, Ai, ldi, n, xdig, kchunk, rexp, part);
    return cudaGetLastError();
}
cudaError_t launch_resint(int src, int nrhs, dim3 g, cudaStream_t st, const double* A, int lda, long long* Ai, int ldi,
                          int n, const int* xdig, int kchunk, const int* rexp, long long* part) {
#define MG_RI(NRV, S) launch_resint_t<NRV, S>(g, st, A, lda, Ai, ldi, n, xdig, kchunk, rexp, part)
#define MG_RI3(NRV) \
    case NRV: return src == 2 ? MG_RI(NRV, 2) : src == 1 ? MG_RI(NRV, 1) : MG_RI(NRV, 0);
    switch (nrhs) {
        MG_RI3(1) MG_RI3(2) MG_RI3(3) MG_RI3(4) MG_RI3(5) MG_RI3(6) MG_RI3(7)
        default: return src == 2 ? MG_RI(8, 2) : src == 1 ? MG_RI(8, 1) : MG_RI(8, 0);
    }
#undef MG_RI3
#undef MG_RI
}

// (A V)(i,j) from the int partials of residual_int_kernel (nrhs = its NR):
// the classes summed over the chunks in 128-bit integers, combined as
// T = s4 2^52 + s3 2^31 + s2 2^21 + s1 2^10 + s0 (the weights over 2^21),
// rounded to double, scaled by 2^21 and the two units.
__device__ __forceinline__ double int_av(const long long* __restrict__ part, int nchunks, int n, int nrhs, int i, int j,
                                         int ea, int ex) {
    __int128 a[RI_CLASSES] = {0, 0, 0, 0, 0};
    for (int c = 0; c < nchunks; ++c)
#pragma unroll
        for (int q = 0; q < RI_CLASSES; ++q) a[q] += part[(((size_t)c * RI_CLASSES + q) * n + i) * nrhs + j];
    const __int128 t = (a[4] << 52) + (a[3] << 31) + (a[2] << 21) + (a[1] << 10) + a[0];
    const bool neg = t < 0;
    const unsigned __int128 u = neg ? (unsigned __int128)(-t) : (unsigned __int128)t;
    const double v = fma((double)(unsigned long long)(u >> 64), 0x1p64, (double)(unsigned long long)u);
    return ldexp(neg ? -v : v, ea + ex - 2147);
}

// r = b - A x from the int partials; rnorm / xnorm as residual_reduce_kernel.
// A non-finite x (flag set by colexp_kernel) gives r = NaN.
__global__ void residual_int_reduce_kernel(const long long* __restrict__ part, int nchunks, int n, int nrhs,
                                           const int* __restrict__ rexp, const int* __restrict__ cexp,
                                           const int* __restrict__ xnonfinite, const double* __restrict__ B, int ldb,
                                           const double* __restrict__ X, int ldx, double* __restrict__ R, int ldr,
                                           double* __restrict__ norms) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool bad = *xnonfinite != 0;
    for (int j = 0; j < nrhs; ++j) {
        const double v = int_av(part, nchunks, n, nrhs, i, j, rexp[i], cexp[j]);
        const double r = bad ? __longlong_as_double(0x7ff8000000000000LL) : B[i + (size_t)j * ldb] - v;
        R[i + (size_t)j * ldr] = r;
        atomic_max_nonneg(norms + j, fabs(r));
        atomic_max_nonneg(norms + MAX_RHS + j, fabs(X[i + (size_t)j * ldx]));
    }
}

// Y = A V from the int partials (GMRES-IR's products).
__global__ void matvec_int_reduce_kernel(const long long* __restrict__ part, int nchunks, int n, int nrhs,
                                         const int* __restrict__ rexp, const int* __restrict__ cexp,
                                         const int* __restrict__ vnonfinite, double* __restrict__ Y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool bad = *vnonfinite != 0;
    for (int j = 0; j < nrhs; ++j)
        Y[i + (size_t)j * n] =
            bad ? __longlong_as_double(0x7ff8000000000000LL) : int_av(part, nchunks, n, nrhs, i, j, rexp[i], cexp[j]);
}

// Column chunking of the integer residual: the row blocks x column chunks
// fill whole waves of two resident CTAs per SM (chunks a multiple of 64).
// Bytes of the digit array of V (n x nrhs entries of 16 bytes, padded).
size_t xdig_bytes(int n, int nrhs) { return ((size_t)n * nrhs + (size_t)RI_KT * MAX_RHS) * 16; }

// Column chunks of the integer residual: at most 1024 columns (the exact
// int64 bound), a multiple of 64, whole waves of three CTAs per SM where the
// chunk count allows.
int resint_kchunk(int n, int num_sms) {
    const int rb = (n + RI_ROWS - 1) / RI_ROWS;
    const int slots = 3 * num_sms;
    int kch = std::max(1, (n + 1023) / 1024);
    const int waves = (rb * kch + slots - 1) / slots;
    kch = std::max(kch, (waves * slots) / rb);
    const int chunk = (n + kch - 1) / kch;
    return std::min(1024, (chunk + 63) / 64 * 64);
}

// y[i][j] = float(r[pos[i]][j] / s_j)
__global__ void prep_rhs_kernel(int n, int nrhs, const int* __restrict__ pos, const double* __restrict__ R,
                                const double* __restrict__ scale, float* __restrict__ Y) {
    const size_t total = (size_t)n * nrhs;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        const double s = scale[j];
        Y[e] = (float)(s > 0.0 ? R[pos[i] + (size_t)j * n] / s : 0.0);
    }
}

__global__ void update_x_kernel(int n, int nrhs, const float* __restrict__ D, const double* __restrict__ scale,
                                double* __restrict__ X, int ldx) {
    const size_t total = (size_t)n * nrhs;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        X[i + (size_t)j * ldx] += scale[j] * (double)D[e];
    }
}

// ---------------------------------------------------------------- GMRES-IR
// GMRES for the correction equation A d = r, left-preconditioned by the fp32
// factors (M = P^T L U applied in FP64), one Krylov basis per right-hand
// side, all columns advancing in lockstep.  Basis vectors are stored
// [k][j][i] (vector k of column j, row i), so vector k of every column is an
// n x nrhs block with leading dimension n, the residual kernel's X layout.
constexpr int GM_RESTART = 40;   // Krylov vectors per correction (no restart)
constexpr int GM_CTAS = 64;      // CTAs of the Gram-Schmidt dot products
constexpr int GM_THREADS = 256;

// Y(:, j) = sum over the k chunks of partial (A V in FP64, fixed order)
__global__ void matvec_reduce_kernel(const double* __restrict__ partial, int nchunks, int n, int nrhs,
                                     double* __restrict__ Y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int j = 0; j < nrhs; ++j) {
        double s = 0.0;
        for (int c = 0; c < nchunks; ++c) s += partial[((size_t)c * nrhs + j) * n + i];
        Y[i + (size_t)j * n] = s;
    }
}

// partial[cta][q], q = k * nrhs + j < nv * nrhs: this CTA's share of
// V_k(:, j) . W(:, j), summed in a fixed order (each thread its strided rows,
// then a butterfly over the warp, then the warps in order): deterministic.
__global__ void __launch_bounds__(GM_THREADS) gs_dots_kernel(int n, int nv, int nrhs, const double* __restrict__ V,
                                                             const double* __restrict__ W,
                                                             double* __restrict__ partial, int pstride) {
    __shared__ double ws[GM_THREADS / 32];
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    const int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int q = 0; q < nv * nrhs; ++q) {
        const int k = q / nrhs, j = q - k * nrhs;
        const double* v = V + ((size_t)k * nrhs + j) * n;
        const double* x = W + (size_t)j * n;
        double acc = 0.0;
        for (int i = lo + threadIdx.x; i < hi; i += GM_THREADS) acc = fma(v[i], x[i], acc);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
        if (lane == 0) ws[warp] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int u = 0; u < GM_THREADS / 32; ++u) t += ws[u];
            partial[(size_t)blockIdx.x * pstride + q] = t;
        }
        __syncthreads();
    }
}

// W(:, j) -= sum_{k < nv} c[k][j] V_k(:, j)
__global__ void gs_update_kernel(int n, int nv, int nrhs, const double* __restrict__ V, const double* __restrict__ c,
                                 double* __restrict__ W) {
    const size_t total = (size_t)n * nrhs;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        double acc = W[e];
        for (int k = 0; k < nv; ++k) acc = fma(-c[k * nrhs + j], V[((size_t)k * nrhs + j) * n + i], acc);
        W[e] = acc;
    }
}

// Vout(:, j) = W(:, j) * inv[j]
__global__ void gs_scale_kernel(int n, int nrhs, const double* __restrict__ W, const double* __restrict__ inv,
                                double* __restrict__ Vout) {
    const size_t total = (size_t)n * nrhs;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        Vout[e] = W[e] * inv[e / n];
}

// X(:, j) += sum_{k < nv} y[k][j] V_k(:, j)
__global__ void gm_update_x_kernel(int n, int nv, int nrhs, const double* __restrict__ V, const double* __restrict__ y,
                                   double* __restrict__ X, int ldx) {
    const size_t total = (size_t)n * nrhs;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        double acc = X[i + (size_t)j * ldx];
        for (int k = 0; k < nv; ++k) acc = fma(y[k * nrhs + j], V[((size_t)k * nrhs + j) * n + i], acc);
        X[i + (size_t)j * ldx] = acc;
    }
}

// X(:, j) += D(:, j)  (FP64 correction of the QR-form refinement)
__global__ void add_correction_kernel(int n, int nrhs, const double* __restrict__ D, double* __restrict__ X, int ldx) {
    const size_t total = (size_t)n * nrhs;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        X[(e % n) + (e / n) * (size_t)ldx] += D[e];
}

// Inverse of each diagonal block (unit lower when LOWER, else upper) of the
// packed fp32 LU; one CTA per block, one thread per column of the inverse.
template <bool LOWER>
__global__ void inv_diag_blocks_kernel(const float* __restrict__ LU, int lda, int n, float* __restrict__ inv) {
    extern __shared__ float sb[];  // [bs][bs] column-major block, then [bs][bs] inverse
    const int b0 = blockIdx.x * IR_BLOCK;
    const int bs = min(IR_BLOCK, n - b0);
    float* blk = sb;
    float* z = sb + IR_BLOCK * IR_BLOCK;
    for (int e = threadIdx.x; e < bs * bs; e += blockDim.x) {
        const int r = e % bs, c = e / bs;
        blk[r + c * IR_BLOCK] = LU[(b0 + r) + (size_t)(b0 + c) * lda];
    }
    __syncthreads();
    const int c = threadIdx.x;
    if (c < bs) {
        float* zc = z + c * IR_BLOCK;
        // each dot in four partial sums (independent shared-memory loads in
        // flight), added in a fixed order
        auto dot = [&](int i, int ka, int kb) {  // sum over k in [ka, kb) of blk(i, k) zc[k]
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
            int k = ka;
            for (; k + 3 < kb; k += 4) {
                s0 = fmaf(blk[i + k * IR_BLOCK], zc[k], s0);
                s1 = fmaf(blk[i + (k + 1) * IR_BLOCK], zc[k + 1], s1);
                s2 = fmaf(blk[i + (k + 2) * IR_BLOCK], zc[k + 2], s2);
                s3 = fmaf(blk[i + (k + 3) * IR_BLOCK], zc[k + 3], s3);
            }
            for (; k < kb; ++k) s0 = fmaf(blk[i + k * IR_BLOCK], zc[k], s0);
            return (s0 + s1) + (s2 + s3);
        };
        if (LOWER) {
            for (int i = 0; i < bs; ++i) zc[i] = 0.f;
            zc[c] = 1.f;
            for (int i = c + 1; i < bs; ++i) zc[i] = -dot(i, c, i);
        } else {
            for (int i = 0; i < bs; ++i) zc[i] = 0.f;
            zc[c] = 1.f / blk[c + c * IR_BLOCK];
            for (int i = c - 1; i >= 0; --i) zc[i] = -dot(i, i + 1, c + 1) / blk[i + i * IR_BLOCK];
        }
    }
    __syncthreads();
    float* out = inv + (size_t)blockIdx.x * IR_BLOCK * IR_BLOCK;
    for (int e = threadIdx.x; e < IR_BLOCK * IR_BLOCK; e += blockDim.x) out[e] = z[e];
}

// Blocked triangular solves after "pre-inversion": every block column of the
// strictly lower part of L is replaced once, after the factorization, by
// M(:, b) = L(:, b) * Linv_b (and the blocks above the diagonal of U by
// N(:, b) = U(:, b) * Uinv_b).  Forward substitution then reads
//     y_b final after the updates of blocks < b;  w_r -= M(r, b) y_b (r > b)
// and x_b = Linv_b y_b is applied to all blocks at once at the end, so the
// dependent chain per block step is one parallel update with no inverse on it.
template <bool LOWER, int NR>
__global__ void __launch_bounds__(256) trsv_update_kernel(const float* __restrict__ M, int lda, int n,
                                                          float* __restrict__ W, int b) {
    __shared__ float yb[NR][IR_BLOCK];
    __shared__ float part[2][NR][IR_BLOCK];
    const int b0 = b * IR_BLOCK, bs = min(IR_BLOCK, n - b0);
    const int rb = LOWER ? b + 1 + blockIdx.x : blockIdx.x;
    const int r0 = rb * IR_BLOCK, rows = min(IR_BLOCK, n - r0);
    for (int q = threadIdx.x; q < bs * NR; q += blockDim.x) yb[q / bs][q % bs] = W[b0 + q % bs + (size_t)(q / bs) * n];
    __syncthreads();
    const int r = threadIdx.x & (IR_BLOCK - 1), hf = threadIdx.x >> 7;
    const int k0 = hf * (IR_BLOCK / 2), k1 = min(bs, k0 + IR_BLOCK / 2);
    float acc[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) acc[j] = 0.f;
    if (r < rows) {
        const float* mp = M + (size_t)(r0 + r) + (size_t)b0 * lda;
        int k = k0;
        for (; k + 16 <= k1; k += 16) {
            float l[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) l[u] = mp[(size_t)(k + u) * lda];
#pragma unroll
            for (int u = 0; u < 16; ++u)
#pragma unroll
                for (int j = 0; j < NR; ++j) acc[j] = fmaf(l[u], yb[j][k + u], acc[j]);
        }
        for (; k < k1; ++k) {
            const float l = mp[(size_t)k * lda];
#pragma unroll
            for (int j = 0; j < NR; ++j) acc[j] = fmaf(l, yb[j][k], acc[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < NR; ++j) part[hf][j][r] = acc[j];
    __syncthreads();
    if (hf == 0 && r < rows)
#pragma unroll
        for (int j = 0; j < NR; ++j) {
            float* wp = W + r0 + r + (size_t)j * n;
            *wp = *wp - (part[0][j][r] + part[1][j][r]);
        }
}

// Out[block b] = inv_b * W[block b] for every block (one CTA per block, the
// 128 x 128 inverse staged in shared memory).
template <int NR>
__global__ void __launch_bounds__(256) blockdiag_apply_kernel(const float* __restrict__ invs,
                                                              const float* __restrict__ W, float* __restrict__ Out,
                                                              int n) {
    extern __shared__ float sinv[];  // IR_BLOCK * IR_BLOCK
    __shared__ float wb[NR][IR_BLOCK];
    __shared__ float part[2][NR][IR_BLOCK];
    const int b0 = blockIdx.x * IR_BLOCK, bs = min(IR_BLOCK, n - b0);
    const float4* src = reinterpret_cast<const float4*>(invs + (size_t)blockIdx.x * IR_BLOCK * IR_BLOCK);
    float4* dst = reinterpret_cast<float4*>(sinv);
    for (int e = threadIdx.x; e < IR_BLOCK * IR_BLOCK / 4; e += blockDim.x) dst[e] = src[e];
    for (int q = threadIdx.x; q < bs * NR; q += blockDim.x) wb[q / bs][q % bs] = W[b0 + q % bs + (size_t)(q / bs) * n];
    __syncthreads();
    const int r = threadIdx.x & (IR_BLOCK - 1), hf = threadIdx.x >> 7;
    const int k0 = hf * (IR_BLOCK / 2), k1 = min(bs, k0 + IR_BLOCK / 2);
    float acc[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) acc[j] = 0.f;
    if (r < bs)
        for (int k = k0; k < k1; ++k) {
            const float v = sinv[r + k * IR_BLOCK];
#pragma unroll
            for (int j = 0; j < NR; ++j) acc[j] = fmaf(v, wb[j][k], acc[j]);
        }
#pragma unroll
    for (int j = 0; j < NR; ++j) part[hf][j][r] = acc[j];
    __syncthreads();
    if (hf == 0 && r < bs)
#pragma unroll
        for (int j = 0; j < NR; ++j) Out[b0 + r + (size_t)j * n] = part[0][j][r] + part[1][j][r];
}

// One blocked triangular solve as a single cooperative dataflow kernel:
// CTA j owns row block j.  For LOWER (L unit lower, forward) it consumes the
// solved blocks b = 0..j-1 in order, for the upper solve b = nblk-1..j+1:
// before waiting it loads its 128x128 block T(j, b) of the packed LU into
// registers, then waits (bounded) for block b's flag, reads x_b and
// accumulates T(j, b) x_b.  When all are in, it forms w_j = rhs_j - sum,
// applies the inverse of its own diagonal block (Dinv, 128 x 128, ld 128),
// writes x_j and raises its flag.  The chain per block step is one flag
// hand-off, one read of x_b and the owner's 128 x 128 inverse apply; every
// other block's update overlaps it.  All CTAs must be co-resident
// (cooperative launch); flags start at zero.
template <bool LOWER, int NR>
__global__ void __launch_bounds__(256) trsv_flow_kernel(const float* __restrict__ LU, int lda, int n,
                                                        const float* __restrict__ Dinv,
                                                        const float* __restrict__ Win, float* __restrict__ Xout,
                                                        unsigned* __restrict__ flags, int* __restrict__ err) {
    extern __shared__ float sdinv[];  // IR_BLOCK * IR_BLOCK
    __shared__ float xb[NR][IR_BLOCK];
    __shared__ float wb[NR][IR_BLOCK];
    __shared__ float part[2][NR][IR_BLOCK];
    __shared__ int s_ok;
    const int nblk = gridDim.x, me = blockIdx.x;
    const int r0 = me * IR_BLOCK, rows = min(IR_BLOCK, n - r0);
    const int r = threadIdx.x & (IR_BLOCK - 1), hf = threadIdx.x >> 7;
    const int k0 = hf * (IR_BLOCK / 2);
    {  // own diagonal-block inverse, needed last (16-byte loads, all in flight together)
        const float4* src = reinterpret_cast<const float4*>(Dinv + (size_t)me * IR_BLOCK * IR_BLOCK);
        float4 t[IR_BLOCK * IR_BLOCK / 4 / 256];
#pragma unroll
        for (int q = 0; q < IR_BLOCK * IR_BLOCK / 4 / 256; ++q) t[q] = src[threadIdx.x + q * 256];
#pragma unroll
        for (int q = 0; q < IR_BLOCK * IR_BLOCK / 4 / 256; ++q)
            reinterpret_cast<float4*>(sdinv)[threadIdx.x + q * 256] = t[q];
    }
    float acc[NR], win[NR];  // this block's right-hand side, loaded now: it is needed at the end of the chain
#pragma unroll
    for (int j = 0; j < NR; ++j) {
        acc[j] = 0.f;
        win[j] = (hf == 0 && r < rows) ? Win[r0 + r + (size_t)j * n] : 0.f;
    }
    const int nsteps = LOWER ? me : nblk - 1 - me;
    for (int t = 0; t < nsteps; ++t) {
        const int b = LOWER ? t : nblk - 1 - t;
        const int c0 = b * IR_BLOCK, bs = min(IR_BLOCK, n - c0);
        float l[IR_BLOCK / 2];
        const float* tp = LU + (size_t)(r0 + r) + (size_t)(c0 + k0) * lda;
#pragma unroll
        for (int u = 0; u < IR_BLOCK / 2; ++u) l[u] = (r < rows && k0 + u < bs) ? tp[(size_t)u * lda] : 0.f;
        if (threadIdx.x == 0) {
            int ok = 1;
            unsigned spins = 0;
            while (mg::ld_acquire_u32(flags + b) == 0u) {
                if (++spins > mg::kSpinLimit) {
                    atomicExch(err, 8 /* MG_TIMEOUT */);
                    ok = 0;
                    break;
                }
                if (spins > 4096) __nanosleep(100);  // a block step takes a few us: poll tightly first
            }
            s_ok = ok;
        }
        __syncthreads();
        if (!s_ok) return;
        for (int q = threadIdx.x; q < bs * NR; q += blockDim.x) {
            const int j = q / bs, i = q - j * bs;
            xb[j][i] = __ldcg(Xout + c0 + i + (size_t)j * n);
        }
        for (int q = bs + threadIdx.x; q < IR_BLOCK; q += blockDim.x)
#pragma unroll
            for (int j = 0; j < NR; ++j) xb[j][q] = 0.f;
        __syncthreads();
#pragma unroll
        for (int u = 0; u < IR_BLOCK / 2; ++u)
#pragma unroll
            for (int j = 0; j < NR; ++j) acc[j] = fmaf(l[u], xb[j][k0 + u], acc[j]);
        __syncthreads();  // xb is rewritten by the next step
    }
#pragma unroll
    for (int j = 0; j < NR; ++j) part[hf][j][r] = acc[j];
    __syncthreads();
    if (hf == 0)
#pragma unroll
        for (int j = 0; j < NR; ++j)
            wb[j][r] = r < rows ? win[j] - (part[0][j][r] + part[1][j][r]) : 0.f;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NR; ++j) acc[j] = 0.f;
    if (r < rows)
        for (int k = k0; k < k0 + IR_BLOCK / 2 && k < rows; ++k) {
            const float v = sdinv[r + k * IR_BLOCK];
#pragma unroll
            for (int j = 0; j < NR; ++j) acc[j] = fmaf(v, wb[j][k], acc[j]);
        }
#pragma unroll
    for (int j = 0; j < NR; ++j) part[hf][j][r] = acc[j];
    __syncthreads();
    if (hf == 0 && r < rows)
#pragma unroll
        for (int j = 0; j < NR; ++j) Xout[r0 + r + (size_t)j * n] = part[0][j][r] + part[1][j][r];
    __syncthreads();
    if (threadIdx.x == 0) mg::st_release_u32(flags + me, 1u);  // publishes the block's x
}

// Largest block count the dataflow solve can take as one cooperative grid.
template <int NR>
int trsv_flow_capacity(mg_handle_t h) {
    const size_t smem = (size_t)IR_BLOCK * IR_BLOCK * sizeof(float);
    if (cudaFuncSetAttribute(trsv_flow_kernel<true, NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess ||
        cudaFuncSetAttribute(trsv_flow_kernel<false, NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int a = 0, b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, trsv_flow_kernel<true, NR>, 256, smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, trsv_flow_kernel<false, NR>, 256, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return std::min(a, b) * h->num_sms;
}

// Both triangular solves of one correction with the dataflow kernel:
// Y (in) -> Z = L^-1 Y -> Y = U^-1 Z.  flags: 2 * nblk words.
template <int NR>
mg_status_t lu_solve_flow(mg_handle_t h, const float* LU, int n, const float* Linv, const float* Uinv, float* Y,
                          float* Z, unsigned* flags, int* err) {
    cudaStream_t st = h->stream;
    const int nblk = (n + IR_BLOCK - 1) / IR_BLOCK;
    const size_t smem = (size_t)IR_BLOCK * IR_BLOCK * sizeof(float);
    MG_CHECK_CUDA(h, cudaMemsetAsync(flags, 0, 2 * (size_t)nblk * sizeof(unsigned), st));
    int lda = n;
    unsigned* fl = flags;
    unsigned* fu = flags + nblk;
    void* a1[] = {(void*)&LU, &lda, &n, (void*)&Linv, (void*)&Y, (void*)&Z, (void*)&fl, (void*)&err};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)trsv_flow_kernel<true, NR>, dim3(nblk), dim3(256), a1,
                                                smem, st);
    if (e != cudaSuccess) return mg::cuda_fail(h, e, "trsv_flow_kernel<lower> launch");
    h->launches++;
    void* a2[] = {(void*)&LU, &lda, &n, (void*)&Uinv, (void*)&Z, (void*)&Y, (void*)&fu, (void*)&err};
    e = cudaLaunchCooperativeKernel((const void*)trsv_flow_kernel<false, NR>, dim3(nblk), dim3(256), a2, smem, st);
    if (e != cudaSuccess) return mg::cuda_fail(h, e, "trsv_flow_kernel<upper> launch");
    h->launches++;
    return MG_OK;
}

// The upper solve alone with the dataflow kernel: Out = U^-1 In (the mixed
// QR's R).  flags: nblk words.
template <int NR>
mg_status_t upper_solve_flow(mg_handle_t h, const float* LU, int n, const float* Uinv, float* In, float* Out,
                             unsigned* flags, int* err) {
    cudaStream_t st = h->stream;
    const int nblk = (n + IR_BLOCK - 1) / IR_BLOCK;
    const size_t smem = (size_t)IR_BLOCK * IR_BLOCK * sizeof(float);
    MG_CHECK_CUDA(h, cudaMemsetAsync(flags, 0, (size_t)nblk * sizeof(unsigned), st));
    int lda = n;
    void* a2[] = {(void*)&LU, &lda, &n, (void*)&Uinv, (void*)&In, (void*)&Out, (void*)&flags, (void*)&err};
    const cudaError_t e =
        cudaLaunchCooperativeKernel((const void*)trsv_flow_kernel<false, NR>, dim3(nblk), dim3(256), a2, smem, st);
    if (e != cudaSuccess) return mg::cuda_fail(h, e, "trsv_flow_kernel<upper> launch");
    h->launches++;
    return MG_OK;
}

// Both triangular solves of one correction: Y (in, destroyed) -> Y = U^-1 L^-1 Y, Z scratch.
template <int NR>
mg_status_t lu_solve_blocked(mg_handle_t h, const float* LU, int n, const float* Linv, const float* Uinv, float* Y,
                             float* Z) {
    cudaStream_t st = h->stream;
    const int nblk = (n + IR_BLOCK - 1) / IR_BLOCK;
    const size_t ism = (size_t)IR_BLOCK * IR_BLOCK * sizeof(float);
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(blockdiag_apply_kernel<NR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)ism));
    for (int b = 0; b + 1 < nblk; ++b) {
        trsv_update_kernel<true, NR><<<nblk - 1 - b, 256, 0, st>>>(LU, n, n, Y, b);
        MG_TRY(mg::post_launch(h, "trsv_update_kernel<lower>"));
    }
    blockdiag_apply_kernel<NR><<<nblk, 256, ism, st>>>(Linv, Y, Z, n);
    MG_TRY(mg::post_launch(h, "blockdiag_apply_kernel"));
    for (int b = nblk - 1; b > 0; --b) {
        trsv_update_kernel<false, NR><<<b, 256, 0, st>>>(LU, n, n, Z, b);
        MG_TRY(mg::post_launch(h, "trsv_update_kernel<upper>"));
    }
    blockdiag_apply_kernel<NR><<<nblk, 256, ism, st>>>(Uinv, Z, Y, n);
    return mg::post_launch(h, "blockdiag_apply_kernel");
}

// Replaces the off-diagonal block columns of the packed LU by M = L(:,b) Linv_b
// (below the diagonal) and N = U(:,b) Uinv_b (above it), with split-BF16
// tensor-core GEMMs (fp32-level accuracy).
mg_status_t preinvert_blocks(mg_handle_t h, float* LU, int n, const float* Linv, const float* Uinv, int nterms,
                             void* splitA, void* splitB, int* gemm_err) {
    const int nblk = (n + IR_BLOCK - 1) / IR_BLOCK;
    for (int b = 0; b < nblk; ++b) {
        const int b0 = b * IR_BLOCK, bs = IR_BLOCK < n - b0 ? IR_BLOCK : n - b0, b1 = b0 + bs;
        if (b1 < n) {  // below: (n - b1) x bs
            float* C = LU + b1 + (size_t)b0 * n;
            MG_TRY(mg::bf16x_split<float>(h, true, C, n, n - b1, bs, nterms, splitA));
            MG_TRY(mg::bf16x_split<float>(h, false, Linv + (size_t)b * IR_BLOCK * IR_BLOCK, IR_BLOCK, bs, bs,
                                          nterms, splitB));
            MG_TRY(mg::bf16x_gemm_presplit(h, nterms, n - b1, bs, bs, 1.0f, splitA, splitB, 0.0f, C, n, gemm_err));
        }
        if (b0 > 0) {  // above: b0 x bs
            float* C = LU + (size_t)b0 * n;
            MG_TRY(mg::bf16x_split<float>(h, true, C, n, b0, bs, nterms, splitA));
            MG_TRY(mg::bf16x_split<float>(h, false, Uinv + (size_t)b * IR_BLOCK * IR_BLOCK, IR_BLOCK, bs, bs,
                                          nterms, splitB));
            MG_TRY(mg::bf16x_gemm_presplit(h, nterms, b0, bs, bs, 1.0f, splitA, splitB, 0.0f, C, n, gemm_err));
        }
    }
    return MG_OK;
}

struct IrWs {
    unsigned* flags;  // dataflow triangular-solve flags, 2 * nblk
    float* A32;
    int* pos;
    void* xchg;
    void* splitA;
    void* splitA2;
    void* splitB;
    int* gemm_err;
    float* Linv;
    float* Uinv;
    double* R;
    double* partial;  // also the integer residual's partials (long long)
    int* rexp;        // the integer residual's row exponents (n)
    long long* Ai;    // A's integers for the integer residual (n x n, ld n), written by the first
    int* xdig;        // the digits of the integer residual's right-hand factor (n x 3 x nrhs + padding)
    double* norms;  // [0..8) rnorm, [8..16) xnorm, [16] anorm, [24..32) scale
    float* Y;
    float* Z;
    double* gV;     // GMRES basis, (GM_RESTART + 1) x nrhs x n
    double* gW;     // n x nrhs
    double* gP;     // Gram-Schmidt partial sums, GM_CTAS x (GM_RESTART + 1) x nrhs
    double* gC;     // coefficients for the device, (GM_RESTART + 1) x nrhs
    void* qws;      // mixed QR: panel reflectors, products, partial sums (QR mode only)
};

size_t carve_ir(mg_handle_t h, int n, int nrhs, int nterms, IrWs* w, bool qr, bool ai) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = mg::align_up(off + bytes, 1024);
        return o;
    };
    const int nblk = (n + IR_BLOCK - 1) / IR_BLOCK;
    const int kch = (n + RES_KCHUNK - 1) / RES_KCHUNK;
    const size_t oA = take((size_t)n * n * sizeof(float));
    const size_t oP = take((size_t)n * sizeof(int));
    const size_t oX = take(mg::sgetrf_xchg_bytes(h->num_sms));
    const size_t oSA = take(mg::bf16x_split_bytes(n, IR_BLOCK, nterms));
    const size_t oSA2 = take(mg::bf16x_split_bytes(n, IR_BLOCK, nterms));
    const size_t oSB = take(mg::bf16x_split_bytes(n, IR_BLOCK, nterms));
    const size_t oE = take(64);
    const size_t oLi = take((size_t)nblk * IR_BLOCK * IR_BLOCK * sizeof(float));
    const size_t oUi = take((size_t)nblk * IR_BLOCK * IR_BLOCK * sizeof(float));
    const size_t oR = take((size_t)n * nrhs * sizeof(double));
    const int kd2s = (n + D2S_KCHUNK - 1) / D2S_KCHUNK;
    const int rich = (n + resint_kchunk(n, h->num_sms) - 1) / resint_kchunk(n, h->num_sms);
    const size_t oPa = take((size_t)std::max({kch * std::max(nrhs, 1), kd2s, RI_CLASSES * rich * std::max(nrhs, 1)}) *
                            n * sizeof(double));
    const size_t oRe = take((size_t)n * sizeof(int));
    const size_t oAi = take(ai ? (size_t)n * n * sizeof(long long) : 0);
    const size_t oXd = take(xdig_bytes(n, nrhs));
    const size_t oN = take(64 * sizeof(double));
    const size_t oF = take(2 * (size_t)nblk * sizeof(unsigned));
    const size_t oY = take((size_t)n * nrhs * sizeof(float));
    const size_t oZ = take((size_t)n * nrhs * sizeof(float));
    const size_t ogV = take((size_t)(GM_RESTART + 1) * nrhs * n * sizeof(double));
    const size_t ogW = take((size_t)n * nrhs * sizeof(double));
    const size_t ogP = take((size_t)GM_CTAS * (GM_RESTART + 1) * nrhs * sizeof(double));
    const size_t ogC = take((size_t)(GM_RESTART + 1) * nrhs * sizeof(double));
    const size_t oQ = take(qr ? mg::qr_mixed_ws_bytes(n, n, h->num_sms) : 0);
    if (w) {
        char* b = (char*)h->ws;
        w->A32 = (float*)(b + oA);
        w->pos = (int*)(b + oP);
        w->xchg = b + oX;
        w->splitA = b + oSA;
        w->splitA2 = b + oSA2;
        w->splitB = b + oSB;
        w->gemm_err = (int*)(b + oE);
        w->Linv = (float*)(b + oLi);
        w->Uinv = (float*)(b + oUi);
        w->R = (double*)(b + oR);
        w->partial = (double*)(b + oPa);
        w->rexp = (int*)(b + oRe);
        w->Ai = ai ? (long long*)(b + oAi) : nullptr;
        w->xdig = (int*)(b + oXd);
        w->norms = (double*)(b + oN);
        w->flags = (unsigned*)(b + oF);
        w->Y = (float*)(b + oY);
        w->Z = (float*)(b + oZ);
        w->gV = (double*)(b + ogV);
        w->gW = (double*)(b + ogW);
        w->gP = (double*)(b + ogP);
        w->gC = (double*)(b + ogC);
        w->qws = qr ? b + oQ : nullptr;
    }
    return off;
}

int grid_for(size_t total, int threads, int cap) {
    size_t b = (total + threads - 1) / threads;
    if (b > (size_t)cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace

static __global__ void pos_iota_kernel(int* pos, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) pos[i] = i;
}

// The mixed solve: the fp32 factorization (LU with partial or tournament
// pivoting; for spd, Cholesky rewritten as the packed LU of the same
// matrix), then plain refinement, GMRES-IR and the FP64 fallback.
enum class MixedKind { LU, SPD, QR };

static mg_status_t mixed_solve(mg_handle_t h, int n, int nrhs, const double* A, int lda, const double* B, int ldb,
                               double* X, int ldx, const mg_ir_opts* opts, mg_ir_report* rep, MixedKind kind) {
    const bool spd = kind == MixedKind::SPD, qr = kind == MixedKind::QR;
    using clk = std::chrono::steady_clock;
    if (!h) return MG_ERR_ARG;
    if (n < 0 || nrhs < 0 || nrhs > MAX_RHS || lda < (n > 1 ? n : 1) || ldb < (n > 1 ? n : 1) ||
        ldx < (n > 1 ? n : 1))
        return mg::fail(h, MG_ERR_ARG, "mixed solve: bad arguments (n=%d nrhs=%d, nrhs must be <= %d)", n, nrhs,
                        MAX_RHS);
    mg_ir_opts o = {1e-14, 30, 3, 1, 1, 0, 0};
    if (opts) o = *opts;
    if (o.nterms < 1 || o.nterms > 3) return mg::fail(h, MG_ERR_ARG, "mixed solve: nterms must be 1..3");
    if (o.max_iter < 1) o.max_iter = 1;
    mg_ir_report r = {};
    r.path = 0;
    if (n == 0 || nrhs == 0) {
        if (rep) *rep = r;
        return MG_OK;
    }
    if (!A || !B || !X) return mg::fail(h, MG_ERR_ARG, "mixed solve: null pointer");

    const auto t0 = clk::now();
    MG_TRY(mg::ensure_ws(h, carve_ir(h, n, nrhs, o.nterms, nullptr, qr, o.residual == 0)));
    MG_TRY(mg::ensure_hws(h, 512 + sizeof(double) * GM_CTAS * (GM_RESTART + 1) * MAX_RHS));
    IrWs w;
    carve_ir(h, n, nrhs, o.nterms, &w, qr, o.residual == 0);
    cudaStream_t st = h->stream;
    const int cap = h->num_sms * 8;
    const int kch = (n + RES_KCHUNK - 1) / RES_KCHUNK;
    const int nblk = (n + IR_BLOCK - 1) / IR_BLOCK;
    double* hn = (double*)h->hws;

    // ||A||_inf and ||B||_inf (column-wise) --------------------------------
    std::optional<mg::ProfScope> setup;  // closed (its events recorded and released) on every return path
    setup.emplace(h, "ir_setup", 0.0, 12.0 * n * (double)n);
    MG_CHECK_CUDA(h, cudaMemsetAsync(w.gemm_err, 0, 64, st));
    MG_CHECK_CUDA(h, cudaMemsetAsync(w.norms, 0, 64 * sizeof(double), st));
    MG_CHECK_CUDA(h, cudaMemsetAsync(w.rexp, 0, (size_t)n * sizeof(int), st));
    // fp32 copy and the row sums of |A| (one pass, also the row exponents of
    // the integer residual and A's non-finite flag, error word 4), then ||A||_inf
    const int kd2s = (n + D2S_KCHUNK - 1) / D2S_KCHUNK;
    if ((lda & 3) == 0 && (n & 3) == 0 && ((reinterpret_cast<uintptr_t>(A) & 15) == 0)) {
        d2s_absrow_kernel<<<dim3((n + D2S_ROWS - 1) / D2S_ROWS, kd2s), 256, 0, st>>>(A, lda, n, w.A32, n, w.partial,
                                                                                   w.norms + 17, w.rexp,
                                                                                   w.gemm_err + 4);
        MG_TRY(mg::post_launch(h, "d2s_absrow_kernel"));
    } else {
        d2s_absrow_scalar_kernel<<<dim3((n + 255) / 256, kd2s), 256, 0, st>>>(A, lda, n, w.A32, n, w.partial,
                                                                            w.norms + 17, w.rexp, w.gemm_err + 4);
        MG_TRY(mg::post_launch(h, "d2s_absrow_scalar_kernel"));
    }
    absrow_reduce_kernel<<<(n + 255) / 256, 256, 0, st>>>(w.partial, kd2s, n, w.norms + 16);
    MG_TRY(mg::post_launch(h, "absrow_reduce_kernel"));
    setup.reset();

    // fp32 factorization ---------------------------------------------------------
    int info = 0;
    mg_status_t s = MG_OK;
    if (spd) {
        // Cholesky of the lower triangle, then L L^T as a packed LU with pos = identity
        pos_iota_kernel<<<(n + 255) / 256, 256, 0, st>>>(w.pos, n);
        MG_TRY(mg::post_launch(h, "pos_iota_kernel"));
        s = mg::spotrf_mixed(h, n, w.A32, n, o.nterms, w.splitA, w.Linv, w.gemm_err, &info);
        if (s != MG_OK && s != MG_NOT_SPD) return s;
        if (s == MG_NOT_SPD) {  // the fp32 Cholesky broke down: straight to the FP64 solve
            r.info = info;
            if (!o.fallback) {
                if (rep) *rep = r;
                return mg::fail(h, MG_NOT_SPD, "mg_dsposv_ir: fp32 Cholesky broke down at column %d", info);
            }
            int finfo = 0;
            const mg_status_t fs = mg_dgesv(h, n, nrhs, A, lda, B, ldb, X, ldx, &finfo);
            if (fs != MG_OK) return fs;
            r.path = 2;
            if (rep) *rep = r;
            return MG_FALLBACK_USED;
        }
        MG_TRY(mg::chol_to_lu_f32(h, n, w.A32, n, w.Y));
    } else if (qr) {
        // Householder QR of the fp32 copy: R and the reflectors in A32, T blocks
        // in Linv's area, tau (FP64) in splitA's (the LU's split area, unused
        // here); pos = identity for the correction's right-hand-side scaling
        MG_TRY(mg::sgeqrf_mixed(h, n, n, w.A32, n, (double*)w.splitA, w.Linv, w.qws, w.gemm_err + 2));
        pos_iota_kernel<<<(n + 255) / 256, 256, 0, st>>>(w.pos, n);
        MG_TRY(mg::post_launch(h, "pos_iota_kernel"));
    } else {
        s = mg::sgetrf_mixed(h, n, w.A32, n, w.pos, IR_BLOCK, o.nterms, w.xchg, w.splitA, w.splitA2, w.splitB,
                             w.gemm_err, &info, o.panel == 2);
        if (s != MG_OK && s != MG_SINGULAR) return s;
    }
    r.info = info;
    // max |U| for the pivot-growth report, on the side stream beside the
    // refinement (read back at the end of the solve)
    MG_TRY(mg::ensure_lookahead(h));
    MG_CHECK_CUDA(h, cudaEventRecord(h->pp_ev[0], st));
    MG_CHECK_CUDA(h, cudaStreamWaitEvent(h->pp_stream, h->pp_ev[0], 0));
    absmax_upper_kernel<<<n, 256, 0, h->pp_stream>>>(w.A32, n, w.norms + 18);
    MG_TRY(mg::post_launch(h, "absmax_upper_kernel"));
    MG_CHECK_CUDA(h, cudaEventRecord(h->pp_ev[1], h->pp_stream));
    auto read_growth = [&]() -> mg_status_t {
        MG_CHECK_CUDA(h, cudaStreamWaitEvent(st, h->pp_ev[1], 0));
        MG_CHECK_CUDA(h, cudaMemcpyAsync(hn + 40, w.norms + 17, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
        MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
        r.pivot_growth = hn[40] > 0 ? hn[41] / hn[40] : 0.0;
        return MG_OK;
    };
    bool flow = false;
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(inv_diag_blocks_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          2 * IR_BLOCK * IR_BLOCK * (int)sizeof(float)));
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(inv_diag_blocks_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          2 * IR_BLOCK * IR_BLOCK * (int)sizeof(float)));
    if (qr) {
        // inverses of R's diagonal blocks for the correction's dataflow upper
        // solve; without a co-resident dataflow grid the correction stays on
        // the FP64 path
        inv_diag_blocks_kernel<false><<<nblk, IR_BLOCK, 2 * IR_BLOCK * IR_BLOCK * sizeof(float), st>>>(w.A32, n, n,
                                                                                                      w.Uinv);
        MG_TRY(mg::post_launch(h, "inv_diag_blocks_kernel<upper>"));
        int flow_cap = 0;
        switch (nrhs) {
    #define MG_CAP(NRV) \
        case NRV: flow_cap = trsv_flow_capacity<NRV>(h); break;
            MG_CAP(1) MG_CAP(2) MG_CAP(3) MG_CAP(4) MG_CAP(5) MG_CAP(6) MG_CAP(7)
            default: flow_cap = trsv_flow_capacity<8>(h); break;
    #undef MG_CAP
        }
        flow = nblk <= flow_cap;
    } else {
        // inverses of the diagonal blocks of L and U (the solves' block steps);
        // L's blocks are final once their panel is done (later interchanges only
        // touch rows below them)
        // L's on the look-ahead stream beside U's
        MG_CHECK_CUDA(h, cudaEventRecord(h->la_ev[0], st));
        MG_CHECK_CUDA(h, cudaStreamWaitEvent(h->la_stream, h->la_ev[0], 0));
        inv_diag_blocks_kernel<true><<<nblk, IR_BLOCK, 2 * IR_BLOCK * IR_BLOCK * sizeof(float), h->la_stream>>>(
            w.A32, n, n, w.Linv);
        MG_TRY(mg::post_launch(h, "inv_diag_blocks_kernel<lower>"));
        MG_CHECK_CUDA(h, cudaEventRecord(h->la_ev[1], h->la_stream));
        inv_diag_blocks_kernel<false><<<nblk, IR_BLOCK, 2 * IR_BLOCK * IR_BLOCK * sizeof(float), st>>>(w.A32, n, n,
                                                                                                      w.Uinv);
        MG_TRY(mg::post_launch(h, "inv_diag_blocks_kernel<upper>"));
        MG_CHECK_CUDA(h, cudaStreamWaitEvent(st, h->la_ev[1], 0));
        int flow_cap = 0;
        switch (nrhs) {
    #define MG_CAP(NRV) \
        case NRV: flow_cap = trsv_flow_capacity<NRV>(h); break;
            MG_CAP(1) MG_CAP(2) MG_CAP(3) MG_CAP(4) MG_CAP(5) MG_CAP(6) MG_CAP(7)
            default: flow_cap = trsv_flow_capacity<8>(h); break;
    #undef MG_CAP
        }
        flow = nblk <= flow_cap;
        if (!flow) {  // launch-per-block-step solves need the pre-inverted block columns
            mg::ProfScope prof(h, "ir_preinvert", 2.0 * n * (double)n * IR_BLOCK * 6, 8.0 * n * (double)n);
            MG_TRY(preinvert_blocks(h, w.A32, n, w.Linv, w.Uinv, o.nterms, w.splitA, w.splitB, w.gemm_err));
        }
    }
    MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
    const auto t1 = clk::now();
    r.factor_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();

    // refinement --------------------------------------------------------------
    const dim3 rgrid((n + RES_ROWS - 1) / RES_ROWS, kch);
    // the integer residual unless asked for FP64 or A holds an infinity or NaN
    // (error word 4, read back with the first residual, before any product)
    bool int_res = o.residual == 0;
    bool ai_ready = false;  // w.Ai holds A's integers
    const int ri_chunk = resint_kchunk(n, h->num_sms);
    const int ri_kch = (n + ri_chunk - 1) / ri_chunk;
    int* const vexp = w.gemm_err + 8;      // the integer residual's column exponents (8)
    int* const vbad = w.gemm_err + 5;      // ... and V's non-finite flag
    long long* const ipart = reinterpret_cast<long long*>(w.partial);
    // partial sums of A V (V n x nrhs, ld ldv) in w.partial: fp64 FMA, or the
    // integer residual's classes
    auto launch_av = [&](const double* V, int ldv) -> mg_status_t {
        if (int_res) {
            MG_CHECK_CUDA(h, cudaMemsetAsync(vbad, 0, 11 * sizeof(int), st));
            colexp_kernel<<<dim3(std::min(64, (n + 255) / 256), nrhs), 256, 0, st>>>(V, ldv, n, nrhs, vexp, vbad);
            MG_TRY(mg::post_launch(h, "colexp_kernel"));
            const dim3 g((n + RI_ROWS - 1) / RI_ROWS, ri_kch);
            // the first product also stores A's integers; the later ones read them
            xdigits_kernel<<<grid_for((size_t)n * nrhs, 256, cap), 256, 0, st>>>(V, ldv, n, nrhs, vexp, w.xdig);
            MG_TRY(mg::post_launch(h, "xdigits_kernel"));
            MG_CHECK_CUDA(h, launch_resint(ai_ready ? 2 : 1, nrhs, g, st, A, lda, w.Ai, n, n, w.xdig, ri_chunk, w.rexp,
                                           ipart));
            ai_ready = true;
            return mg::post_launch(h, "residual_int_kernel");
        }
        switch (nrhs) {
#define MG_RES(NRV) \
    case NRV: residual_partial_kernel<NRV><<<rgrid, RES_ROWS, 0, st>>>(A, lda, n, V, ldv, w.partial); break;
            MG_RES(1) MG_RES(2) MG_RES(3) MG_RES(4) MG_RES(5) MG_RES(6) MG_RES(7)
            default: residual_partial_kernel<8><<<rgrid, RES_ROWS, 0, st>>>(A, lda, n, V, ldv, w.partial); break;
#undef MG_RES
        }
        return mg::post_launch(h, "residual_partial_kernel");
    };
    // Y = A V from the partials of launch_av
    auto reduce_av = [&](double* Y) -> mg_status_t {
        if (int_res) {
            matvec_int_reduce_kernel<<<(n + 255) / 256, 256, 0, st>>>(ipart, ri_kch, n, nrhs, w.rexp, vexp, vbad, Y);
            return mg::post_launch(h, "matvec_int_reduce_kernel");
        }
        matvec_reduce_kernel<<<(n + 255) / 256, 256, 0, st>>>(w.partial, kch, n, nrhs, Y);
        return mg::post_launch(h, "matvec_reduce_kernel");
    };
    double bnorm[MAX_RHS] = {0};
    int nres = 0;  // residuals evaluated (plain and GMRES-IR steps): the history index
    // r = b - A x (x_zero: x = 0, r = b) and the max-over-columns normwise
    // backward error; also checks the device error words
    auto residual = [&](bool x_zero, double* eta_out) -> mg_status_t {
        MG_CHECK_CUDA(h, cudaMemsetAsync(w.norms, 0, 16 * sizeof(double), st));
        {
            mg::ProfScope pr(h, "ir_residual", x_zero ? 0.0 : 2.0 * n * (double)n * nrhs,
                             x_zero ? 0.0 : 8.0 * n * (double)n);
            if (!x_zero) MG_TRY(launch_av(X, ldx));
            if (!x_zero && int_res) {
                residual_int_reduce_kernel<<<(n + 255) / 256, 256, 0, st>>>(ipart, ri_kch, n, nrhs, w.rexp, vexp, vbad,
                                                                           B, ldb, X, ldx, w.R, n, w.norms);
                MG_TRY(mg::post_launch(h, "residual_int_reduce_kernel"));
            } else {
                residual_reduce_kernel<<<(n + 255) / 256, 256, 0, st>>>(w.partial, x_zero ? 0 : kch, n, nrhs, B, ldb,
                                                                       X, ldx, w.R, n, w.norms);
                MG_TRY(mg::post_launch(h, "residual_reduce_kernel"));
            }
        }
        MG_CHECK_CUDA(h, cudaMemcpyAsync(hn, w.norms, 32 * sizeof(double), cudaMemcpyDeviceToHost, st));
        int* herr = (int*)(hn + 48);  // device error words: split GEMM, triangular solves, QR panel, -, A non-finite
        MG_CHECK_CUDA(h, cudaMemcpyAsync(herr, w.gemm_err, 5 * sizeof(int), cudaMemcpyDeviceToHost, st));
        MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
        if (herr[0] || herr[1] || herr[2])
            return mg::fail(h, MG_TIMEOUT, "mixed solve: a bounded device wait timed out (%s)",
                            herr[0] ? "split GEMM" : herr[1] ? "triangular solve" : "QR panel");
        if (herr[4]) int_res = false;  // A holds an infinity or NaN: FP64 residuals propagate it
        const double anorm = hn[16];
        double eta = 0.0;
        for (int j = 0; j < nrhs; ++j) {
            if (x_zero) bnorm[j] = hn[j];  // x = 0: r = b
            const double den = anorm * hn[MAX_RHS + j] + bnorm[j];
            const double e = den > 0 ? hn[j] / den : 0.0;
            eta = std::max(eta, e);
        }
        r.anorm_inf = anorm;
        r.backward_error = eta;
        if (nres < 32) r.history[nres] = eta;
        ++nres;
        *eta_out = eta;
        return MG_OK;
    };

    // plain refinement: x = 0, so the first residual is b itself
    MG_CHECK_CUDA(h, cudaMemset2DAsync(X, (size_t)ldx * sizeof(double), 0, (size_t)n * sizeof(double), nrhs, st));
    double prev_eta = INFINITY;
    int slow = 0;
    bool converged = false;
    for (int it = 0; it <= o.max_iter; ++it) {
        double eta = 0.0;
        MG_TRY(residual(it == 0, &eta));
        r.iterations = it;
        if (it > 0 && eta <= o.tol) {
            converged = true;
            break;
        }
        if (it > 1) {
            slow = eta > 0.5 * prev_eta ? slow + 1 : 0;
            if (slow >= 2) break;
        }
        if (it == o.max_iter) break;
        prev_eta = eta;
        if (qr && !flow) {  // correction d = R^{-1} Q^T r in FP64 with the fp32 factors, x += d
            mg::ProfScope ps(h, "ir_qr_solve", 4.0 * n * (double)n * nrhs, 6.0 * n * (double)n);
            MG_TRY(mg::qr_solve_f32_factors(h, n, nrhs, w.A32, n, w.Linv, w.R, n, w.gW, n, w.qws));
            add_correction_kernel<<<grid_for((size_t)n * nrhs, 256, cap), 256, 0, st>>>(n, nrhs, w.gW, X, ldx);
            MG_TRY(mg::post_launch(h, "add_correction_kernel"));
            continue;
        }
        if (qr) {  // correction in fp32 as the LU's: d = R^{-1} Q^T (r / s), x += s d
            for (int j = 0; j < nrhs; ++j) hn[24 + j] = hn[j];
            MG_CHECK_CUDA(h, cudaMemcpyAsync(w.norms + 24, hn + 24, MAX_RHS * sizeof(double), cudaMemcpyHostToDevice,
                                             st));
            mg::ProfScope ps(h, "ir_qr_solve", 4.0 * n * (double)n * nrhs, 6.0 * n * (double)n);
            prep_rhs_kernel<<<grid_for((size_t)n * nrhs, 256, cap), 256, 0, st>>>(n, nrhs, w.pos, w.R, w.norms + 24,
                                                                                 w.Y);
            MG_TRY(mg::post_launch(h, "prep_rhs_kernel"));
            int* terr = w.gemm_err + 1;
            MG_TRY(mg::qr_apply_qt_f32(h, n, nrhs, w.A32, n, w.Linv, w.Y, n, w.qws, terr));
            switch (nrhs) {
#define MG_USOLVE(NRV)                                                                         \
    case NRV:                                                                                  \
        MG_TRY(upper_solve_flow<NRV>(h, w.A32, n, w.Uinv, w.Y, w.Z, w.flags, terr));           \
        break;
                MG_USOLVE(1) MG_USOLVE(2) MG_USOLVE(3) MG_USOLVE(4) MG_USOLVE(5) MG_USOLVE(6) MG_USOLVE(7)
                default: MG_USOLVE(8)
#undef MG_USOLVE
            }
            update_x_kernel<<<grid_for((size_t)n * nrhs, 256, cap), 256, 0, st>>>(n, nrhs, w.Z, w.norms + 24, X, ldx);
            MG_TRY(mg::post_launch(h, "update_x_kernel"));
            continue;
        }
        // correction: d = U^-1 L^-1 P (r / s), x += s d
        for (int j = 0; j < nrhs; ++j) hn[24 + j] = hn[j];
        MG_CHECK_CUDA(h, cudaMemcpyAsync(w.norms + 24, hn + 24, MAX_RHS * sizeof(double), cudaMemcpyHostToDevice, st));
        mg::ProfScope ps(h, "ir_trsv", 2.0 * n * (double)n * nrhs, 4.0 * n * (double)n);
        prep_rhs_kernel<<<grid_for((size_t)n * nrhs, 256, cap), 256, 0, st>>>(n, nrhs, w.pos, w.R, w.norms + 24, w.Y);
        MG_TRY(mg::post_launch(h, "prep_rhs_kernel"));
        int* terr = w.gemm_err + 1;
        switch (nrhs) {
#define MG_SOLVE(NRV)                                                                                       \
    case NRV:                                                                                               \
        if (flow)                                                                                           \
            MG_TRY(lu_solve_flow<NRV>(h, w.A32, n, w.Linv, w.Uinv, w.Y, w.Z, w.flags, terr));               \
        else                                                                                                \
            MG_TRY(lu_solve_blocked<NRV>(h, w.A32, n, w.Linv, w.Uinv, w.Y, w.Z));                           \
        break;
            MG_SOLVE(1) MG_SOLVE(2) MG_SOLVE(3) MG_SOLVE(4) MG_SOLVE(5) MG_SOLVE(6) MG_SOLVE(7)
            default: MG_SOLVE(8)
#undef MG_SOLVE
        }
        update_x_kernel<<<grid_for((size_t)n * nrhs, 256, cap), 256, 0, st>>>(n, nrhs, w.Y, w.norms + 24, X, ldx);
        MG_TRY(mg::post_launch(h, "update_x_kernel"));
    }

    // GMRES-IR: each correction A d = r solved by FP64 GMRES left-
    // preconditioned by the fp32 factors (applied in FP64: the fixed operator
    // M^{-1}, M = P^T L U), from x = 0.  Needs the factors as factored (the
    // launch-per-block solves of very large n pre-invert L's and U's block
    // columns in place).
    // the preconditioner of GMRES-IR: M^{-1} applied in FP64 with the fp32 factors
    auto precond = [&](const double* Src, double* Dst) -> mg_status_t {
        if (qr) return mg::qr_solve_f32_factors(h, n, nrhs, w.A32, n, w.Linv, Src, n, Dst, n, w.qws);
        return mg::lu_solve_f32_factors(h, n, nrhs, w.A32, n, w.pos, Src, n, Dst, n);
    };
    if (!converged && o.gmres && (flow || qr)) {
        constexpr int kOuter = 10;
        constexpr double kInnerTol = 1e-8;
        const int pstride = (GM_RESTART + 1) * nrhs;
        double* hp = hn + 64;  // GM_CTAS x pstride partial sums
        const int egrid = grid_for((size_t)n * nrhs, 256, cap);
        std::vector<double> H((size_t)nrhs * (GM_RESTART + 1) * GM_RESTART), g((size_t)nrhs * (GM_RESTART + 1)),
            cs((size_t)nrhs * GM_RESTART), sn((size_t)nrhs * GM_RESTART), beta(nrhs), coef((size_t)pstride);
        auto Hat = [&](int j, int i, int k) -> double& { return H[((size_t)j * (GM_RESTART + 1) + i) * GM_RESTART + k]; };
        // host sums (CTAs in order) of V_k(:, j) . Wv(:, j), k < nv -> coef[k * nrhs + j]
        auto dots = [&](const double* Vb, int nv, const double* Wv) -> mg_status_t {
            gs_dots_kernel<<<GM_CTAS, GM_THREADS, 0, st>>>(n, nv, nrhs, Vb, Wv, w.gP, pstride);
            MG_TRY(mg::post_launch(h, "gs_dots_kernel"));
            MG_CHECK_CUDA(h, cudaMemcpy2DAsync(hp, (size_t)nv * nrhs * sizeof(double), w.gP, pstride * sizeof(double),
                                               (size_t)nv * nrhs * sizeof(double), GM_CTAS, cudaMemcpyDeviceToHost,
                                               st));
            MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
            for (int q = 0; q < nv * nrhs; ++q) {
                double t = 0.0;
                for (int c = 0; c < GM_CTAS; ++c) t += hp[(size_t)c * nv * nrhs + q];
                coef[q] = t;
            }
            return MG_OK;
        };
        auto upload = [&](int count) -> mg_status_t {  // coef[0 .. count) -> w.gC
            MG_CHECK_CUDA(h, cudaMemcpyAsync(w.gC, coef.data(), (size_t)count * sizeof(double),
                                             cudaMemcpyHostToDevice, st));
            return MG_OK;
        };
        MG_CHECK_CUDA(h, cudaMemset2DAsync(X, (size_t)ldx * sizeof(double), 0, (size_t)n * sizeof(double), nrhs, st));
        prev_eta = INFINITY;
        slow = 0;
        for (int ot = 0; ot < kOuter; ++ot) {
            double eta = 0.0;
            MG_TRY(residual(ot == 0, &eta));
            r.iterations += 1;
            if (eta <= o.tol) {
                converged = true;
                r.path = 1;
                break;
            }
            if (ot > 1) {
                slow = eta > 0.5 * prev_eta ? slow + 1 : 0;
                if (slow >= 2) break;
            }
            prev_eta = eta;
            mg::ProfScope pg(h, "gmres", 0.0, 0.0);
            // V_0 = z / beta, z = M^{-1} r
            MG_TRY(precond(w.R, w.gW));
            MG_TRY(dots(w.gW, 1, w.gW));
            for (int j = 0; j < nrhs; ++j) {
                beta[j] = std::sqrt(coef[j]);
                coef[j] = beta[j] > 0.0 ? 1.0 / beta[j] : 0.0;
            }
            MG_TRY(upload(nrhs));
            gs_scale_kernel<<<egrid, 256, 0, st>>>(n, nrhs, w.gW, w.gC, w.gV);
            MG_TRY(mg::post_launch(h, "gs_scale_kernel"));
            std::fill(H.begin(), H.end(), 0.0);
            std::fill(g.begin(), g.end(), 0.0);
            for (int j = 0; j < nrhs; ++j) g[(size_t)j * (GM_RESTART + 1)] = beta[j];
            int kk = 0;
            for (int k = 0; k < GM_RESTART; ++k) {
                const double* Vk = w.gV + (size_t)k * nrhs * n;
                // w = M^{-1} A V_k (A V_k summed into w.R, free until the next residual)
                MG_TRY(launch_av(Vk, n));
                MG_TRY(reduce_av(w.R));
                MG_TRY(precond(w.R, w.gW));
                // classical Gram-Schmidt, twice
                for (int pass = 0; pass < 2; ++pass) {
                    MG_TRY(dots(w.gV, k + 1, w.gW));
                    for (int i = 0; i <= k; ++i)
                        for (int j = 0; j < nrhs; ++j) Hat(j, i, k) += coef[i * nrhs + j];
                    MG_TRY(upload((k + 1) * nrhs));
                    gs_update_kernel<<<egrid, 256, 0, st>>>(n, k + 1, nrhs, w.gV, w.gC, w.gW);
                    MG_TRY(mg::post_launch(h, "gs_update_kernel"));
                }
                MG_TRY(dots(w.gW, 1, w.gW));
                for (int j = 0; j < nrhs; ++j) {
                    const double hn1 = std::sqrt(coef[j]);
                    Hat(j, k + 1, k) = hn1;
                    coef[j] = hn1 > 0.0 ? 1.0 / hn1 : 0.0;
                }
                MG_TRY(upload(nrhs));
                gs_scale_kernel<<<egrid, 256, 0, st>>>(n, nrhs, w.gW, w.gC, w.gV + (size_t)(k + 1) * nrhs * n);
                MG_TRY(mg::post_launch(h, "gs_scale_kernel"));
                // Givens rotations of column k of each column's Hessenberg matrix
                bool done = true;
                for (int j = 0; j < nrhs; ++j) {
                    double* cj = cs.data() + (size_t)j * GM_RESTART;
                    double* sj = sn.data() + (size_t)j * GM_RESTART;
                    double* gj = g.data() + (size_t)j * (GM_RESTART + 1);
                    for (int i = 0; i < k; ++i) {
                        const double t = cj[i] * Hat(j, i, k) + sj[i] * Hat(j, i + 1, k);
                        Hat(j, i + 1, k) = -sj[i] * Hat(j, i, k) + cj[i] * Hat(j, i + 1, k);
                        Hat(j, i, k) = t;
                    }
                    const double a0 = Hat(j, k, k), b0 = Hat(j, k + 1, k), rho = std::hypot(a0, b0);
                    cj[k] = rho > 0.0 ? a0 / rho : 1.0;
                    sj[k] = rho > 0.0 ? b0 / rho : 0.0;
                    Hat(j, k, k) = rho;
                    Hat(j, k + 1, k) = 0.0;
                    gj[k + 1] = -sj[k] * gj[k];
                    gj[k] = cj[k] * gj[k];
                    if (std::fabs(gj[k + 1]) > kInnerTol * beta[j]) done = false;
                }
                kk = k + 1;
                if (done) break;
            }
            // y = H(0:kk, 0:kk)^{-1} g(0:kk) per column; x += V y
            for (int j = 0; j < nrhs; ++j) {
                const double* gj = g.data() + (size_t)j * (GM_RESTART + 1);
                for (int i = kk - 1; i >= 0; --i) {
                    double t = gj[i];
                    for (int l = i + 1; l < kk; ++l) t -= Hat(j, i, l) * coef[l * nrhs + j];
                    coef[i * nrhs + j] = Hat(j, i, i) != 0.0 ? t / Hat(j, i, i) : 0.0;
                }
            }
            MG_TRY(upload(kk * nrhs));
            gm_update_x_kernel<<<egrid, 256, 0, st>>>(n, kk, nrhs, w.gV, w.gC, X, ldx);
            MG_TRY(mg::post_launch(h, "gm_update_x_kernel"));
            r.gmres_iterations += kk;
        }
    }
    const auto t2 = clk::now();
    r.refine_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
    mg_status_t result = converged && r.path == 1 ? MG_FALLBACK_USED : MG_OK;
    if (!converged) {
        if (o.fallback) {
            int finfo = 0;
            mg_status_t fs = mg_dgesv(h, n, nrhs, A, lda, B, ldb, X, ldx, &finfo);
            if (fs != MG_OK) return fs;
            r.path = 2;
            result = MG_FALLBACK_USED;
        } else {
            result = mg::fail(h, MG_IR_STALLED, "refinement stalled at backward error %.3e", r.backward_error);
        }
    }
    MG_TRY(read_growth());
    if (rep) *rep = r;
    return result;
}

// R = B - A X on its own (the residual of the mixed solves): mode 0 the exact
// fixed-point integer form (FP64 when A or X holds an infinity or NaN),
// mode 1 FP64 FMA.  Synchronises (to read A's non-finite flag).
extern "C" mg_status_t mg_dresidual(mg_handle_t h, int n, int nrhs, const double* A, int lda, const double* X, int ldx,
                                    const double* B, int ldb, double* R, int ldr, int mode) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || nrhs < 0 || nrhs > MAX_RHS || lda < std::max(1, n) || ldx < std::max(1, n) ||
        ldb < std::max(1, n) || ldr < std::max(1, n) || (mode != 0 && mode != 1))
        return mg::fail(h, MG_ERR_ARG, "mg_dresidual: bad sizes or mode (nrhs <= %d)", MAX_RHS);
    if (n == 0 || nrhs == 0) return MG_OK;
    if (!A || !X || !B || !R) return mg::fail(h, MG_ERR_ARG, "mg_dresidual: null pointer");
    const int kch = (n + RES_KCHUNK - 1) / RES_KCHUNK;
    const int ri_chunk = resint_kchunk(n, h->num_sms);
    const int ri_kch = (n + ri_chunk - 1) / ri_chunk;
    const size_t opart = 0;
    const size_t orexp = mg::align_up((size_t)std::max(kch, RI_CLASSES * ri_kch) * nrhs * n * sizeof(double), 1024);
    const size_t oflag = mg::align_up(orexp + (size_t)n * sizeof(int), 1024);
    const size_t onorm = oflag + 1024;
    const size_t oxd = onorm + 1024;
    MG_TRY(mg::ensure_ws(h, oxd + xdig_bytes(n, nrhs)));
    MG_TRY(mg::ensure_hws(h, 64));
    char* b = (char*)h->ws;
    double* partial = (double*)(b + opart);
    long long* ipart = (long long*)(b + opart);
    int* rexp = (int*)(b + orexp);
    int* flags = (int*)(b + oflag);  // [0] A non-finite, [1] X non-finite, [8..16) column exponents
    double* norms = (double*)(b + onorm);
    int* xdig = (int*)(b + oxd);
    const cudaStream_t st = h->stream;
    bool int_res = mode == 0;
    if (int_res) {
        MG_CHECK_CUDA(h, cudaMemsetAsync(rexp, 0, (size_t)n * sizeof(int), st));
        MG_CHECK_CUDA(h, cudaMemsetAsync(flags, 0, 16 * sizeof(int), st));
        rowexp_kernel<<<dim3((n + 255) / 256, (n + 255) / 256), 256, 0, st>>>(A, lda, n, rexp, flags);
        MG_TRY(mg::post_launch(h, "rowexp_kernel"));
        int* hf = (int*)h->hws;
        MG_CHECK_CUDA(h, cudaMemcpyAsync(hf, flags, sizeof(int), cudaMemcpyDeviceToHost, st));
        MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
        int_res = hf[0] == 0;
    }
    MG_CHECK_CUDA(h, cudaMemsetAsync(norms, 0, 16 * sizeof(double), st));
    if (int_res) {
        colexp_kernel<<<dim3(std::min(64, (n + 255) / 256), nrhs), 256, 0, st>>>(X, ldx, n, nrhs, flags + 8, flags + 1);
        MG_TRY(mg::post_launch(h, "colexp_kernel"));
        const dim3 g((n + RI_ROWS - 1) / RI_ROWS, ri_kch);
        xdigits_kernel<<<std::max(1, std::min(h->num_sms * 8, (n * nrhs + 255) / 256)), 256, 0, st>>>(X, ldx, n, nrhs,
                                                                                                     flags + 8, xdig);
        MG_TRY(mg::post_launch(h, "xdigits_kernel"));
        MG_CHECK_CUDA(h, launch_resint(0, nrhs, g, st, A, lda, nullptr, n, n, xdig, ri_chunk, rexp, ipart));
        MG_TRY(mg::post_launch(h, "residual_int_kernel"));
        residual_int_reduce_kernel<<<(n + 255) / 256, 256, 0, st>>>(ipart, ri_kch, n, nrhs, rexp, flags + 8,
                                                                   flags + 1, B, ldb, X, ldx, R, ldr, norms);
        return mg::post_launch(h, "residual_int_reduce_kernel");
    }
    const dim3 rgrid((n + RES_ROWS - 1) / RES_ROWS, kch);
    switch (nrhs) {
#define MG_RES(NRV) \
    case NRV: residual_partial_kernel<NRV><<<rgrid, RES_ROWS, 0, st>>>(A, lda, n, X, ldx, partial); break;
        MG_RES(1) MG_RES(2) MG_RES(3) MG_RES(4) MG_RES(5) MG_RES(6) MG_RES(7)
        default: residual_partial_kernel<8><<<rgrid, RES_ROWS, 0, st>>>(A, lda, n, X, ldx, partial); break;
#undef MG_RES
    }
    MG_TRY(mg::post_launch(h, "residual_partial_kernel"));
    residual_reduce_kernel<<<(n + 255) / 256, 256, 0, st>>>(partial, kch, n, nrhs, B, ldb, X, ldx, R, ldr, norms);
    return mg::post_launch(h, "residual_reduce_kernel");
}

extern "C" mg_status_t mg_dsgesv_ir(mg_handle_t h, int n, int nrhs, const double* A, int lda, const double* B,
                                    int ldb, double* X, int ldx, const mg_ir_opts* opts, mg_ir_report* rep) {
    return mixed_solve(h, n, nrhs, A, lda, B, ldb, X, ldx, opts, rep, MixedKind::LU);
}

extern "C" mg_status_t mg_dsposv_ir(mg_handle_t h, int n, int nrhs, const double* A, int lda, const double* B,
                                    int ldb, double* X, int ldx, const mg_ir_opts* opts, mg_ir_report* rep) {
    return mixed_solve(h, n, nrhs, A, lda, B, ldb, X, ldx, opts, rep, MixedKind::SPD);
}

extern "C" mg_status_t mg_dsqrsv_ir(mg_handle_t h, int n, int nrhs, const double* A, int lda, const double* B,
                                    int ldb, double* X, int ldx, const mg_ir_opts* opts, mg_ir_report* rep) {
    return mixed_solve(h, n, nrhs, A, lda, B, ldb, X, ldx, opts, rep, MixedKind::QR);
}
