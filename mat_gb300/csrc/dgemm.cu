// FP64 GEMM for sm_103a: C = alpha * op(A) * op(B) + beta * C, column-major.
//
// Replaces Mat's packed GEMM engine: the dispatcher operator* (Mat-8.3.1/Mul/
// Mul.h:204-235), the blocked driver __mulAB_2 (Mul.h:155-202), the packers
// (Mul/__pack_double.h) and the AVX-512 16x12 register micro-kernel
// (Mul/__micro_kernel_packed_double.h:14-110), and the subtracting trailing
// updates __mulAB_packed_n / _lower_tri_ / _upper_tri_ (Mul.h:240-322).
//
// Design.  tcgen05 has no f64 kind, so FP64 products run on the FP64 MMA
// path (mma.sync m16n8k4 .f64, "DMMA").  On GB300 the FP64 rate is about two
// fused multiply-adds per clock per SM, far below what HBM and shared memory
// can feed, so the kernel is built to keep the DMMA pipe busy: warps with
// 8-16 independent MMAs per k-step, a 3-stage cp.async ring into padded
// shared memory (strides chosen so fragment loads are bank-conflict free),
// and zero-filled copies for the ragged M/N/K edges so the main loop has no
// edge code.  The copies are 8-byte cp.async so any leading dimension and
// any sub-matrix offset works (Mat's ld = rows is often odd).
//
// Every output element is one fused chain over k = 0..K-1 in order (the
// DMMA k-step accumulates its four products in k order), starting from 0 or
// from C in the in-place modes: exactly the per-element operation sequence
// of Mat's micro-kernels, so results are bit-identical to Mat's operator*.
// K is therefore never split across CTAs; small problems use a 32x32 tile
// (one warp, up to 7 CTAs per SM) so the GPU is still filled.
#include <algorithm>

#include "mg_internal.cuh"

namespace {

constexpr int BK = 16;
constexpr int STAGES = 3;
constexpr int SB = BK + 4;  // sB[n][k] stride = 4 (mod 16) doubles

// Tile configuration: WM x WN warps, each holding MI x NJ fragments of 16x8.
template <int WM_, int WN_, int MI_, int NJ_>
struct TileCfg {
    static constexpr int WM = WM_, WN = WN_, MI = MI_, NJ = NJ_;
    static constexpr int THREADS = WM * WN * 32;
    static constexpr int BM = WM * MI * 16;
    static constexpr int BN = WN * NJ * 8;
    static constexpr int SA = BM + 4;  // sA[k][m], stride = 4 (mod 16) doubles
    static constexpr int STAGE_DOUBLES = BK * SA + BN * SB;
    static constexpr size_t SMEM = (size_t)STAGES * STAGE_DOUBLES * sizeof(double);
    static_assert((BM * BK) % THREADS == 0 && (BN * BK) % THREADS == 0, "loader split");
};
using Big = TileCfg<2, 4, 4, 4>;    // 128 x 128, 8 warps
using Small = TileCfg<1, 1, 2, 4>;  // 32 x 32, 1 warp
using Thin = TileCfg<1, 1, 3, 2>;   // 48 x 16, 1 warp: M = 48 block-reflector products (QR, adjoint)
// 16 x 16, 1 warp: products with few outputs and a moderate K; the small
// tile spreads the outputs over more SMs.  (An SM takes a DMMA about every
// 270 cycles, but through four sub-partition pipes of about 1,100 cycles each:
// a lone warp per SM keeps only one of them issuing.)
using Tiny = TileCfg<1, 1, 1, 2>;
// 16 x 32, 4 warps of one 16x8 accumulator each: products with few rows and
// a long K (W = V^T R2 of the QR, M = 48, K = the panel height).  Each
// accumulator is one fused K chain; spreading the chains over four warps per
// CTA keeps every sub-partition's FP64 pipe issuing, where the 1-warp tiles
// left two or three of an SM's four idle.
using Quad = TileCfg<1, 4, 1, 1>;

__device__ __forceinline__ void cp_async8(double* smem, const double* gmem, bool pred) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int n = pred ? 8 : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ void dmma_16x8x4(double (&c)[4], double a0, double a1, double b0) {
    asm volatile(
        "mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, "
        "{%0,%1,%2,%3};\n"
        : "+d"(c[0]), "+d"(c[1]), "+d"(c[2]), "+d"(c[3])
        : "d"(a0), "d"(a1), "d"(b0));
}

// Loads one BK slice of op(A) (rows bm.., k-columns k0..) and op(B) into a stage.
template <class CF, int TA, int TB>
__device__ __forceinline__ void load_stage(double* sA, double* sB, const double* __restrict__ A, int lda,
                                           const double* __restrict__ B, int ldb, int M, int N, int K, int bm,
                                           int bn, int k0, int tid) {
    constexpr int NA = CF::BM * BK / CF::THREADS, NB = CF::BN * BK / CF::THREADS;
#pragma unroll
    for (int j = 0; j < NA; ++j) {
        const int e = tid + j * CF::THREADS;
        // op(A)(m,k): TA=0 -> A[m + k*lda] (coalesce over m), TA=1 -> A[k + m*lda] (over k)
        const int m = TA == 0 ? e % CF::BM : e / BK;
        const int k = TA == 0 ? e / CF::BM : e % BK;
        const int gm = bm + m, gk = k0 + k;
        const bool p = gm < M && gk < K;
        const double* src = TA == 0 ? A + gm + (size_t)gk * lda : A + gk + (size_t)gm * lda;
        cp_async8(sA + k * CF::SA + m, p ? src : A, p);
    }
#pragma unroll
    for (int j = 0; j < NB; ++j) {
        const int e = tid + j * CF::THREADS;
        // op(B)(k,n): TB=0 -> B[k + n*ldb] (over k), TB=1 -> B[n + k*ldb] (over n)
        const int k = TB == 0 ? e % BK : e / CF::BN;
        const int n = TB == 0 ? e / BK : e % CF::BN;
        const int gn = bn + n, gk = k0 + k;
        const bool p = gn < N && gk < K;
        const double* src = TB == 0 ? B + gk + (size_t)gn * ldb : B + gn + (size_t)gk * ldb;
        cp_async8(sB + n * SB + k, p ? src : B, p);
    }
}

// MODE selects how the accumulators meet C (Mat's micro-kernels load C and
// fuse every product into it, Mul/__micro_kernel_packed_double.h:14-110,
// :301-398, so the in-place modes keep that per-element chain):
//   0: acc = 0,  C = alpha*acc            (beta == 0; operator*)
//   1: acc = C,  acc -= A*B, C = acc      (alpha == -1, beta == 1; __mulAB_packed_n)
//   2: acc = C,  acc += A*B, C = acc      (alpha == 1, beta == 1)
//   3: acc = 0,  C = alpha*acc + beta*C   (general)
// TRI = 1: only tiles containing elements with row >= col are computed.
template <class CF, int TA, int TB, int MODE, int TRI>
__global__ void __launch_bounds__(CF::THREADS)
    dgemm_kernel(int M, int N, int K, double alpha, const double* __restrict__ A, int lda,
                 const double* __restrict__ B, int ldb, double beta, double* __restrict__ C, int ldc) {
    extern __shared__ __align__(16) double smem[];
    constexpr int MI = CF::MI, NJ = CF::NJ;
    const int tid = threadIdx.x;
    const int bm = blockIdx.x * CF::BM, bn = blockIdx.y * CF::BN;
    if (TRI && bm + CF::BM - 1 < bn) return;

    const int warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    const int wm = (warp % CF::WM) * (MI * 16);
    const int wn = (warp / CF::WM) * (NJ * 8);

    double acc[MI][NJ][4];
#pragma unroll
    for (int i = 0; i < MI; ++i)
#pragma unroll
        for (int j = 0; j < NJ; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                double v = 0.0;
                if (MODE == 1 || MODE == 2) {
                    const int row = bm + wm + 16 * i + g + (r >= 2 ? 8 : 0);
                    const int col = bn + wn + 8 * j + 2 * t + (r & 1);
                    if (row < M && col < N) v = C[row + (size_t)col * ldc];
                }
                acc[i][j][r] = v;
            }

    const int ktiles = (K + BK - 1) / BK;
#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < ktiles) {
            double* st = smem + s * CF::STAGE_DOUBLES;
            load_stage<CF, TA, TB>(st, st + BK * CF::SA, A, lda, B, ldb, M, N, K, bm, bn, s * BK, tid);
        }
        cp_async_commit();
    }

    for (int kt = 0; kt < ktiles; ++kt) {
        cp_async_wait<STAGES - 2>();
        __syncthreads();
        // Prefetch the stage STAGES-1 ahead (its buffer was consumed at kt-1).
        {
            const int nk = kt + STAGES - 1;
            if (nk < ktiles) {
                double* st = smem + (nk % STAGES) * CF::STAGE_DOUBLES;
                load_stage<CF, TA, TB>(st, st + BK * CF::SA, A, lda, B, ldb, M, N, K, bm, bn, nk * BK, tid);
            }
            cp_async_commit();
        }
        const double* sA = smem + (kt % STAGES) * CF::STAGE_DOUBLES;
        const double* sB = sA + BK * CF::SA;
#pragma unroll
        for (int ks = 0; ks < BK; ks += 4) {
            double a[MI][2], b[NJ];
#pragma unroll
            for (int i = 0; i < MI; ++i) {
                a[i][0] = sA[(ks + t) * CF::SA + wm + 16 * i + g];
                a[i][1] = sA[(ks + t) * CF::SA + wm + 16 * i + g + 8];
                if (MODE == 1) {
                    a[i][0] = -a[i][0];
                    a[i][1] = -a[i][1];
                }
            }
#pragma unroll
            for (int j = 0; j < NJ; ++j) b[j] = sB[(wn + 8 * j + g) * SB + ks + t];
#pragma unroll
            for (int i = 0; i < MI; ++i)
#pragma unroll
                for (int j = 0; j < NJ; ++j) dmma_16x8x4(acc[i][j], a[i][0], a[i][1], b[j]);
        }
    }
    cp_async_wait<0>();

    // Epilogue: c0,c1 -> (g, 2t..2t+1), c2,c3 -> (g+8, 2t..2t+1) of each 16x8 fragment.
#pragma unroll
    for (int i = 0; i < MI; ++i) {
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int row = bm + wm + 16 * i + g + (r >= 2 ? 8 : 0);
                const int col = bn + wn + 8 * j + 2 * t + (r & 1);
                if (row < M && col < N) {
                    double* cp = C + row + (size_t)col * ldc;
                    if (MODE == 1 || MODE == 2) {
                        *cp = acc[i][j][r];
                    } else {
                        const double v = alpha * acc[i][j][r];
                        *cp = MODE == 0 ? v : fma(beta, *cp, v);
                    }
                }
            }
        }
    }
}

template <class CF, int TA, int TB, int MODE, int TRI>
cudaError_t launch_t(cudaStream_t st, int M, int N, int K, double alpha, const double* A, int lda, const double* B,
                     int ldb, double beta, double* C, int ldc) {
    auto kern = dgemm_kernel<CF, TA, TB, MODE, TRI>;
    static bool configured = false;  // per instantiation
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CF::SMEM);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    dim3 grid((M + CF::BM - 1) / CF::BM, (N + CF::BN - 1) / CF::BN);
    kern<<<grid, CF::THREADS, CF::SMEM, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
    return cudaGetLastError();
}

template <class CF>
cudaError_t dispatch(cudaStream_t st, int ta, int tb, int mode, int m, int n, int k, double alpha, const double* A,
                     int lda, const double* B, int ldb, double beta, double* C, int ldc) {
#define MG_MODE(TA, TB)                                                                              \
    switch (mode) {                                                                                  \
        case 0: return launch_t<CF, TA, TB, 0, 0>(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc); \
        case 1: return launch_t<CF, TA, TB, 1, 0>(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc); \
        case 2: return launch_t<CF, TA, TB, 2, 0>(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc); \
        default: return launch_t<CF, TA, TB, 3, 0>(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc); \
    }
    if (!ta && !tb) {
        MG_MODE(0, 0)
    } else if (ta && !tb) {
        MG_MODE(1, 0)
    } else if (!ta && tb) {
        MG_MODE(0, 1)
    } else {
        MG_MODE(1, 1)
    }
#undef MG_MODE
}

// Output area the busiest SM computes when `tiles` tiles of bm x bn are
// spread over the SMs.  On GB300 one warp with a few independent DMMA
// fragments already keeps an SM's FP64 pipe busy (the pipe retires about one
// m16n8k4 DMMA per ~290 cycles), so the time of a launch follows this area,
// not the tile's data reuse: thin operands (M = 48 in the QR and Cholesky
// adjoint updates) need small tiles to reach every SM.
double busiest_sm_area(long long tiles, int num_sms, int bm, int bn) {
    return (double)((tiles + num_sms - 1) / num_sms) * bm * bn;
}

// Scales C by beta (K == 0 or alpha == 0 cases).
__global__ void scale_kernel(int M, int N, double beta, double* C, int ldc) {
    const size_t total = (size_t)M * N;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t r = e % M, c = e / M;
        double* p = C + r + c * (size_t)ldc;
        *p = beta == 0.0 ? 0.0 : beta * *p;
    }
}

}  // namespace

namespace mg {

mg_status_t dgemm_launch(mg_handle_t h, int transA, int transB, int m, int n, int k, double alpha,
                         const double* A, int lda, const double* B, int ldb, double beta, double* C, int ldc,
                         int tri) {
    if (m == 0 || n == 0) return MG_OK;
    cudaStream_t st = h->stream;
    if (k == 0 || alpha == 0.0) {
        if (beta == 1.0) return MG_OK;
        scale_kernel<<<h->num_sms * 4, 256, 0, st>>>(m, n, beta, C, ldc);
        return post_launch(h, "scale_kernel");
    }
    const int mode = beta == 0.0                      ? 0
                     : (alpha == -1.0 && beta == 1.0) ? 1
                     : (alpha == 1.0 && beta == 1.0)  ? 2
                                                      : 3;
    cudaError_t e;
    ProfScope prof(h, "dgemm_f64", (tri ? 1.0 : 2.0) * m * (double)n * k,
                   8.0 * ((double)m * k + (double)k * n + (beta == 0.0 ? 1.0 : 2.0) * m * n));
    if (tri) {
        // Cholesky trailing update: C -= A * B^T on lower tiles only
        if (transA || !transB || mode != 1)
            return fail(h, MG_ERR_UNSUPPORTED, "dgemm_launch: triangular mode is C -= A*B^T only");
        auto lower_tiles = [&](int bm, int bn) {  // tiles meeting the lower triangle of the m x n block
            long long c = 0;
            for (int r0 = 0; r0 < m; r0 += bm) c += std::min<long long>((n + bn - 1) / bn, (r0 + bm - 1) / bn + 1);
            return c;
        };
        if (busiest_sm_area(lower_tiles(Big::BM, Big::BN), h->num_sms, Big::BM, Big::BN) <=
            busiest_sm_area(lower_tiles(Small::BM, Small::BN), h->num_sms, Small::BM, Small::BN))
            e = launch_t<Big, 0, 1, 1, 1>(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
        else
            e = launch_t<Small, 0, 1, 1, 1>(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    } else {
        const long long tb = (long long)((m + Big::BM - 1) / Big::BM) * ((n + Big::BN - 1) / Big::BN);
        const long long ts = (long long)((m + Small::BM - 1) / Small::BM) * ((n + Small::BN - 1) / Small::BN);
        const long long tt = (long long)((m + Thin::BM - 1) / Thin::BM) * ((n + Thin::BN - 1) / Thin::BN);
        const double ab = busiest_sm_area(tb, h->num_sms, Big::BM, Big::BN);
        const double as = busiest_sm_area(ts, h->num_sms, Small::BM, Small::BN);
        const double at = busiest_sm_area(tt, h->num_sms, Thin::BM, Thin::BN);
        const long long tn = (long long)((m + Tiny::BM - 1) / Tiny::BM) * ((n + Tiny::BN - 1) / Tiny::BN);
        const double an = busiest_sm_area(tn, h->num_sms, Tiny::BM, Tiny::BN);
        // the 16 x 16 tile reloads more operand bytes per flop: only when it
        // shortens the busiest SM's work clearly
        if (m <= 64 && k >= 2048)
            e = dispatch<Quad>(st, transA, transB, mode, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
        else if (an < 0.75 * std::min(at, std::min(ab, as)))
            e = dispatch<Tiny>(st, transA, transB, mode, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
        else if (at < ab && at < as)
            e = dispatch<Thin>(st, transA, transB, mode, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
        else if (ab <= as)
            e = dispatch<Big>(st, transA, transB, mode, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
        else
            e = dispatch<Small>(st, transA, transB, mode, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "dgemm_kernel launch");
    h->launches++;
    return MG_OK;
}

}  // namespace mg

extern "C" mg_status_t mg_dgemm(mg_handle_t h, int transA, int transB, int m, int n, int k, double alpha,
                                const double* A, int lda, const double* B, int ldb, double beta, double* C,
                                int ldc) {
    if (!h) return MG_ERR_ARG;
    if (m < 0 || n < 0 || k < 0)
        return mg::fail(h, MG_ERR_ARG, "mg_dgemm: negative size (%d,%d,%d)", m, n, k);
    const int arows = transA ? k : m, brows = transB ? n : k;
    if (lda < (arows > 1 ? arows : 1) || ldb < (brows > 1 ? brows : 1) || ldc < (m > 1 ? m : 1))
        return mg::fail(h, MG_ERR_ARG, "mg_dgemm: leading dimension too small");
    if (m && n && ((!C) || (k && (!A || !B))))
        return mg::fail(h, MG_ERR_ARG, "mg_dgemm: null pointer");
    return mg::dgemm_launch(h, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, 0);
}
