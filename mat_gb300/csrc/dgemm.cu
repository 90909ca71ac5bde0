// FP64 GEMM for sm_103a: C = alpha * op(A) * op(B) + beta * C, column-major.
//
// Replaces Mat's packed GEMM engine: the dispatcher operator* (Mat-8.3.1/Mul/
// Mul.h:204-235), the blocked driver __mulAB_2 (Mul.h:155-202), the packers
// (Mul/__pack_double.h) and the AVX-512 16x12 register micro-kernel
// (Mul/__micro_kernel_packed_double.h:14-110), and the subtracting trailing
// updates __mulAB_packed_n / _lower_tri_ / _upper_tri_ (Mul.h:240-322).
//
// Design.  tcgen05 has no f64 kind, so FP64 products run on the FP64 MMA
// path (mma.sync m16n8k4 .f64, "DMMA").  On GB300 the FP64 rate is a few
// flops per clock per SM, far below what HBM and shared memory can feed, so
// the kernel is built to keep the DMMA pipe busy with the least issue
// overhead: a 128x128 CTA tile, 8 warps with a 64x32 warp tile (16
// independent MMAs per k-step), a 3-stage cp.async ring into padded shared
// memory (strides chosen so fragment loads are bank-conflict free), and
// zero-filled copies for the ragged M/N/K edges so the main loop has no edge
// code.  The copies are 8-byte cp.async so any leading dimension and any
// sub-matrix offset works (Mat's ld = rows is often odd).
#include "mg_internal.cuh"

namespace {

constexpr int BM = 128, BN = 128, BK = 16;
constexpr int SA = BM + 4;  // sA[k][m], stride = 4 (mod 16) doubles
constexpr int SB = BK + 4;  // sB[n][k]
constexpr int STAGES = 3;
constexpr int THREADS = 256;
constexpr int STAGE_DOUBLES = BK * SA + BN * SB;
constexpr size_t SMEM_BYTES = (size_t)STAGES * STAGE_DOUBLES * sizeof(double);

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
template <int TA, int TB>
__device__ __forceinline__ void load_stage(double* sA, double* sB, const double* __restrict__ A, int lda,
                                           const double* __restrict__ B, int ldb, int M, int N, int K,
                                           int bm, int bn, int k0, int tid) {
    // op(A)(m,k): TA=0 -> A[m + k*lda], TA=1 -> A[k + m*lda]
    if (TA == 0) {
        const int m = tid % BM, kk = tid / BM;  // 2 k-rows per pass
        const int gm = bm + m;
#pragma unroll
        for (int j = 0; j < BK / 2; ++j) {
            const int k = kk + 2 * j, gk = k0 + k;
            const bool p = gm < M && gk < K;
            cp_async8(sA + k * SA + m, p ? A + gm + (size_t)gk * lda : A, p);
        }
    } else {
        const int k = tid % BK, mm = tid / BK;  // 16 m per pass
        const int gk = k0 + k;
#pragma unroll
        for (int j = 0; j < BM / 16; ++j) {
            const int m = mm + 16 * j, gm = bm + m;
            const bool p = gm < M && gk < K;
            cp_async8(sA + k * SA + m, p ? A + gk + (size_t)gm * lda : A, p);
        }
    }
    // op(B)(k,n): TB=0 -> B[k + n*ldb], TB=1 -> B[n + k*ldb]
    if (TB == 0) {
        const int k = tid % BK, nn = tid / BK;
        const int gk = k0 + k;
#pragma unroll
        for (int j = 0; j < BN / 16; ++j) {
            const int n = nn + 16 * j, gn = bn + n;
            const bool p = gn < N && gk < K;
            cp_async8(sB + n * SB + k, p ? B + gk + (size_t)gn * ldb : B, p);
        }
    } else {
        const int n = tid % BN, kk = tid / BN;
        const int gn = bn + n;
#pragma unroll
        for (int j = 0; j < BK / 2; ++j) {
            const int k = kk + 2 * j, gk = k0 + k;
            const bool p = gn < N && gk < K;
            cp_async8(sB + n * SB + k, p ? B + gn + (size_t)gk * ldb : B, p);
        }
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
template <int TA, int TB, int MODE, int TRI>
__global__ void __launch_bounds__(THREADS, 1)
    dgemm_kernel(int M, int N, int K, double alpha, const double* __restrict__ A, int lda,
                 const double* __restrict__ B, int ldb, double beta, double* __restrict__ C, int ldc) {
    extern __shared__ __align__(16) double smem[];
    const int tid = threadIdx.x;
    const int bm = blockIdx.x * BM, bn = blockIdx.y * BN;
    if (TRI && bm + BM - 1 < bn) return;

    const int warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    const int wm = (warp & 1) * 64;   // 2 warps along M
    const int wn = (warp >> 1) * 32;  // 4 warps along N

    double acc[4][4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
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
            double* st = smem + s * STAGE_DOUBLES;
            load_stage<TA, TB>(st, st + BK * SA, A, lda, B, ldb, M, N, K, bm, bn, s * BK, tid);
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
                double* st = smem + (nk % STAGES) * STAGE_DOUBLES;
                load_stage<TA, TB>(st, st + BK * SA, A, lda, B, ldb, M, N, K, bm, bn, nk * BK, tid);
            }
            cp_async_commit();
        }
        const double* sA = smem + (kt % STAGES) * STAGE_DOUBLES;
        const double* sB = sA + BK * SA;
#pragma unroll
        for (int ks = 0; ks < BK; ks += 4) {
            double a[4][2], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                a[i][0] = sA[(ks + t) * SA + wm + 16 * i + g];
                a[i][1] = sA[(ks + t) * SA + wm + 16 * i + g + 8];
                if (MODE == 1) {
                    a[i][0] = -a[i][0];
                    a[i][1] = -a[i][1];
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = sB[(wn + 8 * j + g) * SB + ks + t];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) dmma_16x8x4(acc[i][j], a[i][0], a[i][1], b[j]);
        }
    }
    cp_async_wait<0>();

    // Epilogue: c0,c1 -> (g, 2t..2t+1), c2,c3 -> (g+8, 2t..2t+1) of each 16x8 fragment.
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
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

template <int TA, int TB, int MODE, int TRI>
cudaError_t launch_t(cudaStream_t st, int M, int N, int K, double alpha, const double* A, int lda,
                     const double* B, int ldb, double beta, double* C, int ldc) {
    auto kern = dgemm_kernel<TA, TB, MODE, TRI>;
    static bool configured = false;  // per instantiation
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN);
    kern<<<grid, THREADS, SMEM_BYTES, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
    return cudaGetLastError();
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
    const int mode = beta == 0.0                    ? 0
                     : (alpha == -1.0 && beta == 1.0) ? 1
                     : (alpha == 1.0 && beta == 1.0)  ? 2
                                                      : 3;
    cudaError_t e;
#define MG_MODE(TA, TB, MODE)                                                                \
    e = tri ? launch_t<TA, TB, MODE, 1>(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc)    \
            : launch_t<TA, TB, MODE, 0>(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
#define MG_DISPATCH(TA, TB)          \
    switch (mode) {                  \
        case 0: MG_MODE(TA, TB, 0) break; \
        case 1: MG_MODE(TA, TB, 1) break; \
        case 2: MG_MODE(TA, TB, 2) break; \
        default: MG_MODE(TA, TB, 3) break; \
    }
    if (!transA && !transB) {
        MG_DISPATCH(0, 0)
    } else if (transA && !transB) {
        MG_DISPATCH(1, 0)
    } else if (!transA && transB) {
        MG_DISPATCH(0, 1)
    } else {
        MG_DISPATCH(1, 1)
    }
#undef MG_MODE
#undef MG_DISPATCH
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
