// FP32 GEMM C = alpha op(A) op(B) + beta C (SIMT FFMA), for the FP32 forms
// of the Cholesky, its adjoint and the Gaussian-process gradient, and for
// Mat's operator* on MAT<float> (Mul/Mul.h:204-235, the float template).
//
// 128 x 128 CTA tile, K step 8, 256 threads each accumulating an 8 x 8 block
// (rows ty*4 + {0..3} and 64 + ty*4 + {0..3}, columns likewise from tx, so the
// shared-memory reads of a warp are broadcasts or conflict-free float4s).
// The next K step is loaded into registers while the current one is
// multiplied, then stored to the other shared buffer.  `tri` computes only
// the tiles that meet the lower triangle (row >= column somewhere in the
// tile): the Cholesky trailing update and tril(.) accumulations, whose strict
// upper triangle is never read.
#include "mg_internal.cuh"

namespace {

constexpr int SB_M = 128, SB_N = 128, SB_K = 8, SB_T = 256;

template <int TA, int TB>
__global__ void __launch_bounds__(SB_T) sgemm_kernel(int m, int n, int k, float alpha, const float* __restrict__ A,
                                                     int lda, const float* __restrict__ B, int ldb, float beta,
                                                     float* __restrict__ C, int ldc, int tri) {
    __shared__ __align__(16) float As[2][SB_K][SB_M];
    __shared__ __align__(16) float Bs[2][SB_K][SB_N];
    const int m0 = blockIdx.x * SB_M, n0 = blockIdx.y * SB_N;
    if (tri && m0 + SB_M - 1 < n0) return;  // tile strictly above the diagonal
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;

    // loader mapping: 1024 elements of each tile, 4 per thread
    // A (not transposed): element (i, kk) = A[i + kk*lda]: consecutive i per thread group
    // A (transposed):     element (i, kk) = A[kk + i*lda]: consecutive kk
    float ra[4], rb[4];
    auto load = [&](int k0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + q * SB_T;
            int i, kk;
            if (TA) {
                kk = e & 7;
                i = e >> 3;
            } else {
                i = e & 127;
                kk = e >> 7;
            }
            const int gi = m0 + i, gk = k0 + kk;
            ra[q] = (gi < m && gk < k) ? (TA ? A[gk + (size_t)gi * lda] : A[gi + (size_t)gk * lda]) : 0.f;
            int j, kb;
            if (TB) {
                j = e & 127;
                kb = e >> 7;
            } else {
                kb = e & 7;
                j = e >> 3;
            }
            const int gj = n0 + j, gkb = k0 + kb;
            rb[q] = (gj < n && gkb < k) ? (TB ? B[gj + (size_t)gkb * ldb] : B[gkb + (size_t)gj * ldb]) : 0.f;
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + q * SB_T;
            if (TA)
                As[buf][e & 7][e >> 3] = ra[q];
            else
                As[buf][e >> 7][e & 127] = ra[q];
            if (TB)
                Bs[buf][e >> 7][e & 127] = rb[q];
            else
                Bs[buf][e & 7][e >> 3] = rb[q];
        }
    };

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

    load(0);
    store(0);
    __syncthreads();
    int buf = 0;
    for (int k0 = 0; k0 < k; k0 += SB_K) {
        const bool more = k0 + SB_K < k;
        if (more) load(k0 + SB_K);
#pragma unroll
        for (int kk = 0; kk < SB_K; ++kk) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][64 + ty * 4]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][64 + tx * 4]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        if (more) {
            store(buf ^ 1);
            __syncthreads();
            buf ^= 1;
        }
    }

#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int gi = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
        if (gi >= m) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int gj = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
            if (gj >= n) continue;
            float* cp = C + gi + (size_t)gj * ldc;
            *cp = beta == 0.f ? alpha * acc[i][j] : fmaf(alpha, acc[i][j], beta * *cp);
        }
    }
}

__global__ void sscale_kernel(int m, int n, float beta, float* __restrict__ C, int ldc) {
    const size_t total = (size_t)m * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        float* cp = C + (e % m) + (e / m) * ldc;
        *cp = beta == 0.f ? 0.f : beta * *cp;
    }
}

}  // namespace

namespace mg {

mg_status_t sgemm_launch(mg_handle_t h, int transA, int transB, int m, int n, int k, float alpha, const float* A,
                         int lda, const float* B, int ldb, float beta, float* C, int ldc, int tri) {
    if (m == 0 || n == 0) return MG_OK;
    cudaStream_t st = h->stream;
    if (k == 0 || alpha == 0.f) {
        if (beta == 1.f) return MG_OK;
        sscale_kernel<<<h->num_sms * 4, 256, 0, st>>>(m, n, beta, C, ldc);
        return post_launch(h, "sscale_kernel");
    }
    ProfScope prof(h, "sgemm_f32", (tri ? 1.0 : 2.0) * m * (double)n * k,
                   4.0 * ((double)m * k + (double)k * n + (beta == 0.f ? 1.0 : 2.0) * m * n));
    const dim3 grid((m + SB_M - 1) / SB_M, (n + SB_N - 1) / SB_N);
    if (transA && transB)
        sgemm_kernel<1, 1><<<grid, SB_T, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri);
    else if (transA)
        sgemm_kernel<1, 0><<<grid, SB_T, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri);
    else if (transB)
        sgemm_kernel<0, 1><<<grid, SB_T, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri);
    else
        sgemm_kernel<0, 0><<<grid, SB_T, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri);
    return post_launch(h, "sgemm_kernel");
}

namespace {

int tc_slot(mg_handle_t h) { return h->stream && h->stream == h->la_stream ? 1 : h->stream && h->stream == h->pp_stream ? 2 : 0; }

// Grows the split area of `slot` to `bytes`.  A growth waits for the whole
// device: the area may be in use on any of the handle's streams.
mg_status_t ensure_tcws(mg_handle_t h, int slot, size_t bytes) {
    if (!h->tcerr) {
        if (cudaMalloc((void**)&h->tcerr, 3 * 64 * sizeof(int)) != cudaSuccess) {
            h->tcerr = nullptr;
            return fail(h, MG_ERR_ALLOC, "tensor-core GEMM error words: cudaMalloc failed");
        }
        MG_CHECK_CUDA(h, cudaMemset(h->tcerr, 0, 3 * 64 * sizeof(int)));
    }
    if (bytes <= h->tcws_bytes[slot]) return MG_OK;
    bytes = align_up(bytes + (bytes >> 3), 1 << 20);
    if (h->tcws[slot]) {
        MG_CHECK_CUDA(h, cudaDeviceSynchronize());
        MG_CHECK_CUDA(h, cudaFree(h->tcws[slot]));
        h->tcws[slot] = nullptr;
        h->tcws_bytes[slot] = 0;
    }
    if (cudaMalloc(&h->tcws[slot], bytes) != cudaSuccess) {
        h->tcws[slot] = nullptr;
        return fail(h, MG_ERR_ALLOC, "tensor-core GEMM area cudaMalloc(%zu) failed", bytes);
    }
    h->tcws_bytes[slot] = bytes;
    return MG_OK;
}

}  // namespace

mg_status_t sgemm_auto(mg_handle_t h, int ta, int tb, int m, int n, int k, float alpha, const float* A, int lda,
                       const float* B, int ldb, float beta, float* C, int ldc, int tri) {
    if (k < 32 || (double)m * n * k < (double)(1 << 24) || alpha == 0.f)
        return sgemm_launch(h, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri);
    constexpr int np = 3;
    const size_t as = align_up(bf16x_split_bytes(m, k, np), 1024), bs = align_up(bf16x_split_bytes(n, k, np), 1024);
    const int slot = tc_slot(h);
    MG_TRY(ensure_tcws(h, slot, as + bs));
    char* base = (char*)h->tcws[slot];
    int* err = h->tcerr + 64 * slot;
    // op(A) rows as split rows: A itself (ta = 0) or the columns of A (ta = 1);
    // op(B) columns as split rows: the columns of B (tb = 0) or its rows (tb = 1)
    MG_TRY(bf16x_split<float>(h, ta == 0, A, lda, m, k, np, base));
    MG_TRY(bf16x_split<float>(h, tb != 0, B, ldb, n, k, np, base + as));
    // Few output tiles over a long K (the mixed QR's V^T C: 128 rows): split
    // K so that the whole GPU works, each slice adding into C (cleared first
    // when beta = 0), with at least 8 k-blocks of 32 per slice
    const int tiles = ((m + 127) / 128) * ((n + 255) / 256), kblk = (k + 31) / 32;
    int ksplit = 1;
    if ((beta == 0.f || beta == 1.f) && ((uintptr_t)C & 15) == 0 && (ldc & 3) == 0 && 2 * tiles <= h->num_sms) {
        ksplit = h->num_sms / tiles;
        if (ksplit > kblk / 8) ksplit = kblk / 8;
        if (ksplit < 2) ksplit = 1;
    }
    if (ksplit > 1) {
        if (beta == 0.f)
            MG_CHECK_CUDA(h, cudaMemset2DAsync(C, (size_t)ldc * sizeof(float), 0, (size_t)m * sizeof(float), n,
                                               h->stream));
        return bf16x_gemm_presplit(h, np, m, n, k, alpha, base, base + as, 1.0f, C, ldc, err, 0, 0, 0, true, true,
                                   false, true, ksplit);
    }
    return bf16x_gemm_presplit(h, np, m, n, k, alpha, base, base + as, beta, C, ldc, err, 0, 0, 0, true, true, false,
                               true);
}

mg_status_t tc_sgemm_error(mg_handle_t h, int* err_out) {
    *err_out = 0;
    if (!h->tcerr) return MG_OK;
    int e[3 * 64];
    MG_CHECK_CUDA(h, cudaMemcpyAsync(e, h->tcerr, sizeof(e), cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    *err_out = e[0] | e[64] | e[128];
    return MG_OK;
}

}  // namespace mg

extern "C" mg_status_t mg_sgemm(mg_handle_t h, int transA, int transB, int m, int n, int k, float alpha,
                                const float* A, int lda, const float* B, int ldb, float beta, float* C, int ldc) {
    if (!h) return MG_ERR_ARG;
    if (m < 0 || n < 0 || k < 0) return mg::fail(h, MG_ERR_ARG, "mg_sgemm: negative size (%d,%d,%d)", m, n, k);
    const int arows = transA ? k : m, brows = transB ? n : k;
    if (lda < (arows > 1 ? arows : 1) || ldb < (brows > 1 ? brows : 1) || ldc < (m > 1 ? m : 1))
        return mg::fail(h, MG_ERR_ARG, "mg_sgemm: leading dimension too small");
    if (m && n && ((!C) || (k && (!A || !B)))) return mg::fail(h, MG_ERR_ARG, "mg_sgemm: null pointer");
    return mg::sgemm_launch(h, transA, transB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, 0);
}
