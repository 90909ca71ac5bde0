// Split-BF16 GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// C (fp32, column-major) = alpha * sum_{(i,j) in S} A_i * B_j^T + beta * C
// where A = A_0 + A_1 + A_2 and B = B_0 + B_1 + B_2 are fp32 operands split
// into bf16 terms (A_0 = bf16(A), A_1 = bf16(A - A_0), ...).  With three terms
// and the six products of total order <= 2 the product carries ~24 bits, the
// accuracy of an fp32 GEMM; two terms / three products give ~16 bits; one
// term is a plain bf16 GEMM.  Accumulation is fp32 in tensor memory.
//
// This is the mixed-precision replacement for the trailing-matrix updates of
// Mat's blocked factorizations (__mulAB_packed_n, Mat-8.3.1/Mul/Mul.h:240-263)
// and the split-precision product of the benchmark configuration
// M=N=K=16384; Mat itself has no mixed-precision path.
//
// Kernel: persistent, one CTA per SM, warp-specialised:
//   warp 0      TMA producer: per k-block of 32 it loads every term of the
//               128-row A tile and the 256-row B tile (64-byte swizzle) into
//               one pipeline stage; one mbarrier per stage counts the bytes.
//   warp 1      allocates 512 TMEM columns (two 128x256 fp32 accumulators)
//               and one elected lane issues tcgen05.mma (M=128, N=256, K=16),
//               committing each stage back to the producer and each finished
//               tile to the epilogue.
//   warps 2-9   epilogue: tcgen05.ld the accumulator (each warp its 32 TMEM
//               lanes = 32 rows, warps w and w+4 the two halves of the
//               columns), apply alpha/beta, store C coalesced by column.  Two
//               accumulators let tile t+1's MMAs run under tile t's
//               epilogue; two warps per lane quarter keep twice the C loads
//               in flight, which the read-modify-write of C in a K = 128
//               trailing update needs to approach HBM speed.
// Every mbarrier wait is bounded; on a timeout the kernel records MG_TIMEOUT,
// drains its own outstanding copies/MMAs and frees TMEM before returning.
#include <cuda_bf16.h>

#include "mg_internal.cuh"
#include "tc_common.cuh"

namespace {

constexpr int BM = 128, BN = 256, BK = 32;  // BK * 2 B = 64 B = one swizzle row
constexpr int EPI_WARPS = 8;  // two per TMEM lane quarter, each half of the tile's columns
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr int TMEM_COLS = 512;

// RED: the epilogue adds alpha * (A B) into C with TMA reductions (beta = 1)
// from two 32 x 32 staging buffers per epilogue warp, which take the shared
// memory of one or more operand stages.
template <int NP, bool RED = false>
struct Cfg {
    static constexpr int A_TILE = BM * BK * 2;                 // bytes per A term tile
    static constexpr int B_TILE = BN * BK * 2;                 // bytes per B term tile
    static constexpr int STAGE = NP * (A_TILE + B_TILE);
    static constexpr int STAGES = RED ? (NP == 3 ? 2 : NP == 2 ? 3 : 6) : (NP == 3 ? 3 : NP == 2 ? 4 : 8);
    static constexpr int NPROD = NP == 3 ? 6 : NP == 2 ? 3 : 1;
    static constexpr int EPI_BUF = 32 * 32 * 4;                // one 32 x 32 fp32 chunk
    static constexpr int EPI_BYTES = RED ? EPI_WARPS * 2 * EPI_BUF : 0;
    static constexpr size_t SMEM = (size_t)STAGES * STAGE + EPI_BYTES + 1024 /*align*/ + 256 /*barriers*/;
};

// Products (A term, B term), smallest first.
__device__ __constant__ int kProdA[6] = {2, 1, 0, 1, 0, 0};
__device__ __constant__ int kProdB[6] = {0, 1, 2, 0, 1, 0};
__device__ __forceinline__ int prod_a(int np, int p) { return np == 3 ? kProdA[p] : np == 2 ? (p == 0 ? 1 : 0) : 0; }
__device__ __forceinline__ int prod_b(int np, int p) { return np == 3 ? kProdB[p] : np == 2 ? (p == 1 ? 1 : 0) : 0; }

// Lower mode (a symmetric update of which only the lower triangle is kept):
// the tiles that meet the triangle row >= column, by column blocks; column
// block nb (columns nb*BN ..) meets it from m-block nb*BN/BM on.
static_assert(BN % BM == 0, "lower mode assumes whole m-blocks per column block");
constexpr int BN_BM = BN / BM;
__host__ __device__ __forceinline__ int lower_tiles(int num_m, int num_n) {
    int total = 0;
    for (int nb = 0; nb < num_n; ++nb) total += num_m > BN_BM * nb ? num_m - BN_BM * nb : 0;
    return total;
}
__device__ __forceinline__ void tile_coords_lower(int t, int num_m, int num_n, int& mb, int& nb) {
    nb = 0;
    for (; nb < num_n - 1; ++nb) {
        const int cnt = num_m > BN_BM * nb ? num_m - BN_BM * nb : 0;
        if (t < cnt) break;
        t -= cnt;
    }
    mb = BN_BM * nb + t;
}

__device__ __forceinline__ void tile_coords(int t, int num_m, int num_n, int& mb, int& nb) {
    // grouped raster: 16 m-blocks per group, n fastest inside the group
    constexpr int GM = 16;
    const int per_group = GM * num_n;
    const int g = t / per_group;
    const int first_m = g * GM;
    const int gsize = min(GM, num_m - first_m);
    const int r = t - g * per_group;
    mb = first_m + r % gsize;
    nb = r / gsize;
}

// A C that streams through L2 once (a far trailing update, a large product)
// is loaded and stored with an evict-first L2 policy, so that it does not
// push out what is reused (the split operands, and the panel that a
// concurrent factorization step works on); a C that is read again soon (the
// next panel's columns) keeps the normal policy.  The loads do not allocate
// in L1.
__device__ __forceinline__ uint64_t l2_policy(bool stream) {
    uint64_t p;
    if (stream)
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
    else
        asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;\n" : "=l"(p));
    return p;
}

__device__ __forceinline__ float ld_stream(const float* p, uint64_t pol) {
    float v;
    asm volatile("ld.global.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;\n" : "=f"(v) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ void st_stream(float* p, float v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;\n" ::"l"(p), "f"(v), "l"(pol) : "memory");
}

// Epilogue helpers: 32 consecutive columns of one row of C.
__device__ __forceinline__ void epi_load(bool rd, const float* crow, int ldc, int col0, int N, uint64_t pol,
                                         float (&cv)[32]) {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const int col = col0 + j;
        cv[j] = (rd && col < N) ? ld_stream(crow + (size_t)col * ldc, pol) : 0.f;
    }
}

__device__ __forceinline__ void epi_store(bool wr, float* crow, int ldc, int col0, int N, uint64_t pol, uint32_t taddr, float alpha,
                                          float beta, const float (&cv)[32]) {
    uint32_t r[32];
    tc::tmem_ld_32x32b_x32(taddr, r);
    tc::tmem_ld_wait();
    if (!wr) return;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const int col = col0 + j;
        if (col < N) {
            const float v = alpha * __uint_as_float(r[j]);
            st_stream(crow + (size_t)col * ldc, beta == 0.f ? v : fmaf(beta, cv[j], v), pol);
        }
    }
}

template <int NP, bool RED>
__global__ void __launch_bounds__(THREADS, 1)
    bf16x_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      const __grid_constant__ CUtensorMap tmC, float* __restrict__ C, int ldc, int M, int N, int Kp,
                      float alpha, float beta, int stream_c, int two_pass, int lower, int ksplit,
                      int* __restrict__ err) {
    using CF = Cfg<NP, RED>;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float* const epi_sm = (float*)(smem + (size_t)CF::STAGES * CF::STAGE);  // RED staging
    uint64_t* bars = (uint64_t*)(smem + (size_t)CF::STAGES * CF::STAGE + CF::EPI_BYTES);
    uint64_t* full = bars;
    uint64_t* empty = bars + CF::STAGES;
    uint64_t* acc_full = bars + 2 * CF::STAGES;
    uint64_t* acc_empty = acc_full + 2;
    uint64_t* mma_done = acc_empty + 2;
    uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);
    __shared__ int s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int num_m = (M + BM - 1) / BM, num_n = (N + BN - 1) / BN;
    const int tiles = lower ? lower_tiles(num_m, num_n) : num_m * num_n;
    // split-K (RED only): work item t is tile t % tiles over the k-blocks of
    // slice t / tiles, its product added into C like every other slice's
    const int total = tiles * ksplit;
    const int kblocks = Kp / BK;
    auto slice_k = [&](int t, int& kb0, int& nk) {
        const int sl = t / tiles;
        kb0 = sl * kblocks / ksplit;
        nk = (sl + 1) * kblocks / ksplit - kb0;
    };
    // two_pass (NP >= 2): every k-block's lower-order products first, then
    // a second pass over K for the leading product A_0 B_0 alone, so that
    // the tensor cores' accumulation (which rounds relative to the running
    // sum) adds the small terms while the accumulator is still small
    const int npass = (two_pass && NP >= 2) ? 2 : 1;

    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int s = 0; s < CF::STAGES; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], 32 * EPI_WARPS);
        }
        tc::mbar_init(mma_done, 1);
        tc::fence_barrier_init();
        tc::prefetch_tmap(&tmA);
        tc::prefetch_tmap(&tmB);
        if (RED) tc::prefetch_tmap(&tmC);
    }
    if (warp == 1) {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // ---------------------------------------------------------------- producer
            int stage = 0;
            uint32_t phase = 0;
            bool issued[CF::STAGES];
            uint32_t last_phase[CF::STAGES];
            for (int s = 0; s < CF::STAGES; ++s) issued[s] = false, last_phase[s] = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < total && ok; t += gridDim.x) {
                int mb, nb;
                if (lower)
                    tile_coords_lower(t % tiles, num_m, num_n, mb, nb);
                else
                    tile_coords(t % tiles, num_m, num_n, mb, nb);
                int kb0, nk;
                slice_k(t, kb0, nk);
                for (int ks = 0; ks < npass * nk && ok; ++ks) {
                    const int kb = kb0 + ks % nk;
                    // the leading-product pass needs only the terms A_0, B_0
                    const int nterm = (npass == 2 && ks >= nk) ? 1 : NP;
                    if (!tc::mbar_wait(&empty[stage], phase ^ 1)) {
                        ok = false;
                        break;
                    }
                    if (*(volatile int*)&s_abort) {
                        ok = false;
                        break;
                    }
                    unsigned char* st = smem + (size_t)stage * CF::STAGE;
                    tc::mbar_arrive_expect_tx(&full[stage], (uint32_t)nterm * (CF::A_TILE + CF::B_TILE));
                    for (int p = 0; p < nterm; ++p) {
                        tc::tma_load_3d(st + p * CF::A_TILE, &tmA, &full[stage], kb * BK, mb * BM, p);
                        tc::tma_load_3d(st + NP * CF::A_TILE + p * CF::B_TILE, &tmB, &full[stage], kb * BK,
                                        nb * BN, p);
                    }
                    issued[stage] = true;
                    last_phase[stage] = phase;
                    if (++stage == CF::STAGES) stage = 0, phase ^= 1;
                }
            }
            if (!ok) {
                atomicExch(err, 8);
                s_abort = 1;
            }
            // drain: every copy this thread issued has landed before exit
            for (int s = 0; s < CF::STAGES; ++s)
                if (issued[s]) tc::mbar_wait(&full[s], last_phase[s]);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ------------------------------------------------------------ MMA issuer
            constexpr uint32_t idesc = tc::idesc_bf16_f32(BM, BN);
            int stage = 0;
            uint32_t phase = 0;
            int it = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < total && ok; t += gridDim.x, ++it) {
                const int buf = it & 1;
                if (!tc::mbar_wait(&acc_empty[buf], ((it >> 1) & 1) ^ 1)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t d = tmem_base + (uint32_t)(buf * BN);
                int kb0, nk;
                slice_k(t, kb0, nk);
                for (int ks = 0; ks < npass * nk; ++ks) {
                    if (!tc::mbar_wait(&full[stage], phase) || *(volatile int*)&s_abort) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    const uint32_t st = tc::smem_u32(smem + (size_t)stage * CF::STAGE);
                    // products of this k-block: all (one pass), the lower-order
                    // ones (first pass) or the leading one (second pass); the
                    // leading product is the last of the list
                    const int p_lo = (npass == 2 && ks >= nk) ? CF::NPROD - 1 : 0;
                    const int p_hi = (npass == 2 && ks < nk) ? CF::NPROD - 1 : CF::NPROD;
#pragma unroll
                    for (int p = 0; p < CF::NPROD; ++p) {
                        if (p < p_lo || p >= p_hi) continue;
                        const uint32_t a0 = st + prod_a(NP, p) * CF::A_TILE;
                        const uint32_t b0 = st + NP * CF::A_TILE + prod_b(NP, p) * CF::B_TILE;
#pragma unroll
                        for (int kk = 0; kk < BK / 16; ++kk) {
                            // advance 16 bf16 = 32 B inside the 64-byte swizzled row
                            const uint64_t ad = tc::smem_desc_sw64(a0 + kk * 32);
                            const uint64_t bd = tc::smem_desc_sw64(b0 + kk * 32);
                            tc::mma_bf16(d, ad, bd, idesc, (ks | (p - p_lo) | kk) != 0);
                        }
                    }
                    tc::mma_commit(&empty[stage]);
                    if (++stage == CF::STAGES) stage = 0, phase ^= 1;
                }
                if (!ok) break;
                tc::mma_commit(&acc_full[buf]);
            }
            if (!ok) {
                atomicExch(err, 8);
                s_abort = 1;
            }
            // all MMAs of this thread complete before TMEM is released
            tc::mma_commit(mma_done);
            tc::mbar_wait(mma_done, 0);
        }
    } else {
        // ------------------------------------------------------------------ epilogue
        const int q = warp & 3;  // TMEM lane quarter this warp may access
        const int row_in_tile = q * 32 + lane;
        constexpr int CH_PER = BN / 32 / (EPI_WARPS / 4);  // 32-column chunks per warp
        const int ch0 = ((warp - 2) / 4) * CH_PER;           // this warp's first chunk
        int it = 0;
        int nred = 0;  // RED: reductions issued by this warp (alternating staging buffers)
        for (int t = blockIdx.x; t < total; t += gridDim.x, ++it) {
            const int buf = it & 1;
            if (!tc::mbar_wait(&acc_full[buf], (it >> 1) & 1) || *(volatile int*)&s_abort) {
                atomicExch(err, 8);
                s_abort = 1;
                break;
            }
            tc::tc_fence_after();
            int mb, nb;
            if (lower)
                tile_coords_lower(t % tiles, num_m, num_n, mb, nb);
            else
                tile_coords(t % tiles, num_m, num_n, mb, nb);
            const int row = mb * BM + row_in_tile;
            const uint32_t taddr = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * BN);
            if constexpr (RED) {
                // each 32 x 32 chunk: accumulator -> staging buffer (lane = row,
                // column-major like the tensor map's box) -> one TMA reduction
                // into C, which clips rows >= M and columns >= N; the buffer's
                // previous reduction must have read it first
                float* const wbuf = epi_sm + (size_t)(warp - 2) * 2 * 1024;
#pragma unroll 1
                for (int ch = ch0; ch < ch0 + CH_PER; ++ch) {
                    if (nb * BN + ch * 32 >= N || mb * BM + q * 32 >= M) continue;  // outside C
                    uint32_t r[32];
                    tc::tmem_ld_32x32b_x32(taddr + ch * 32, r);
                    tc::tmem_ld_wait();
                    float* const sb = wbuf + (nred++ & 1) * 1024;
                    if (lane == 0) tc::bulk_wait_group_read<1>();
                    __syncwarp();
#pragma unroll
                    for (int j = 0; j < 32; ++j) sb[j * 32 + lane] = alpha * __uint_as_float(r[j]);
                    tc::fence_proxy_async_shared();
                    __syncwarp();
                    if (lane == 0) {
                        tc::tma_reduce_add_2d(&tmC, sb, mb * BM + q * 32, nb * BN + ch * 32);
                        tc::bulk_commit_group();
                    }
                }
                tc::tc_fence_before();
                tc::mbar_arrive(&acc_empty[buf]);
                continue;
            }
            // Software-pipelined by chunks of 32 columns: the C values of chunk
            // ch+1 are loaded (32 independent loads per thread in flight) before
            // chunk ch is combined with the accumulator and stored.
            const bool rd = beta != 0.f && row < M;
            const float* crow = C + (size_t)row;
            float ca[32], cb[32];
            const uint64_t pol = l2_policy(stream_c != 0);
            epi_load(rd, crow, ldc, nb * BN + ch0 * 32, N, pol, ca);
#pragma unroll 1
            for (int ch = ch0; ch < ch0 + CH_PER; ch += 2) {
                epi_load(rd, crow, ldc, nb * BN + (ch + 1) * 32, N, pol, cb);
                epi_store(row < M, C + (size_t)row, ldc, nb * BN + ch * 32, N, pol, taddr + ch * 32, alpha, beta, ca);
                if (ch + 2 < ch0 + CH_PER) epi_load(rd, crow, ldc, nb * BN + (ch + 2) * 32, N, pol, ca);
                epi_store(row < M, C + (size_t)row, ldc, nb * BN + (ch + 1) * 32, N, pol, taddr + (ch + 1) * 32, alpha,
                          beta, cb);
            }
            tc::tc_fence_before();
            tc::mbar_arrive(&acc_empty[buf]);
        }
    }

    if (RED && warp >= 2 && lane == 0) tc::bulk_wait_group<0>();  // every reduction complete
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem_base, TMEM_COLS);
    }
}

// ------------------------------------------------------------------ splitting
__device__ __forceinline__ void split3(float x, __nv_bfloat16& h0, __nv_bfloat16& h1, __nv_bfloat16& h2) {
    h0 = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h0);
    h1 = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(h1);
    h2 = __float2bfloat16_rn(r2);
}

// A (rows x K, column-major, ld) -> parts[p][row][k] (row stride Kp, zero
// padded for k >= K): a 32x32 tiled transpose through shared memory.
template <typename TIN>
__global__ void split_rows_kernel(const TIN* __restrict__ A, int lda, int rows, int K, int Kp, int np,
                                  __nv_bfloat16* __restrict__ out, size_t part_stride) {
    __shared__ float tile[32][33];
    const int k0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    for (int j = ty; j < 32; j += 8) {
        const int k = k0 + j, r = r0 + tx;
        tile[j][tx] = (k < K && r < rows) ? (float)A[(size_t)r + (size_t)k * lda] : 0.f;
    }
    __syncthreads();
    for (int j = ty; j < 32; j += 8) {
        const int r = r0 + j, k = k0 + tx;
        if (r < rows && k < Kp) {
            __nv_bfloat16 h0, h1, h2;
            split3(tile[tx][j], h0, h1, h2);
            const size_t o = (size_t)r * Kp + k;
            out[o] = h0;
            if (np > 1) out[part_stride + o] = h1;
            if (np > 2) out[2 * part_stride + o] = h2;
        }
    }
}

// B (K x cols, column-major, ld) -> parts[p][col][k]: column c of B is row c.
template <typename TIN>
__global__ void split_cols_kernel(const TIN* __restrict__ B, int ldb, int K, int cols, int Kp, int np,
                                  __nv_bfloat16* __restrict__ out, size_t part_stride) {
    const size_t total = (size_t)cols * Kp;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(e / Kp), k = (int)(e % Kp);
        const float x = k < K ? (float)B[(size_t)k + (size_t)c * ldb] : 0.f;
        __nv_bfloat16 h0, h1, h2;
        split3(x, h0, h1, h2);
        out[e] = h0;
        if (np > 1) out[part_stride + e] = h1;
        if (np > 2) out[2 * part_stride + e] = h2;
    }
}

// X (rows x 64, ld ldx) := X G in FP32, G = L^{-T} (64 x 64 upper
// triangular, column-major, ld 64), the split terms of the result as a
// K = 64 operand (parts[p][row][64]), and, with ntop > 0, the update of the
// next block column C (rows x ntop, ld ldx) -= X Xt^T in FP32, Xt (64 x 64,
// ld 64; rows ntop .. zero) being the first ntop rows of the result, formed
// beforehand by the diagonal block's kernel.  One CTA of 128 threads per
// 32 rows (two CTAs per SM at 8128 rows); each thread 4 rows x 4 columns of
// both products, over the X tile, G (pitch 65
// words: the two column groups of a warp read different banks) and Xt
// staged in shared memory; the result staged again (column-major, pitch 68
// for 16-byte accesses) for the coalesced column stores of X, the 16-byte
// row stores of the terms and the second product.  This is the block-column
// solve X := X L^{-T} of the mixed SPD factorization as a product by the
// diagonal block's inverse, with the look-ahead part of the trailing update.
constexpr int XS_ROWS = 32;              // rows per CTA
constexpr int XS_T = XS_ROWS * 4;         // threads: 4 x 4 outputs each over XS_ROWS x 64
constexpr int XS_TX = XS_ROWS / 4;        // row groups
constexpr int XS_P = 65;
constexpr int XS_OP = XS_ROWS + 4;        // column pitch of the staged result (16-byte aligned)
constexpr size_t XS_SMEM = (size_t)(XS_P * 64 + 64 * XS_ROWS + 64 * 64) * sizeof(float);
static_assert(XS_OP * 64 <= XS_P * 64 + 64 * XS_ROWS, "the staged result fits over G and the X tile");

__global__ void __launch_bounds__(XS_T) xlt_split64_kernel(const float* __restrict__ G, float* __restrict__ X, int ldx,
                                                          int rows, int np, __nv_bfloat16* __restrict__ out,
                                                          size_t part_stride, const float* __restrict__ xtop,
                                                          int ntop, float* __restrict__ C) {
    extern __shared__ __align__(16) float xs_sm[];
    float* const gs = xs_sm;                      // G(k, c) at k + XS_P c
    float* const xs = xs_sm + XS_P * 64;          // X(r, k) at r + XS_ROWS k
    float* const xt = xs + 64 * XS_ROWS;          // Xt(c, k) at c + 64 k
    float* const os = xs_sm;                      // result (r, c) at r + XS_OP c, after the first product
    const int t = threadIdx.x;
    const int row0 = blockIdx.x * XS_ROWS;
    const int tx = t % XS_TX, ty = t / XS_TX;  // rows 4 tx .. 4 tx + 3, columns 4 ty .. 4 ty + 3
    // every global load of the kernel issued up front: this thread's part of
    // G, X and Xt, and the 4 x 4 block of C it updates at the end
    float cv[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = row0 + 4 * tx + i, c = 4 * ty + j;
            cv[i][j] = (r < rows && c < ntop) ? C[(size_t)r + (size_t)c * ldx] : 0.f;
        }
    {
        constexpr int NG = 64 * 64 / XS_T, NX = XS_ROWS * 64 / XS_T;
        float gv[NG], xv[NX], tv[NG];
#pragma unroll
        for (int u = 0; u < NG; ++u) {
            const int e = t + XS_T * u;
            gv[u] = __ldg(G + e);
            tv[u] = ntop > 0 ? __ldg(xtop + e) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < NX; ++u) {
            const int e = t + XS_T * u, r = e % XS_ROWS, c = e / XS_ROWS;
            xv[u] = row0 + r < rows ? X[(size_t)(row0 + r) + (size_t)c * ldx] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < NG; ++u) {
            const int e = t + XS_T * u;
            gs[(e & 63) + XS_P * (e >> 6)] = gv[u];
            xt[e] = tv[u];
        }
#pragma unroll
        for (int u = 0; u < NX; ++u) xs[t + XS_T * u] = xv[u];
    }
    __syncthreads();
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
#pragma unroll 8
    for (int k = 0; k < 64; ++k) {
        const float4 xv = *reinterpret_cast<const float4*>(xs + XS_ROWS * k + 4 * tx);
        const float xr[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float g = gs[k + XS_P * (4 * ty + j)];
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[i][j] = fmaf(xr[i], g, acc[i][j]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; ++j)
        *reinterpret_cast<float4*>(os + XS_OP * (4 * ty + j) + 4 * tx) =
            make_float4(acc[0][j], acc[1][j], acc[2][j], acc[3][j]);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < XS_ROWS * 64 / XS_T; ++u) {
        const int e = t + XS_T * u, r = e % XS_ROWS, c = e / XS_ROWS;
        if (row0 + r < rows) X[(size_t)(row0 + r) + (size_t)c * ldx] = os[r + XS_OP * c];
    }
#pragma unroll
    for (int u = 0; u < XS_ROWS * 8 / XS_T; ++u) {
        const int e = t + XS_T * u, r = e % XS_ROWS, c8 = (e / XS_ROWS) * 8;
        if (row0 + r >= rows) continue;
        uint32_t w0[4], w1[4], w2[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            __nv_bfloat16 a0, a1, a2, b0, b1, b2;
            split3(os[r + XS_OP * (c8 + 2 * v)], a0, a1, a2);
            split3(os[r + XS_OP * (c8 + 2 * v + 1)], b0, b1, b2);
            w0[v] = (uint32_t)__bfloat16_as_ushort(a0) | ((uint32_t)__bfloat16_as_ushort(b0) << 16);
            w1[v] = (uint32_t)__bfloat16_as_ushort(a1) | ((uint32_t)__bfloat16_as_ushort(b1) << 16);
            w2[v] = (uint32_t)__bfloat16_as_ushort(a2) | ((uint32_t)__bfloat16_as_ushort(b2) << 16);
        }
        const size_t o = (size_t)(row0 + r) * 64 + c8;
        *reinterpret_cast<uint4*>(out + o) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
        if (np > 1) *reinterpret_cast<uint4*>(out + part_stride + o) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
        if (np > 2) *reinterpret_cast<uint4*>(out + 2 * part_stride + o) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
    }
    if (ntop <= 0) return;
    // C(r, c) -= sum_k X(r, k) Xt(c, k) for the next block column
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
#pragma unroll 8
    for (int k = 0; k < 64; ++k) {
        const float4 xv = *reinterpret_cast<const float4*>(os + XS_OP * k + 4 * tx);
        const float4 tv = *reinterpret_cast<const float4*>(xt + 64 * k + 4 * ty);
        const float xr[4] = {xv.x, xv.y, xv.z, xv.w}, tr[4] = {tv.x, tv.y, tv.z, tv.w};
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[i][j] = fmaf(xr[i], tr[j], acc[i][j]);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = row0 + 4 * tx + i, c = 4 * ty + j;
            if (r < rows && c < ntop) C[(size_t)r + (size_t)c * ldx] = cv[i][j] - acc[i][j];
        }
}

// U12 := L11^{-1} A12 (FP32, L11 unit lower w x w, w <= 128) and the split
// terms of U12 as the B operand of the trailing updates ([term][column][Kp],
// zero rows w .. Kp-1), in one pass: one CTA per 64 columns of A12, four
// threads per column; in each 16-row block thread g of a column holds rows
// g, g+4, g+8, g+12.  L11 sits row-major and the columns column-major in
// shared memory, both with a pitch of 4 mod 32 words, which makes every
// access conflict-free: the coalesced global loads and stores (a warp on 32
// consecutive rows of a column), the four rows of L a warp reads at once, a
// column's 16-row slices read as float4s, and the 8 columns x 4 rows of a
// warp's solution values.  Per 16-row block: the updates from every earlier
// block (16 products per row and block), then the 16 x 16 unit-lower solve,
// each solved value passed by a shuffle inside the column's group of four.
// This replaces an explicit inverse of L11, two splits and a tensor-core
// product on the critical path of every step of the mixed LU.
constexpr int TS_W = 128;  // widest panel
constexpr int TS_C = 64;   // columns per CTA
constexpr int TS_TPC = 8;  // threads per column: rows g, g + 8 of every 16-row block
constexpr int TS_RPB = 16 / TS_TPC;
constexpr int TS_THREADS = TS_TPC * TS_C;
constexpr int TS_P = TS_W + 4;  // pitch of both shared arrays (words)
constexpr size_t TS_SMEM = (size_t)(TS_W * TS_P + TS_C * TS_P) * sizeof(float);

__global__ void __launch_bounds__(TS_THREADS) trsm_split_kernel(const float* __restrict__ L, int lda,
                                                               float* __restrict__ A12, int nt, int w, int np, int Kp,
                                                               size_t part_stride, __nv_bfloat16* __restrict__ out) {
    extern __shared__ __align__(16) float ts_sm[];
    float* const sL = ts_sm;                // [TS_W][TS_P]: L11(i, j) at i * TS_P + j, strict lower part only
    float* const sx = ts_sm + TS_W * TS_P;  // [TS_C][TS_P]: row i of column c at c * TS_P + i
    const int tid = threadIdx.x, lane = tid & 31;
    const int c = (tid >> 5) * (32 / TS_TPC) + lane / TS_TPC;  // my column (of this CTA's TS_C)
    const int g = lane & (TS_TPC - 1);                          // my rows g + TS_TPC a of each 16-row block
    const int c0 = blockIdx.x * TS_C;
    const int ncol = min(TS_C, nt - c0);
    float* const xc = sx + c * TS_P;
    // loads in batches of 32 per thread, all in flight together (a load ->
    // shared store loop would wait for each one)
    for (int e0 = 0; e0 < TS_W * TS_W; e0 += 32 * TS_THREADS) {
        float t[32];
#pragma unroll
        for (int u = 0; u < 32; ++u) {
            const int e = e0 + tid + u * TS_THREADS, i = e % TS_W, j = e / TS_W;
            t[u] = (i < w && j < i) ? L[i + (size_t)j * lda] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 32; ++u) {
            const int e = e0 + tid + u * TS_THREADS, i = e % TS_W, j = e / TS_W;
            sL[i * TS_P + j] = t[u];
        }
    }
    {
        float t[TS_W * TS_C / TS_THREADS];
#pragma unroll
        for (int u = 0; u < TS_W * TS_C / TS_THREADS; ++u) {
            const int e = tid + u * TS_THREADS, i = e % TS_W, cc = e / TS_W;
            t[u] = (i < w && cc < ncol) ? A12[i + (size_t)(c0 + cc) * lda] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < TS_W * TS_C / TS_THREADS; ++u) {
            const int e = tid + u * TS_THREADS, i = e % TS_W, cc = e / TS_W;
            sx[cc * TS_P + i] = t[u];
        }
    }
    __syncthreads();
    for (int I = 0; I < w; I += 16) {
        float xi[TS_RPB];  // rows I + g + TS_TPC a
#pragma unroll
        for (int a = 0; a < TS_RPB; ++a) xi[a] = xc[I + g + TS_TPC * a];
        for (int J = 0; J < I; J += 16) {
            float xj[16];
#pragma unroll
            for (int b4 = 0; b4 < 4; ++b4) {
                const float4 v = reinterpret_cast<const float4*>(xc + J)[b4];
                xj[4 * b4 + 0] = v.x;
                xj[4 * b4 + 1] = v.y;
                xj[4 * b4 + 2] = v.z;
                xj[4 * b4 + 3] = v.w;
            }
#pragma unroll
            for (int a = 0; a < TS_RPB; ++a) {
                const float4* lr = reinterpret_cast<const float4*>(sL + (I + g + TS_TPC * a) * TS_P + J);
#pragma unroll
                for (int b4 = 0; b4 < 4; ++b4) {
                    const float4 l = lr[b4];
                    xi[a] = fmaf(-l.x, xj[4 * b4 + 0], xi[a]);
                    xi[a] = fmaf(-l.y, xj[4 * b4 + 1], xi[a]);
                    xi[a] = fmaf(-l.z, xj[4 * b4 + 2], xi[a]);
                    xi[a] = fmaf(-l.w, xj[4 * b4 + 3], xi[a]);
                }
            }
        }
        // the 16 x 16 diagonal block: x_b final -> the rows below it in the block
#pragma unroll
        for (int b = 0; b < 16; ++b) {
            const float xb = __shfl_sync(0xffffffffu, xi[b / TS_TPC], (lane & ~(TS_TPC - 1)) | (b % TS_TPC));
#pragma unroll
            for (int a = 0; a < TS_RPB; ++a)
                if (g + TS_TPC * a > b) xi[a] = fmaf(-sL[(I + g + TS_TPC * a) * TS_P + I + b], xb, xi[a]);
        }
#pragma unroll
        for (int a = 0; a < TS_RPB; ++a) xc[I + g + TS_TPC * a] = xi[a];
        __syncwarp();  // a column's four threads share one warp
    }
    __syncthreads();
    for (int e = tid; e < Kp * ncol; e += TS_THREADS) {
        const int i = e % Kp, cc = e / Kp;
        const float v = i < w ? sx[cc * TS_P + i] : 0.f;
        if (i < w) A12[i + (size_t)(c0 + cc) * lda] = v;
        __nv_bfloat16 h0, h1, h2;
        split3(v, h0, h1, h2);
        const size_t o = (size_t)(c0 + cc) * Kp + i;
        out[o] = h0;
        if (np > 1) out[part_stride + o] = h1;
        if (np > 2) out[2 * part_stride + o] = h2;
    }
}

// --------------------------------------------------------------- tensor maps
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn get_encode() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

// 3-D map over parts[np][rows][Kp] bf16 with box {BK, box_rows, 1}, 64-byte swizzle.
bool make_map(CUtensorMap* map, const void* base, int rows, int Kp, int np, size_t part_stride, int box_rows) {
    EncodeTiledFn enc = get_encode();
    if (!enc) return false;
    cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)np};
    cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)part_stride * 2};
    cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool make_cmap(CUtensorMap* map, float* C, int ldc, int M, int N) {
    EncodeTiledFn enc = get_encode();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)M, (cuuint64_t)N};
    cuuint64_t strides[1] = {(cuuint64_t)ldc * 4};
    cuuint32_t box[2] = {32, 32};
    cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, C, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int NP>
mg_status_t launch_gemm_np(mg_handle_t h, const CUtensorMap& ma, const CUtensorMap& mb, float* C, int ldc, int M,
                           int N, int Kp, float alpha, float beta, int* err, int max_ctas, int stream_c,
                           int two_pass, int lower, bool red_epi, int ksplit) {
    const int num_m = (M + BM - 1) / BM, num_n = (N + BN - 1) / BN;
    const int tiles = (lower ? lower_tiles(num_m, num_n) : num_m * num_n) * ksplit;
    const int cap = max_ctas > 0 && max_ctas < h->num_sms ? max_ctas : h->num_sms;
    const int grid = tiles < cap ? tiles : cap;
    CUtensorMap mc;
    // the TMA-reduction epilogue when asked for (beta = 1, C 16-byte
    // aligned, ldc a multiple of 4 floats)
    const bool red = (red_epi || ksplit > 1) && beta == 1.f && ((uintptr_t)C & 15) == 0 && (ldc & 3) == 0 &&
                     make_cmap(&mc, C, ldc, M, N);
    if (ksplit > 1 && !red) return mg::fail(h, MG_ERR_ARG, "split GEMM: split-K needs beta = 1 and an aligned C");
    if (red) {
        auto kern = bf16x_gemm_kernel<NP, true>;
        MG_CHECK_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)Cfg<NP, true>::SMEM));
        kern<<<grid, THREADS, Cfg<NP, true>::SMEM, h->stream>>>(ma, mb, mc, C, ldc, M, N, Kp, alpha, beta, stream_c,
                                                                two_pass, lower, ksplit, err);
    } else {
        std::memset(&mc, 0, sizeof(mc));
        auto kern = bf16x_gemm_kernel<NP, false>;
        MG_CHECK_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)Cfg<NP, false>::SMEM));
        kern<<<grid, THREADS, Cfg<NP, false>::SMEM, h->stream>>>(ma, mb, mc, C, ldc, M, N, Kp, alpha, beta, stream_c,
                                                                 two_pass, lower, 1, err);
    }
    return mg::post_launch(h, "bf16x_gemm_kernel");
}

}  // namespace

namespace mg {

size_t bf16x_split_bytes(int rows, int K, int np) {
    const int Kp = (K + BK - 1) / BK * BK;
    return align_up((size_t)np * rows * Kp * 2, 1024);
}

// Splits an fp32/fp64 operand into np bf16 terms.  a_side: rows x K column-
// major (transposed into K-major rows); else K x cols column-major.
template <typename TIN>
mg_status_t bf16x_split(mg_handle_t h, bool a_side, const TIN* X, int ldx, int rows_or_cols, int K, int np,
                        void* out) {
    const int Kp = (K + BK - 1) / BK * BK;
    const size_t ps = (size_t)rows_or_cols * Kp;
    if (a_side) {
        dim3 grid((Kp + 31) / 32, (rows_or_cols + 31) / 32);
        split_rows_kernel<TIN><<<grid, dim3(32, 8), 0, h->stream>>>(X, ldx, rows_or_cols, K, Kp, np,
                                                                     (__nv_bfloat16*)out, ps);
        return post_launch(h, "split_rows_kernel");
    }
    size_t blocks = (ps + 255) / 256;
    if (blocks > (size_t)h->num_sms * 16) blocks = (size_t)h->num_sms * 16;
    split_cols_kernel<TIN><<<(unsigned)blocks, 256, 0, h->stream>>>(X, ldx, K, rows_or_cols, Kp, np,
                                                                    (__nv_bfloat16*)out, ps);
    return post_launch(h, "split_cols_kernel");
}
template mg_status_t bf16x_split<float>(mg_handle_t, bool, const float*, int, int, int, int, void*);
mg_status_t bf16x_xlt_split64(mg_handle_t h, const float* G, float* X, int ldx, int rows, int np, void* out,
                              const float* xtop, int ntop, float* C) {
    if (rows <= 0) return MG_OK;
    static_assert(64 % BK == 0, "a 64-column operand needs no K padding");
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(xlt_split64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)XS_SMEM));
    xlt_split64_kernel<<<(rows + XS_ROWS - 1) / XS_ROWS, XS_T, XS_SMEM, h->stream>>>(
        G, X, ldx, rows, np, (__nv_bfloat16*)out, (size_t)rows * 64, xtop, ntop, C);
    return post_launch(h, "xlt_split64_kernel");
}

template mg_status_t bf16x_split<double>(mg_handle_t, bool, const double*, int, int, int, int, void*);

mg_status_t bf16x_trsm_split(mg_handle_t h, const float* L11, int lda, float* A12, int nt, int w, int np, void* out) {
    if (nt <= 0 || w <= 0) return MG_OK;
    if (w > TS_W) return fail(h, MG_ERR_ARG, "bf16x_trsm_split: panel width %d > %d", w, TS_W);
    const int Kp = (w + BK - 1) / BK * BK;
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(trsm_split_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TS_SMEM));
    trsm_split_kernel<<<(nt + TS_C - 1) / TS_C, TS_THREADS, TS_SMEM, h->stream>>>(L11, lda, A12, nt, w, np, Kp,
                                                                                 (size_t)nt * Kp, (__nv_bfloat16*)out);
    return post_launch(h, "trsm_split_kernel");
}

// C = alpha * (split A)(split B) + beta * C from pre-split operands.
int bf16x_kpad(int K) { return (K + BK - 1) / BK * BK; }

mg_status_t bf16x_gemm_presplit(mg_handle_t h, int np, int M, int N, int K, float alpha, const void* Asplit,
                                const void* Bsplit, float beta, float* C, int ldc, int* err, size_t a_term,
                                size_t b_term, int max_ctas, bool stream_c, bool two_pass, bool lower,
                                bool red_epi, int ksplit) {
    if (M == 0 || N == 0) return MG_OK;
    if (lower && M != N) return fail(h, MG_ERR_ARG, "split GEMM: lower mode needs a square C (M=%d N=%d)", M, N);
    if (ksplit < 1 || ksplit > (K + BK - 1) / BK) return fail(h, MG_ERR_ARG, "split GEMM: bad split-K %d", ksplit);
    const int Kp = (K + BK - 1) / BK * BK;
    if (!a_term) a_term = (size_t)M * Kp;
    if (!b_term) b_term = (size_t)N * Kp;
    CUtensorMap ma, mb;
    if (!make_map(&ma, Asplit, M, Kp, np, a_term, BM) || !make_map(&mb, Bsplit, N, Kp, np, b_term, BN))
        return fail(h, MG_ERR_CUDA, "cuTensorMapEncodeTiled failed (M=%d N=%d Kp=%d)", M, N, Kp);
    const int nprod = np == 3 ? 6 : np == 2 ? 3 : 1;
    // flops: every bf16 product the tensor cores execute; bytes: C read+write plus the split operands once
    // lower mode: the tiles meeting the lower triangle, about half of C
    const double frac = lower ? (lower_tiles((M + BM - 1) / BM, (N + BN - 1) / BN) * (double)BM * BN) / ((double)M * N)
                              : 1.0;
    ProfScope prof(h, "gemm_bf16x", frac * 2.0 * M * N * (double)Kp * nprod,
                   frac * (beta == 0.f ? 4.0 : 8.0) * M * N + 2.0 * np * (double)(M + N) * Kp);
    switch (np) {
        case 1: return launch_gemm_np<1>(h, ma, mb, C, ldc, M, N, Kp, alpha, beta, err, max_ctas, stream_c, 0, lower, red_epi, ksplit);
        case 2:
            return launch_gemm_np<2>(h, ma, mb, C, ldc, M, N, Kp, alpha, beta, err, max_ctas, stream_c, two_pass, lower, red_epi, ksplit);
        default:
            return launch_gemm_np<3>(h, ma, mb, C, ldc, M, N, Kp, alpha, beta, err, max_ctas, stream_c, two_pass, lower, red_epi, ksplit);
    }
}

}  // namespace mg

extern "C" mg_status_t mg_sgemm_bf16x(mg_handle_t h, int nterms, int m, int n, int k, float alpha, const float* A,
                                      int lda, const float* B, int ldb, float beta, float* C, int ldc) {
    return mg_sgemm_bf16x_ex(h, nterms, 0, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

extern "C" mg_status_t mg_sgemm_bf16x_ex(mg_handle_t h, int nterms, int flags, int m, int n, int k, float alpha,
                                         const float* A, int lda, const float* B, int ldb, float beta, float* C,
                                         int ldc) {
    if (!h) return MG_ERR_ARG;
    if (flags & ~MG_BF16X_ORDERED) return mg::fail(h, MG_ERR_ARG, "mg_sgemm_bf16x_ex: unknown flags %d", flags);
    if (nterms < 1 || nterms > 3 || m < 0 || n < 0 || k < 0 || lda < (m > 1 ? m : 1) || ldb < (k > 1 ? k : 1) ||
        ldc < (m > 1 ? m : 1))
        return mg::fail(h, MG_ERR_ARG, "mg_sgemm_bf16x_ex: bad arguments");
    if (m == 0 || n == 0) return MG_OK;
    if (k == 0) {
        return mg::fail(h, MG_ERR_ARG, "mg_sgemm_bf16x_ex: k == 0 unsupported");
    }
    const size_t as = mg::bf16x_split_bytes(m, k, nterms), bs = mg::bf16x_split_bytes(n, k, nterms);
    MG_TRY(mg::ensure_ws(h, 1024 + as + bs));
    MG_TRY(mg::ensure_hws(h, 64));
    char* ws = (char*)h->ws;
    int* err = (int*)ws;
    MG_CHECK_CUDA(h, cudaMemsetAsync(err, 0, sizeof(int), h->stream));
    void* Asp = ws + 1024;
    void* Bsp = ws + 1024 + as;
    MG_TRY(mg::bf16x_split<float>(h, true, A, lda, m, k, nterms, Asp));
    MG_TRY(mg::bf16x_split<float>(h, false, B, ldb, n, k, nterms, Bsp));
    MG_TRY(mg::bf16x_gemm_presplit(h, nterms, m, n, k, alpha, Asp, Bsp, beta, C, ldc, err, 0, 0, 0, true,
                                   (flags & MG_BF16X_ORDERED) != 0));
    return MG_OK;
}

extern "C" mg_status_t mg_bf16x_check_error(mg_handle_t h, int* device_err_flag) {
    // reads the device error word of the last split GEMM (synchronises)
    if (!h || !device_err_flag) return MG_ERR_ARG;
    if (!h->ws) {
        *device_err_flag = 0;
        return mg::tc_sgemm_error(h, device_err_flag);
    }
    MG_CHECK_CUDA(h, cudaMemcpyAsync(device_err_flag, h->ws, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    int terr = 0;  // and the FP32 GEMMs of the factorizations that ran on the tensor cores
    MG_TRY(mg::tc_sgemm_error(h, &terr));
    *device_err_flag |= terr;
    return MG_OK;
}
