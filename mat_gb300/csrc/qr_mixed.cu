// Mixed-precision Householder QR: the FP32 form of Mat's blocked Householder
// QR (Mat-8.3.1/QR/__Householder_Blocked.h:63-245, FP64 there) for the mixed
// QR solve.  Panels of QB = 128 columns; per column the norm, beta, tau and
// the scale factor of the reflector are formed in FP64 from the fp32 column,
// the reflector, its dot products with the panel's other columns and their
// updates in fp32; the compact WY factor T in fp32; the trailing update
// R2 -= V (T^T (V^T R2)) as three FP32 GEMMs whose large products run on the
// split-BF16 tensor cores (sgemm_auto: 3 terms, lower-order products first,
// fp32 accumulation).
//
// Reflector c of a panel: x = the column from row c down, alpha = x_c,
// beta = -sign(alpha) sqrt(alpha^2 + |x below c|^2), tau = (beta - alpha) /
// beta, v = x / (alpha - beta) below c, v_c = 1 (LAPACK's dlarfg, which Mat's
// blocked panel also follows, :63-84); R(c,c) = beta.  H = I - tau v v^T.
//
// The panel runs as one cooperative grid: its rows dealt to P CTAs in
// contiguous runs (the slab in shared memory); per column one bounded grid
// barrier (the norm's and the dot products' partial sums together), every
// CTA summing the partials in the same order.
#include <cooperative_groups.h>

#include <cmath>

#include "grid_sync.cuh"
#include "mg_internal.cuh"
#include "tc_common.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int QB = 128;
constexpr int QP_THREADS = 256;
constexpr int QG_ROWS = 32;                                    // rows per chunk of the in-kernel V^T V
constexpr size_t QG_TILE_BYTES = (size_t)QG_ROWS * (QB + 4) * sizeof(float) + 16;  // + alignment slack

// The panel slab in shared memory: column c of a CTA's rows at slab + c * lds,
// lds = rpc | 1 (odd, so that lanes reading one row of consecutive columns hit
// distinct banks).

// This CTA's part of G = V^T V over its rows of the panel slab (explicit V:
// 1 on the diagonal, 0 above; rows >= h are zero): chunks of QG_ROWS rows
// transposed into a tile after the slab, an 8 x 8 block of G per thread,
// written to gp (QB x QB, ld QB).
__device__ __forceinline__ void gram_part(const float* slab, int w, int lds, int rpc, int r0, int h, float* gp) {
    const int tid = threadIdx.x;
    float* const tile = const_cast<float*>(slab) + (((size_t)w * lds + 3) & ~(size_t)3);  // 16-byte aligned
    constexpr int LT = QB + 4;
    const int ta = tid >> 4, tb = tid & 15;  // G rows 8 ta .., columns 8 tb ..
    float g[8][8];
#pragma unroll
    for (int x = 0; x < 8; ++x)
#pragma unroll
        for (int y = 0; y < 8; ++y) g[x][y] = 0.f;
    for (int i0 = 0; i0 < rpc; i0 += QG_ROWS) {
        __syncthreads();
        for (int e = tid; e < QG_ROWS * QB; e += QP_THREADS) {
            const int cc = e / QG_ROWS, ii = e - cc * QG_ROWS, i = i0 + ii, gi = r0 + i;
            float x = 0.f;
            if (cc < w && i < rpc && gi < h) x = gi > cc ? slab[(size_t)cc * lds + i] : (gi == cc ? 1.f : 0.f);
            tile[ii * LT + cc] = x;
        }
        __syncthreads();
        for (int ii = 0; ii < QG_ROWS; ++ii) {
            const float4* ra = reinterpret_cast<const float4*>(tile + ii * LT + 8 * ta);
            const float4* rb = reinterpret_cast<const float4*>(tile + ii * LT + 8 * tb);
            const float4 a0 = ra[0], a1 = ra[1], b0 = rb[0], b1 = rb[1];
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int x = 0; x < 8; ++x)
#pragma unroll
                for (int y = 0; y < 8; ++y) g[x][y] = fmaf(av[x], bv[y], g[x][y]);
        }
    }
#pragma unroll
    for (int x = 0; x < 8; ++x)
#pragma unroll
        for (int y = 0; y < 8; ++y) gp[(8 * ta + x) + (size_t)(8 * tb + y) * QB] = g[x][y];
}

// The dots of column c (the rows below the diagonal) with the panel's later
// columns jj > c: a thread per (column, half of the rows), four independent
// accumulators along the rows (a fixed order), the halves added in shared
// memory (part: 2 x QB floats); then out(jj, dot) for each jj.  With them,
// under the same CTA barrier, the FP64 sum of squares of those rows: each
// warp reduces its threads' partial sums by a shuffle tree before the
// barrier (overlapping the other warps' dots), warp 0 sums the 8 warps'
// partials after it (a fixed tree) and passes the total to norm_out in
// lane 0.  Called by every thread of the CTA.
template <class Out, class NormOut>
__device__ __forceinline__ void panel_dots_norm(const float* slab, int lds, int rpc, int w, int c, int r0, int h,
                                                float* part, double* red, Out out, NormOut norm_out) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, half = tid >> 7, jj = c + 1 + (tid & 127);
    const int ilo = max(0, c + 1 - r0), ihi = min(rpc, h - r0);  // my rows below the diagonal
    const float* col = slab + (size_t)c * lds;
    if (jj < w) {
        const int mid = ilo + max(0, ihi - ilo) / 2;
        const float* a = slab + (size_t)jj * lds;
        const int lo = half ? mid : ilo, hi = half ? max(ihi, mid) : mid;
        float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
        int i = lo;
        for (; i + 3 < hi; i += 4) {
            d0 = fmaf(col[i], a[i], d0);
            d1 = fmaf(col[i + 1], a[i + 1], d1);
            d2 = fmaf(col[i + 2], a[i + 2], d2);
            d3 = fmaf(col[i + 3], a[i + 3], d3);
        }
        for (; i < hi; ++i) d0 = fmaf(col[i], a[i], d0);
        part[half * QB + jj] = (d0 + d1) + (d2 + d3);
    }
    double s = 0.0;
    for (int i = tid; i < rpc; i += QP_THREADS) {
        const int gi = r0 + i;
        if (gi > c && gi < h) {
            const double x = col[i];
            s = fma(x, x, s);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) red[warp] = s;
    __syncthreads();
    if (half == 0 && jj < w) out(jj, part[jj] + part[QB + jj]);
    if (warp == 0) {
        double t = lane < QP_THREADS / 32 ? red[lane] : 0.0;
#pragma unroll
        for (int off = QP_THREADS / 64; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
        if (lane == 0) norm_out(t);
    }
}

// The reflector and its update on my rows (a thread per row): v = x * scale
// below the diagonal, beta on it; a_jj += coef_jj v for jj > c (coef = -tau
// (v . a_jj)), four columns at a time with the loads ahead of the stores.
__device__ __forceinline__ void panel_apply(float* slab, int lds, int rpc, int w, int c, int r0, int h, float scf,
                                            float betaf, const float* coef) {
    for (int i = threadIdx.x; i < rpc; i += QP_THREADS) {
        const int gi = r0 + i;
        if (gi < c || gi >= h) continue;
        float* const p = slab + i;
        float v = 1.f;
        if (gi == c) {
            p[(size_t)c * lds] = betaf;
        } else {
            v = p[(size_t)c * lds] * scf;
            p[(size_t)c * lds] = v;
        }
        int jj = c + 1;
        for (; jj + 3 < w; jj += 4) {
            float* const q0 = p + (size_t)jj * lds;
            const float a0 = q0[0], a1 = q0[lds], a2 = q0[2 * (size_t)lds], a3 = q0[3 * (size_t)lds];
            const float c0 = coef[jj], c1 = coef[jj + 1], c2 = coef[jj + 2], c3 = coef[jj + 3];
            q0[0] = fmaf(c0, v, a0);
            q0[lds] = fmaf(c1, v, a1);
            q0[2 * (size_t)lds] = fmaf(c2, v, a2);
            q0[3 * (size_t)lds] = fmaf(c3, v, a3);
        }
        for (; jj < w; ++jj) p[(size_t)jj * lds] = fmaf(coef[jj], v, p[(size_t)jj * lds]);
    }
}

// One grid barrier per column.  Before it every CTA publishes, for the rows
// below the diagonal, its partial sum of squares of the column x (FP64) and
// its partial dots of x with the panel's later columns a_j (fp32); the owner
// of the diagonal row publishes that row.  After it every CTA forms, in the
// same order, S = |x below c|^2, alpha = x_c, beta = -sign(alpha)
// sqrt(alpha^2 + S), tau = (beta - alpha) / beta and the scale 1 / (alpha -
// beta) (FP64), and v . a_j = a_j(c) + scale * (x . a_j) with v = x * scale
// below the diagonal and v_c = 1, so the dots need no second exchange.
// xp: [2][P][QB + 2] doubles by column parity (the norm partial, then the
// fp32 dot partials packed into the rest); drow: [2][QB] floats by parity,
// the diagonal row; tau (w doubles); V the explicit reflectors (h x w, ld
// ldv: 1 on the diagonal, 0 above).  On this part a warp instruction of the
// FP64 pipe costs about 70 cycles of its sub-partition, so the FP64 work per
// column is kept to a few instructions per CTA.
__global__ void __launch_bounds__(QP_THREADS, 1)
    qr_panel_f32_kernel(float* __restrict__ A, int lda, int m, int j0, int w, int rpc, float* __restrict__ V, int ldv,
                        double* __restrict__ tau, double* __restrict__ xp, float* __restrict__ drow, unsigned* bar,
                        float* __restrict__ gpart, int* err) {
    extern __shared__ __align__(16) float slab[];  // [w][lds], then the Gram tile [QG_ROWS][QB + 4]
    __shared__ float sh_part[2 * QB];              // the dots' halves
    __shared__ double red[QP_THREADS / 32];
    __shared__ float s_coef[QB];                   // -tau * (v . a_jj) for the update
    __shared__ double s_tau, s_beta, s_scal;
    const int P = gridDim.x, b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int h = m - j0;
    const int r0 = b * rpc, r1 = min(h, r0 + rpc);
    const int lds = rpc | 1;  // the slab's column stride
    float* const P0 = A + j0 + (size_t)j0 * lda;
    const int stride = QB + 2;
    for (int e = tid; e < w * rpc; e += QP_THREADS) {
        const int c = e / rpc, i = e - c * rpc;
        slab[(size_t)c * lds + i] = r0 + i < h ? P0[r0 + i + (size_t)c * lda] : 0.f;
    }
    __syncthreads();
    unsigned target = 0;
    bool ok = true;
    for (int c = 0; c < w && ok; ++c) {
        double* const xpc = xp + (size_t)(c & 1) * P * stride;
        float* const drc = drow + (c & 1) * QB;
        // 1. partials below the diagonal: sum of squares (FP64), dots with the
        //    later columns (fp32, a warp per column); the diagonal row (owner)
        {
            float* const xd = reinterpret_cast<float*>(xpc + (size_t)b * stride + 2);
            panel_dots_norm(
                slab, lds, rpc, w, c, r0, h, sh_part, red, [&](int jj, float d) { xd[jj] = d; },
                [&](double t) { xpc[(size_t)b * stride] = t; });
        }
        if (c >= r0 && c < r1)
            for (int jj = c + tid; jj < w; jj += QP_THREADS) drc[jj] = slab[(size_t)jj * lds + (c - r0)];
        target += P;
        ok = mg::grid_barrier(bar, target, err);
        if (!ok) break;
        // 2. S over the CTAs (a shuffle tree, fixed order), then beta, tau and
        //    the scale in FP64, identical in every CTA
        if (warp == 0) {
            double xn2 = 0.0;
            for (int u = lane; u < P; u += 32) xn2 += __ldcg(&xpc[(size_t)u * stride]);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) xn2 += __shfl_xor_sync(0xffffffffu, xn2, off);
            if (lane < 2) {  // tau (lane 0) and the scale (lane 1) in one division sequence
                const double alpha = (double)__ldcg(&drc[c]);
                double qv = 0.0, beta = alpha;  // nothing below the diagonal: H = I
                if (xn2 != 0.0) {
                    beta = -copysign(sqrt(fma(alpha, alpha, xn2)), alpha);
                    qv = (lane == 0 ? beta - alpha : 1.0) / (lane == 0 ? beta : alpha - beta);
                }
                if (lane == 0) {
                    s_tau = qv;
                    s_beta = beta;
                    if (b == 0) tau[c] = qv;
                } else {
                    s_scal = qv;
                }
            }
        }
        __syncthreads();
        const double tc = s_tau, sc = s_scal;
        // 3. v . a_jj = a_jj(c) + scale (x . a_jj), the CTAs' fp32 partials in a
        //    fixed order (a thread per column, the loads in flight together);
        //    the update's coefficient -tau (v . a_jj) in fp32
        {
            const float tcf = (float)tc, scf0 = (float)sc;
            for (int jj = c + 1 + tid; jj < w; jj += QP_THREADS) {
                const float* pc = reinterpret_cast<const float*>(xpc + 2) + jj;
                float d = 0.f;
#pragma unroll 8
                for (int u = 0; u < P; ++u) d += __ldcg(pc + (size_t)u * stride * 2);
                s_coef[jj] = -tcf * fmaf(scf0, d, __ldcg(&drc[jj]));
            }
        }
        __syncthreads();
        // 4. v below the diagonal, beta on it; a_jj -= (tau (v . a_jj)) v on my rows
        panel_apply(slab, lds, rpc, w, c, r0, h, (float)sc, (float)s_beta, s_coef);
        __syncthreads();
    }
    gram_part(slab, w, lds, rpc, r0, h, gpart + (size_t)b * QB * QB);
    // write back: R (upper, diagonal = beta) and v below it; V explicit
    for (int e = tid; e < w * rpc; e += QP_THREADS) {
        const int c = e / rpc, i = e - c * rpc, gi = r0 + i;
        if (gi < h) {
            const float x = slab[(size_t)c * lds + i];
            P0[gi + (size_t)c * lda] = x;
            V[gi + (size_t)c * ldv] = gi < c ? 0.f : gi == c ? 1.f : x;
        }
    }
}

// ---- the cluster form of the panel: the same column steps on one 16-CTA
// thread-block cluster, for panels whose slab fits the cluster's shared
// memory.  The per-column exchange is a push instead of a grid barrier:
// every CTA stores its record (the sum of squares as a double, then the dot
// partials) with st.async into its slot of every CTA, the owner of the
// diagonal row stores that row too, and the bytes complete on each
// receiver's mbarrier (double-buffered by column parity: a CTA sends column
// c+2 only after receiving every record of column c+1, which every CTA
// sends only after its threads have finished reading column c's slots).
constexpr int QC_CS = 16;
constexpr int QC_REC = 4 + QB;  // floats per record: the double sum of squares, padding, the dots
// 16-byte chunks of a column's record (the double, padding, the w - c - 1
// dots) and of its diagonal row (w - c entries), and the bytes every CTA
// receives for the column: 16 records and the row.
__device__ __forceinline__ int qc_rec16(int w, int c) { return (4 + (w - c - 1) + 3) / 4; }
__device__ __forceinline__ int qc_diag16(int w, int c) { return (w - c + 3) / 4; }
__device__ __forceinline__ uint32_t qc_rx_bytes(int w, int c) {
    return (uint32_t)(16 * (QC_CS * qc_rec16(w, c) + qc_diag16(w, c)));
}

struct QcShared {
    __align__(16) float recv[2][QC_CS][QC_REC];  // every CTA's record of the column, by parity
    __align__(16) float recv_diag[2][QB];        // the diagonal row, by parity
    __align__(8) uint64_t mbar[2];
    __align__(16) float rec[QC_REC];             // this CTA's record, staged
    __align__(16) float diag[QB];                // the diagonal row, staged by its owner
    float coef[QB];
    double red[QP_THREADS / 32];
    double tau, beta, scal;
};

__global__ void __launch_bounds__(QP_THREADS, 1)
    qr_panel_cluster_kernel(float* __restrict__ A, int lda, int m, int j0, int w, int rpc, float* __restrict__ V,
                            int ldv, double* __restrict__ tau, float* __restrict__ gpart, int* err) {
    extern __shared__ __align__(16) float slab[];  // [w][lds], then the Gram tile
    __shared__ float sh_part[2 * QB];              // the dots' halves
    __shared__ QcShared qs;
    cg::cluster_group cluster = cg::this_cluster();
    const int q = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int h = m - j0;
    const int r0 = q * rpc, r1 = min(h, r0 + rpc);
    const int lds = rpc | 1;  // the slab's column stride
    float* const P0 = A + j0 + (size_t)j0 * lda;
    for (int e = tid; e < w * rpc; e += QP_THREADS) {
        const int c = e / rpc, i = e - c * rpc;
        slab[(size_t)c * lds + i] = r0 + i < h ? P0[r0 + i + (size_t)c * lda] : 0.f;
    }
    if (tid == 0) {
        tc::mbar_init(&qs.mbar[0], 1);
        tc::mbar_init(&qs.mbar[1], 1);
        tc::fence_barrier_init();
        tc::mbar_arrive_expect_tx(&qs.mbar[0], qc_rx_bytes(w, 0));
        if (w > 1) tc::mbar_arrive_expect_tx(&qs.mbar[1], qc_rx_bytes(w, 1));
    }
    cluster.sync();  // the slab is loaded and every CTA's barriers are armed
    bool rx_failed = false;  // warp 0: a receive wait gave up (error recorded; later waits skipped)
    for (int c = 0; c < w; ++c) {
        const int buf = c & 1;
        const bool owner = c >= r0 && c < r1;
        // 1. the record: dots of the unscaled column with the later columns
        //    (fp32, a warp per column), sum of squares (FP64); the diagonal row
        panel_dots_norm(
            slab, lds, rpc, w, c, r0, h, sh_part, qs.red, [&](int jj, float d) { qs.rec[4 + (jj - c - 1)] = d; },
            [&](double t) { *reinterpret_cast<double*>(&qs.rec[0]) = t; });
        if (owner)
            for (int jj = c + tid; jj < w; jj += QP_THREADS) qs.diag[jj - c] = slab[(size_t)jj * lds + (c - r0)];
        __syncthreads();
        // 2. every thread pushes a share of the record into slot [q] of every
        //    CTA (16-byte chunk u to CTA d for e = u * 16 + d), and the owner's
        //    threads the diagonal row; only the columns still ahead travel:
        //    the record's dots and the row's entries are packed from column
        //    c + 1 and c on
        {
            const float4* r4 = reinterpret_cast<const float4*>(qs.rec);
            const int n16 = qc_rec16(w, c);
            for (int e = tid; e < n16 * QC_CS; e += QP_THREADS) {
                const int u = e / QC_CS, d = e - u * QC_CS;
                tc::st_async16(tc::cluster_addr(&qs.recv[buf][q][0], d) + 16u * u, r4[u],
                               tc::cluster_addr(&qs.mbar[buf], d));
            }
            if (owner) {
                const float4* d4 = reinterpret_cast<const float4*>(qs.diag);
                const int nd = qc_diag16(w, c);
                for (int e = tid; e < nd * QC_CS; e += QP_THREADS) {
                    const int u = e / QC_CS, d = e - u * QC_CS;
                    tc::st_async16(tc::cluster_addr(&qs.recv_diag[buf][0], d) + 16u * u, d4[u],
                                   tc::cluster_addr(&qs.mbar[buf], d));
                }
            }
        }
        if (warp == 0) {
            // 3. wait for the 16 records and the diagonal row; S over the CTAs
            //    (a shuffle tree, fixed order), then beta, tau and the scale (FP64)
            int ok = 1;
            if (lane == 0) {
                ok = rx_failed ? 0 : (tc::mbar_wait_cluster(&qs.mbar[buf], (uint32_t)((c >> 1) & 1)) ? 1 : 0);
                if (!ok && !rx_failed) atomicExch(err, 8 /* MG_TIMEOUT */);
                if (ok && c + 2 < w) tc::mbar_arrive_expect_tx(&qs.mbar[buf], qc_rx_bytes(w, c + 2));
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) rx_failed = true;
            __syncwarp();
            double xs = lane < QC_CS ? *reinterpret_cast<const double*>(&qs.recv[buf][lane][0]) : 0.0;
#pragma unroll
            for (int off = QC_CS / 2; off > 0; off >>= 1) xs += __shfl_xor_sync(0xffffffffu, xs, off);
            if (lane < 2) {  // tau (lane 0) and the scale (lane 1) in one division sequence
                const double alpha = (double)qs.recv_diag[buf][0];
                double qv = 0.0, beta = alpha;  // nothing below the diagonal: H = I
                if (xs != 0.0) {
                    beta = -copysign(sqrt(fma(alpha, alpha, xs)), alpha);
                    qv = (lane == 0 ? beta - alpha : 1.0) / (lane == 0 ? beta : alpha - beta);
                }
                if (lane == 0) {
                    qs.tau = qv;
                    qs.beta = beta;
                    if (q == 0) tau[c] = qv;
                } else {
                    qs.scal = qv;
                }
            }
        }
        __syncthreads();
        // 4. v . a_jj = a_jj(c) + scale (x . a_jj) from the 16 records (fixed
        //    order); the update's coefficient -tau (v . a_jj) in fp32
        {
            const float tcf = (float)qs.tau, scf0 = (float)qs.scal;
            for (int jj = c + 1 + tid; jj < w; jj += QP_THREADS) {
                float d = 0.f;
#pragma unroll
                for (int u = 0; u < QC_CS; ++u) d += qs.recv[buf][u][4 + (jj - c - 1)];
                qs.coef[jj] = -tcf * fmaf(scf0, d, qs.recv_diag[buf][jj - c]);
            }
        }
        __syncthreads();
        // 5. v below the diagonal, beta on it; a_jj -= (tau (v . a_jj)) v on my rows
        panel_apply(slab, lds, rpc, w, c, r0, h, (float)qs.scal, (float)qs.beta, qs.coef);
        __syncthreads();
    }
    gram_part(slab, w, lds, rpc, r0, h, gpart + (size_t)q * QB * QB);
    for (int e = tid; e < w * rpc; e += QP_THREADS) {
        const int c = e / rpc, i = e - c * rpc, gi = r0 + i;
        if (gi < h) {
            const float x = slab[(size_t)c * lds + i];
            P0[gi + (size_t)c * lda] = x;
            V[gi + (size_t)c * ldv] = gi < c ? 0.f : gi == c ? 1.f : x;
        }
    }
    cluster.sync();  // no CTA leaves while another may still store into its shared memory
}

// G (QB x QB, ld QB) = the sum of the panel CTAs' parts, in a fixed order.
__global__ void qr_gsum_kernel(const float* __restrict__ gpart, int nparts, float* __restrict__ G) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= QB * QB) return;
    float s = 0.f;
    for (int u = 0; u < nparts; ++u) s += gpart[(size_t)u * QB * QB + e];
    G[e] = s;
}

// T (w x w, upper, fp32, ld QB) of H_0 ... H_{w-1} = I - V T V^T from
// G = V^T V and the taus.  LAPACK's recurrence T(c,c) = tau_c, T(0:c, c) =
// -tau_c T(0:c, 0:c) G(0:c, c) says that T is the inverse of the upper
// triangular U = striu(G) + diag(1 / tau) (column c of T U is e_c).  The
// kernel inverts U right-looking, by the column operations that turn U
// into I applied to I: with C_j the j-th column before scaling (T_j =
// tau_j C_j), C_k = e_k - sum_{j<k} tau_j G(j, k) C_j, so once column j is
// final every later column subtracts tau_j G(j, k) times it; a rank-1 step
// per column, one CTA barrier each, instead of a dot-product chain per
// column.  512 threads hold the 128 x 128 C in registers: warp wi the
// columns wi, wi+16, .., lane l the rows l, l+32, l+64, l+96; the columns
// sit in a window rotated once per 16 steps (static register indices in a
// rolled loop), and the owner of column j publishes it to shared memory.
// The scaling by tau waits until the end.  fp32 throughout (T is an fp32
// factor; an FP64 recurrence here cost ~1 ms per panel).  Columns and rows
// from w on are zero.
constexpr int TF_THREADS = 512;

__global__ void __launch_bounds__(TF_THREADS) qr_tfactor_kernel(const float* __restrict__ G, int ldg,
                                                                const double* __restrict__ tau, int w,
                                                                float* __restrict__ T) {
    extern __shared__ float ms[];  // tau_j G(j, k) at ms[k * QB + j], j < k < w
    __shared__ float colv[2][QB];
    const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
    {
        constexpr int PER = QB * QB / TF_THREADS;
        float g[PER];
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int e = threadIdx.x + u * TF_THREADS, j = e % QB, k = e / QB;
            g[u] = (j < k && k < w) ? (float)tau[j] * G[j + (size_t)k * ldg] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < PER; ++u) ms[threadIdx.x + u * TF_THREADS] = g[u];
    }
    float a[4][8];  // C(lane + 32 q, column of window position p)
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 8; ++p) a[q][p] = (lane + 32 * q == wi + 16 * p) ? 1.f : 0.f;
    __syncthreads();
#pragma unroll 1
    for (int jm = 0; jm < 8; ++jm) {
        const int nlive = 7 - jm;  // window positions 1 .. nlive hold columns after this group of 16
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) {
            const int j = 16 * jm + jj;
            float* const cv = colv[jj & 1];
            if (wi == jj) {
#pragma unroll
                for (int q = 0; q < 4; ++q) cv[lane + 32 * q] = a[q][0];
            }
            __syncthreads();  // column j published; the buffer of column j-1 stays readable
            float cj[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) cj[q] = cv[lane + 32 * q];
            if (wi > jj) {  // window position 0 is column wi + 16 jm, after j
                const float mk = ms[(wi + 16 * jm) * QB + j];
#pragma unroll
                for (int q = 0; q < 4; ++q) a[q][0] = fmaf(-mk, cj[q], a[q][0]);
            }
#pragma unroll
            for (int p = 1; p < 8; ++p) {
                if (p <= nlive) {
                    const float mk = ms[(wi + 16 * (jm + p)) * QB + j];
#pragma unroll
                    for (int q = 0; q < 4; ++q) a[q][p] = fmaf(-mk, cj[q], a[q][p]);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {  // rotate the window: the next group's column first
            const float t0 = a[q][0];
#pragma unroll
            for (int p = 0; p < 7; ++p) a[q][p] = a[q][p + 1];
            a[q][7] = t0;
        }
    }
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        const int c = wi + 16 * p;
        const float tc = c < w ? (float)tau[c] : 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = lane + 32 * q;
            T[i + (size_t)QB * c] = (i < w && c < w && i <= c) ? tc * a[q][p] : 0.f;
        }
    }
}

// ---- Q^T applied to X (n x nrhs, FP64) with the fp32 reflectors of one panel
// (A32 below the diagonal of columns j0 .. j0+w, v_c = 1) and its T, in FP64:
// X(j0:, :) -= V (T^T (V^T X(j0:, :))).
constexpr int QT_CTAS = 64;

__global__ void qt_dots_kernel(const float* __restrict__ A, int lda, int m, int j0, int w, const double* __restrict__ X,
                               int ldx, int nrhs, double* __restrict__ part) {
    const int h = m - j0;
    const int chunk = (h + gridDim.x - 1) / gridDim.x;
    const int lo = blockIdx.x * chunk, hi = min(h, lo + chunk);
    for (int q = threadIdx.x; q < w * nrhs; q += blockDim.x) {
        const int c = q % w, j = q / w;
        const float* v = A + j0 + (size_t)(j0 + c) * lda;
        const double* x = X + j0 + (size_t)j * ldx;
        double d = 0.0;
        for (int i = max(lo, c); i < hi; ++i) d = fma(i == c ? 1.0 : (double)v[i], x[i], d);
        part[(size_t)blockIdx.x * w * nrhs + q] = d;
    }
}

__global__ void qt_tw_kernel(const double* __restrict__ part, int nparts, const float* __restrict__ T, int w, int nrhs,
                             double* __restrict__ y) {
    __shared__ double wv[QB * 8];
    for (int q = threadIdx.x; q < w * nrhs; q += blockDim.x) {
        double d = 0.0;
        for (int u = 0; u < nparts; ++u) d += part[(size_t)u * w * nrhs + q];
        wv[q] = d;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < w * nrhs; q += blockDim.x) {
        const int c = q % w, j = q / w;
        double d = 0.0;
        for (int k = 0; k <= c; ++k) d = fma((double)T[k + (size_t)c * QB], wv[k + j * w], d);  // (T^T w)_c
        y[q] = d;
    }
}

__global__ void qt_update_kernel(const float* __restrict__ A, int lda, int m, int j0, int w, const double* __restrict__ y,
                                 int nrhs, double* __restrict__ X, int ldx) {
    const int h = m - j0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < h; i += gridDim.x * blockDim.x) {
        const int cmax = min(w - 1, i);
        for (int j = 0; j < nrhs; ++j) {
            double acc = X[j0 + i + (size_t)j * ldx];
            for (int c = 0; c <= cmax; ++c) {
                const double v = c == i ? 1.0 : (double)A[j0 + i + (size_t)(j0 + c) * lda];
                acc = fma(-v, y[c + j * w], acc);
            }
            X[j0 + i + (size_t)j * ldx] = acc;
        }
    }
}

// ---- the same Q^T in fp32 for the refinement's correction (a scaled
// residual, as the LU's correction is solved in fp32): X (n x nrhs, ld ldx,
// nrhs <= 8) := (I - V T^T V^T) X panel after panel, in ONE cooperative grid
// (per panel a launch of three small kernels cost ~70 us, launch-bound).
// CTA b owns the rows [b * chunk, (b + 1) * chunk) of X for every panel.  Per
// panel: (1) partial dots V^T X over my rows (a warp per reflector, lanes over
// rows), (2) after a grid barrier each CTA adds up a share of the entries of
// W = V^T X over the CTAs' partials (a fixed order), (3) after another, every
// CTA forms y = T^T W and updates its rows (32 rows x 8 reflector groups per
// step, the groups' sums added in shared memory).  Partials and W are
// double-buffered by panel parity.
__global__ void __launch_bounds__(256) qt32_fused_kernel(const float* __restrict__ A, int lda, int n,
                                                         const float* __restrict__ T, float* __restrict__ X, int ldx,
                                                         int nrhs, float* __restrict__ part, float* __restrict__ W,
                                                         unsigned* bar, int* err) {
    extern __shared__ float tsm[];   // the panel's T block (QB x QB, column-major)
    __shared__ float ys[QB * 8];
    __shared__ float wsm[QB * 8];    // W = V^T X of the panel
    __shared__ float red[8][8][33];  // [group][rhs][row]
    const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int chunk = (n + G - 1) / G, lo = b * chunk, hi = min(n, lo + chunk);
    unsigned target = 0;
    for (int j0 = 0, pn = 0; j0 < n; j0 += QB, ++pn) {
        const int w = min(QB, n - j0);
        float* const pp = part + (size_t)(pn & 1) * G * QB * 8;
        float* const wp = W + (size_t)(pn & 1) * QB * 8;
        // 1. this CTA's partial dots over its rows at or below the panel's diagonal
        for (int c = warp; c < w; c += 8) {
            const float* v = A + j0 + (size_t)(j0 + c) * lda;  // v_c at row i: v[i - j0]
            float acc[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] = 0.f;
            for (int i = max(lo, j0 + c) + lane; i < hi; i += 32) {
                const float vi = i == j0 + c ? 1.f : v[i - j0];
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (j < nrhs) acc[j] = fmaf(vi, X[i + (size_t)j * ldx], acc[j]);
            }
            // the 8 sums over the warp by halving exchanges (4 + 2 + 1 shuffles
            // leave lane l with right-hand side (l >> 2) & 7 summed over 8
            // lanes, two more levels finish it): a fixed order
#pragma unroll
            for (int h = 4, off = 16; h >= 1; h >>= 1, off >>= 1) {
                const bool up = (lane & off) != 0;
#pragma unroll
                for (int j = 0; j < h; ++j) {
                    const float send = up ? acc[j] : acc[j + h];
                    const float keep = up ? acc[j + h] : acc[j];
                    acc[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
                }
            }
            acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], 2);
            acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], 1);
            if ((lane & 3) == 0) pp[((size_t)b * QB + c) * 8 + ((lane >> 2) & 7)] = acc[0];
        }
        target += G;
        if (!mg::grid_barrier(bar, target, err)) return;
        // 2. W's entries dealt to the grid's warps: lane l sums the partials
        //    of CTAs l, l + 32, ... (all its loads in flight together), then a
        //    shuffle tree; a fixed order either way
        for (int e = b * 8 + warp; e < w * 8; e += G * 8) {
            float sum = 0.f;
            for (int u = lane; u < G; u += 32) sum += __ldcg(pp + (size_t)u * QB * 8 + e);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
            if (lane == 0) wp[e] = sum;
        }
        target += G;
        if (!mg::grid_barrier(bar, target, err)) return;
        // 3. y = T^T W from T and W staged in shared memory, then X -= V y on my rows
        const float* Tb = T + (size_t)(j0 / QB) * QB * QB;
        {
            float4 tv[QB * QB / 4 / 256];  // the whole T block, all loads in flight
            const float4* Tb4 = reinterpret_cast<const float4*>(Tb);
#pragma unroll
            for (int u = 0; u < QB * QB / 4 / 256; ++u) tv[u] = __ldg(Tb4 + tid + u * 256);
#pragma unroll
            for (int u = 0; u < QB * QB / 4 / 256; ++u) reinterpret_cast<float4*>(tsm)[tid + u * 256] = tv[u];
        }
        for (int q = tid; q < w * 8; q += blockDim.x) wsm[q] = __ldcg(wp + q);
        __syncthreads();
        for (int q = tid; q < w * 8; q += blockDim.x) {
            const int c = q / 8, j = q % 8;
            float d = 0.f;
            if (j < nrhs)
                for (int k = 0; k <= c; ++k) d = fmaf(tsm[k + c * QB], wsm[k * 8 + j], d);
            ys[q] = d;
        }
        __syncthreads();
        const int rl = tid & 31, g = tid >> 5;
        for (int i0 = max(lo, j0); i0 < hi; i0 += 32) {
            const int i = i0 + rl;
            float acc[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] = 0.f;
            if (i < hi) {
                const int cmax = min(w - 1, i - j0);
                for (int c = g; c <= cmax; c += 8) {
                    const float v = c == i - j0 ? 1.f : A[i + (size_t)(j0 + c) * lda];
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[j] = fmaf(v, ys[c * 8 + j], acc[j]);
                }
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) red[g][j][rl] = acc[j];
            __syncthreads();
            if (g == 0 && i < hi) {
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    if (j >= nrhs) break;
                    float sum = 0.f;
#pragma unroll
                    for (int gg = 0; gg < 8; ++gg) sum += red[gg][j][rl];
                    X[i + (size_t)j * ldx] -= sum;
                }
            }
            __syncthreads();
        }
    }
}

__global__ void copy_f64_kernel(int n, int nrhs, const double* __restrict__ B, int ldb, double* __restrict__ X,
                                int ldx) {
    const size_t total = (size_t)n * nrhs;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        X[(e % n) + (e / n) * (size_t)ldx] = B[(e % n) + (e / n) * (size_t)ldb];
}

}  // namespace

namespace mg {

size_t qr_mixed_ws_bytes(int m, int n, int num_sms) {
    const int P = num_sms;
    return align_up((size_t)m * QB * sizeof(float), 1024)                  // V
           + align_up((size_t)QB * n * sizeof(float), 1024) * 2             // W, W2
           + align_up((size_t)QB * QB * sizeof(float), 1024)                // G
           + align_up((size_t)P * QB * QB * sizeof(float), 1024)            // the panel CTAs' parts of G
           + align_up((size_t)2 * P * (QB + 2) * sizeof(double), 1024)      // panel partials (by parity)
           + align_up((size_t)QT_CTAS * QB * 8 * sizeof(double), 1024)      // Q^T partials
           + align_up((size_t)QB * 8 * sizeof(double), 1024)                // T^T w
           + 4096;                                                          // barrier, diagonal rows, error
}

// In-place FP32 Householder QR of the m x n (m >= n) matrix A (ld lda):
// R on and above the diagonal, the reflectors below it (v_c = 1 implicit);
// tau (n doubles), T (ceil(n / QB) blocks of QB x QB fp32).  ws holds
// qr_mixed_ws_bytes(m, n, num_sms); err receives MG_TIMEOUT from a panel wait.
mg_status_t sgeqrf_mixed(mg_handle_t h, int m, int n, float* A, int lda, double* tau, float* T, void* ws, int* err) {
    if (n == 0) return MG_OK;
    const int P0max = h->num_sms;
    char* p = (char*)ws;
    auto take = [&](size_t bytes) { char* q = p; p += align_up(bytes, 1024); return q; };
    float* V = (float*)take((size_t)m * QB * sizeof(float));
    float* W = (float*)take((size_t)QB * n * sizeof(float));
    float* W2 = (float*)take((size_t)QB * n * sizeof(float));
    float* G = (float*)take((size_t)QB * QB * sizeof(float));
    float* gpart = (float*)take((size_t)P0max * QB * QB * sizeof(float));
    double* xp = (double*)take((size_t)2 * P0max * (QB + 2) * sizeof(double));
    take((size_t)QT_CTAS * QB * 8 * sizeof(double));
    take((size_t)QB * 8 * sizeof(double));
    unsigned* bar = (unsigned*)p;
    float* drow = (float*)(p + 256);  // [2][QB]
    const cudaStream_t st = h->stream;
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(qr_panel_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          h->max_smem_optin - 4096));
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(qr_tfactor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(QB * QB * sizeof(float))));
    // the cluster form when a 16-CTA cluster's shared memory holds the panel
    const size_t qc_static = sizeof(QcShared) + 2048;  // + the other static shared arrays
    const size_t qc_max_dyn = (size_t)h->max_smem_optin > qc_static ? (size_t)h->max_smem_optin - qc_static : 0;
    bool qc_ok = false;
    {
        cudaLaunchAttribute at[1];
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(QC_CS);
        cfg.blockDim = dim3(QP_THREADS);
        cfg.dynamicSmemBytes = qc_max_dyn;
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = QC_CS;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        qc_ok = cudaFuncSetAttribute(qr_panel_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                    cudaSuccess &&
                cudaFuncSetAttribute(qr_panel_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)qc_max_dyn) == cudaSuccess &&
                cudaOccupancyMaxActiveClusters(&nclusters, qr_panel_cluster_kernel, &cfg) == cudaSuccess &&
                nclusters > 0;
        if (!qc_ok) cudaGetLastError();
    }
    for (int j0 = 0; j0 < n; j0 += QB) {
        const int w = n - j0 < QB ? n - j0 : QB;
        const int hgt = m - j0;
        const int qc_rpc = (hgt + QC_CS - 1) / QC_CS;
        const size_t qc_smem = (size_t)(qc_rpc | 1) * w * sizeof(float) + QG_TILE_BYTES;
        int nparts;  // CTAs of the panel (parts of V^T V)
        if (qc_ok && qc_smem <= qc_max_dyn) {
            ProfScope prof(h, "qr_panel_f32", 4.0 * hgt * (double)w * w / 2, 8.0 * hgt * (double)w);
            cudaLaunchAttribute at[1];
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(QC_CS);
            cfg.blockDim = dim3(QP_THREADS);
            cfg.dynamicSmemBytes = qc_smem;
            cfg.stream = st;
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = QC_CS;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            const cudaError_t e = cudaLaunchKernelEx(&cfg, qr_panel_cluster_kernel, A, lda, m, j0, w, qc_rpc, V, hgt,
                                                     tau + j0, gpart, err);
            if (e != cudaSuccess) return cuda_fail(h, e, "qr_panel_cluster_kernel launch");
            h->launches++;
            nparts = QC_CS;
        } else {
            int P = (hgt + 255) / 256;
            if (P > P0max) P = P0max;
            int rpc = (hgt + P - 1) / P;
            while ((size_t)(rpc | 1) * w * sizeof(float) + QG_TILE_BYTES > (size_t)h->max_smem_optin - 4096 && P < P0max) {
                ++P;
                rpc = (hgt + P - 1) / P;
            }
            const size_t smem = (size_t)(rpc | 1) * w * sizeof(float) + QG_TILE_BYTES;
            if (smem > (size_t)h->max_smem_optin - 4096)
                return fail(h, MG_ERR_UNSUPPORTED, "sgeqrf_mixed: panel of %d rows does not fit the SMs", hgt);
            ProfScope prof(h, "qr_panel_f32", 4.0 * hgt * (double)w * w / 2, 8.0 * hgt * (double)w);
            MG_CHECK_CUDA(h, cudaMemsetAsync(bar, 0, sizeof(unsigned), st));
            int lda_ = lda, m_ = m, j0_ = j0, w_ = w, rpc_ = rpc, ldv = hgt;
            float* A_ = A;
            double* tau_ = tau + j0;
            void* args[] = {&A_, &lda_, &m_, &j0_, &w_, &rpc_, &V, &ldv, &tau_, &xp, &drow, &bar, &gpart, &err};
            const cudaError_t e = cudaLaunchCooperativeKernel((const void*)qr_panel_f32_kernel, dim3(P),
                                                              dim3(QP_THREADS), args, smem, st);
            if (e != cudaSuccess) return cuda_fail(h, e, "qr_panel_f32_kernel launch");
            h->launches++;
            nparts = P;
        }
        float* Tb = T + (size_t)(j0 / QB) * QB * QB;
        qr_gsum_kernel<<<QB * QB / 256, 256, 0, st>>>(gpart, nparts, G);
        MG_TRY(post_launch(h, "qr_gsum_kernel"));
        qr_tfactor_kernel<<<1, TF_THREADS, QB * QB * sizeof(float), st>>>(G, QB, tau + j0, w, Tb);
        MG_TRY(post_launch(h, "qr_tfactor_kernel"));
        const int nt = n - j0 - w;
        if (nt > 0) {  // R2 -= V (T^T (V^T R2))
            float* R2 = A + j0 + (size_t)(j0 + w) * lda;
            MG_TRY(sgemm_auto(h, 1, 0, w, nt, hgt, 1.f, V, hgt, R2, lda, 0.f, W, QB, 0));
            MG_TRY(sgemm_auto(h, 1, 0, w, nt, w, 1.f, Tb, QB, W, QB, 0.f, W2, QB, 0));
            MG_TRY(sgemm_auto(h, 0, 0, hgt, nt, w, -1.f, V, hgt, W2, QB, 1.f, R2, lda, 0));
        }
    }
    return MG_OK;
}

// X (fp32, n x nrhs, ld ldx, nrhs <= 8) := Q^T X for the fp32 factors of
// sgeqrf_mixed (square: m = n), in fp32.
mg_status_t qr_apply_qt_f32(mg_handle_t h, int n, int nrhs, const float* A, int lda, const float* T, float* X, int ldx,
                            void* ws, int* err) {
    if (n == 0 || nrhs == 0) return MG_OK;
    if (nrhs > 8) return fail(h, MG_ERR_ARG, "qr_apply_qt_f32: at most 8 right-hand sides");
    char* p = (char*)ws;
    auto take = [&](size_t bytes) { char* q = p; p += align_up(bytes, 1024); return q; };
    take((size_t)n * QB * sizeof(float));
    take((size_t)QB * n * sizeof(float));
    take((size_t)QB * n * sizeof(float));
    take((size_t)QB * QB * sizeof(float));
    float* part = (float*)take((size_t)h->num_sms * QB * QB * sizeof(float));  // the V^T V parts' area
    take((size_t)2 * h->num_sms * (QB + 2) * sizeof(double));
    float* W = (float*)take((size_t)QT_CTAS * QB * 8 * sizeof(double));
    take((size_t)QB * 8 * sizeof(double));
    unsigned* bar = (unsigned*)p;  // the workspace tail's barrier word
    const cudaStream_t st = h->stream;
    const int G = h->num_sms;        // one CTA per SM (2 x G x QB x 8 partials fit the V^T V parts' area)
    int per_sm = 0;
    const size_t tsm_bytes = (size_t)QB * QB * sizeof(float);
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(qt32_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)tsm_bytes));
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, qt32_fused_kernel, 256, tsm_bytes) != cudaSuccess ||
        per_sm < 1)
        return fail(h, MG_ERR_UNSUPPORTED, "qr_apply_qt_f32: the cooperative grid does not fit");
    MG_CHECK_CUDA(h, cudaMemsetAsync(bar, 0, sizeof(unsigned), st));
    int n_ = n, lda_ = lda, ldx_ = ldx, nrhs_ = nrhs;
    void* args[] = {(void*)&A, &lda_, &n_, (void*)&T, (void*)&X, &ldx_, &nrhs_, (void*)&part, (void*)&W, (void*)&bar,
                    (void*)&err};
    const cudaError_t e =
        cudaLaunchCooperativeKernel((const void*)qt32_fused_kernel, dim3(G), dim3(256), args, tsm_bytes, st);
    if (e != cudaSuccess) return cuda_fail(h, e, "qt32_fused_kernel launch");
    h->launches++;
    return MG_OK;
}

// X := R^{-1} (Q^T B)(0:n) in FP64 for the fp32 factors of sgeqrf_mixed
// (square use: m = n): Q^T applied panel by panel, then the upper solve.
mg_status_t qr_solve_f32_factors(mg_handle_t h, int n, int nrhs, const float* A, int lda, const float* T,
                                 const double* B, int ldb, double* X, int ldx, void* ws) {
    if (n == 0 || nrhs == 0) return MG_OK;
    if (nrhs > 8) return fail(h, MG_ERR_ARG, "qr_solve_f32_factors: at most 8 right-hand sides");
    char* p = (char*)ws;
    auto take = [&](size_t bytes) { char* q = p; p += align_up(bytes, 1024); return q; };
    take((size_t)n * QB * sizeof(float));
    take((size_t)QB * n * sizeof(float));
    take((size_t)QB * n * sizeof(float));
    take((size_t)QB * QB * sizeof(float));
    take((size_t)h->num_sms * QB * QB * sizeof(float));
    take((size_t)2 * h->num_sms * (QB + 2) * sizeof(double));
    double* part = (double*)take((size_t)QT_CTAS * QB * 8 * sizeof(double));
    double* y = (double*)take((size_t)QB * 8 * sizeof(double));
    const cudaStream_t st = h->stream;
    const int cap = h->num_sms * 8;
    int g = (int)(((size_t)n * nrhs + 255) / 256);
    copy_f64_kernel<<<g < cap ? g : cap, 256, 0, st>>>(n, nrhs, B, ldb, X, ldx);
    MG_TRY(post_launch(h, "copy_f64_kernel"));
    for (int j0 = 0; j0 < n; j0 += QB) {
        const int w = n - j0 < QB ? n - j0 : QB;
        qt_dots_kernel<<<QT_CTAS, 256, 0, st>>>(A, lda, n, j0, w, X, ldx, nrhs, part);
        MG_TRY(post_launch(h, "qt_dots_kernel"));
        qt_tw_kernel<<<1, 256, 0, st>>>(part, QT_CTAS, T + (size_t)(j0 / QB) * QB * QB, w, nrhs, y);
        MG_TRY(post_launch(h, "qt_tw_kernel"));
        int gu = (n - j0 + 255) / 256;
        qt_update_kernel<<<gu < cap ? gu : cap, 256, 0, st>>>(A, lda, n, j0, w, y, nrhs, X, ldx);
        MG_TRY(post_launch(h, "qt_update_kernel"));
    }
    return upper_solve_f32_factors(h, n, nrhs, A, lda, X, ldx);
}

}  // namespace mg

extern "C" mg_status_t mg_sgeqrf(mg_handle_t h, int m, int n, float* A, int lda, double* tau, float* T) {
    if (!h) return MG_ERR_ARG;
    if (m < 0 || n < 0 || m < n || lda < (m > 1 ? m : 1) || (n && (!A || !tau || !T)))
        return mg::fail(h, MG_ERR_ARG, "mg_sgeqrf: bad arguments (m=%d n=%d lda=%d; m >= n)", m, n, lda);
    if (n == 0) return MG_OK;
    const size_t wsb = mg::qr_mixed_ws_bytes(m, n, h->num_sms);
    MG_TRY(mg::ensure_ws(h, wsb + 256));
    MG_TRY(mg::ensure_hws(h, 64));
    int* err = (int*)((char*)h->ws + wsb);
    MG_CHECK_CUDA(h, cudaMemsetAsync(err, 0, sizeof(int), h->stream));
    MG_TRY(mg::sgeqrf_mixed(h, m, n, A, lda, tau, T, h->ws, err));
    int* hw = (int*)h->hws;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw, err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hw[0]) return mg::fail(h, MG_TIMEOUT, "mg_sgeqrf: a panel grid barrier timed out");
    int terr = 0;
    MG_TRY(mg::tc_sgemm_error(h, &terr));
    if (terr) return mg::fail(h, MG_TIMEOUT, "mg_sgeqrf: a tensor-core update's bounded wait gave up");
    return MG_OK;
}
