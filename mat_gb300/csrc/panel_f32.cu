// FP32 panel factorization (getf2: partial pivoting, first index of the
// largest |a|, reciprocal scaling, fused rank-1 updates) on ONE thread-block
// cluster, for the mixed-precision LU.
//
// Why a cluster: a panel column needs one all-CTA agreement on the pivot.
// Through global memory (a grid barrier over ~128 CTAs) that costs several
// L2 round trips per column, ~4.5 us; inside a 16-CTA cluster each CTA pushes
// its candidate into every CTA's shared memory and waits on a local barrier.
// A 16-CTA cluster cannot hold a 16384 x 128 FP32 panel (8 MiB) on chip, so
// the panel is factored in sub-panels of 16 columns kept in registers
// (each of the 256 threads of a CTA owns RPT <= 4 rows x 16 columns; the
// fully unrolled column loop of a 16-column sub-panel stays small enough for
// the instruction cache):
//
//   for each sub-panel S = [cs0, cs0+16):
//     1. load my rows of S into registers
//     2. for each column c of S: local max |a| (warp redux), each warp's
//        winner row into shared memory -> warp 0 forms the CTA's 80-byte
//        record (row, |a| bits, position) and stores it with st.async into
//        slot [my rank] of every CTA (the diagonal row's owner also sends
//        that row), completing bytes on the receiver's mbarrier -> wait on
//        the local mbarrier for 16 records + the diagonal row -> the same
//        winner in every CTA -> swap in registers -> scale by the reciprocal
//        -> fused rank-1 update of my rows' remaining columns
//     3. store S; apply S's interchanges to the panel's other columns and to
//        pos (one gather/scatter over the touched rows, net permutation kept
//        in a shared-memory map)
//     4. U(S, right) = L11^{-1} A(S, right) (16 x 16 unit lower, every CTA
//        redundantly), then A(below, right) -= L(below, S) U(S, right) for my
//        rows, with L(below, S) still in registers.
//
// Every element sees the same fused operations in the same order as the
// column-at-a-time panel (the multiplier l = a * (1/p), then a := fma(l, -u,
// a) for the pivot columns in increasing order), so the factors are bitwise
// those of the one-column-per-barrier cooperative panel.  Pivot rows are
// identical as well (same comparisons on the same values).
//
// Receive slots and mbarriers are double-buffered by column parity: a CTA
// sends its record for column c+2 only after receiving every record of
// column c+1, and every CTA sends that only after it has consumed its slots of
// column c and re-armed their mbarrier (expect 1344 bytes).  Waits are
// bounded: on a timeout the kernel records MG_TIMEOUT, skips later waits and
// runs on to the end, so every CTA executes the same cluster barriers.
// Global loads inside the kernel go to L2 (__ldcg): rows of the panel are
// rewritten by other CTAs of the cluster (the interchanges are dealt out by
// column), and an SM's L1 is not coherent with their stores.
#include <cooperative_groups.h>

#include <climits>

#include "mg_internal.cuh"
#include "tc_common.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int CP_THREADS = 256;
constexpr int CP_CS = 16;         // CTAs per cluster (non-portable size)
constexpr int CP_MAX_RPT = 4;     // rows per thread
constexpr int CP_SW = 16;       // sub-panel width (columns in registers)
constexpr int CP_MAXW = 128;    // widest panel
constexpr int CP_NOTHER = CP_MAXW - CP_SW;
constexpr int CP_UB_LD = CP_SW + 4;  // padded row of ub (16-byte multiple)
constexpr int CP_GCOLS = 8;          // columns per gather pass (>= 112 / 16)

// One CTA's pivot candidate for a column as read by the other CTAs: the row
// (its sub-panel columns), |a| as bits (non-negative floats order like their
// bit patterns) and the position; 80 bytes, read as five 16-byte loads.
struct __align__(16) CpRec {
    float row[CP_SW];
    unsigned bits;
    int pos;
    int pad[2];
};

struct CpShared {
    float ub[CP_NOTHER][CP_UB_LD];  // U(S, right), [column][row of S]
    float l11[CP_SW][CP_SW + 1];
    CpRec recv[2][CP_CS];            // every CTA's candidate for the column, by column parity
    __align__(16) float recv_diag[2][CP_SW];  // the row at the diagonal (sent by its owner)
    __align__(8) uint64_t mbar[2];            // receive barriers (transaction bytes), by parity
    __align__(16) float pubdiag[2][CP_SW];
    __align__(16) float prow[2][CP_SW];  // the pivot row of a column, by parity
    __align__(16) float drow[2][CP_SW];  // the row at the diagonal, by parity
    __align__(16) float wrow[CP_THREADS / 32][CP_SW];  // each warp's candidate row
    unsigned wbits[CP_THREADS / 32];
    int wpos[CP_THREADS / 32];
    int piv[CP_MAXW];
    int touch[2 * CP_SW];
    float gbuf[CP_GCOLS * 2 * CP_SW];
    int gpos[2 * CP_SW];
    int s_win[2];
    float s_pv[2];
};

// Bytes each CTA receives per column: 16 records and the diagonal row.
constexpr uint32_t CP_RX_BYTES = CP_CS * sizeof(CpRec) + CP_SW * sizeof(float);

__device__ __forceinline__ uint32_t cluster_addr(const void* local, int rank) {
    uint32_t out;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(out) : "r"(tc::smem_u32(local)), "r"(rank));
    return out;
}

// 16-byte store into another CTA's shared memory, counted on that CTA's mbarrier.
__device__ __forceinline__ void st_async16(uint32_t dst, float4 v, uint32_t mbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];\n" ::"r"(
                     dst),
                 "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "r"(mbar)
                 : "memory");
}

template <int RPT>
__global__ void __launch_bounds__(CP_THREADS, 1)
    panel_cluster_kernel(float* __restrict__ A, int lda, int m, int r0, int w, int* __restrict__ pos,
                         int* __restrict__ piv_out, int* __restrict__ info, int* __restrict__ err) {
    constexpr int CS = CP_CS;
    constexpr int RPC = RPT * CP_THREADS;  // positions per CTA
    extern __shared__ __align__(16) float dyn[];
    float* const tile = dyn;                              // [CP_SW][RPC]: my rows of the sub-panel
    int* const map = reinterpret_cast<int*>(dyn + CP_SW * RPC);  // map[p], p in [0, R): the row (at
                                                          // sub-panel start) now at position p
    __shared__ __align__(16) CpShared sh;
    cg::cluster_group cluster = cg::this_cluster();
    const int q = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int R = m - r0;
    const int row0 = q * RPC;
    float* const P0 = A + (size_t)r0 + (size_t)r0 * lda;  // panel origin

    for (int p = tid; p < R; p += CP_THREADS) map[p] = p;
    if (tid == 0) {
        tc::mbar_init(&sh.mbar[0], 1);
        tc::mbar_init(&sh.mbar[1], 1);
        tc::fence_barrier_init();
        tc::mbar_arrive_expect_tx(&sh.mbar[0], CP_RX_BYTES);
        tc::mbar_arrive_expect_tx(&sh.mbar[1], CP_RX_BYTES);
    }
    cluster.sync();  // every CTA's receive barriers are armed before the first record is sent
    bool rx_failed = false;  // warp 0: a receive wait gave up (error recorded; later waits skipped)

    float v[RPT][CP_SW];
    const int nsub = (w + CP_SW - 1) / CP_SW;
    for (int s = 0; s < nsub; ++s) {
        const int cs0 = s * CP_SW;
        const int sw = min(CP_SW, w - cs0);
        __syncthreads();
        // my rows of S -> registers, through the shared tile (coalesced columns;
        // all CP_SW * RPT loads of a thread in flight together)
        {
            float t[CP_SW * RPT];
#pragma unroll
            for (int u = 0; u < CP_SW * RPT; ++u) {
                const int e = tid + u * CP_THREADS, j = e / RPC, i = e - j * RPC, p = row0 + i;
                t[u] = (p < R && j < sw) ? __ldcg(P0 + (size_t)(cs0 + j) * lda + p) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < CP_SW * RPT; ++u) tile[tid + u * CP_THREADS] = t[u];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < RPT; ++k)
#pragma unroll
            for (int j = 0; j < CP_SW; ++j) v[k][j] = tile[j * RPC + k * CP_THREADS + tid];

        // steps 1-2 for sub-panel column cc: candidates, warp slots, the CTA's record
        auto publish = [&](const int cc) {
            const int cabs = cs0 + cc;
            const int buf = cabs & 1;
            unsigned bb = 0u;
            int bp = INT_MAX;
#pragma unroll
            for (int k = 0; k < RPT; ++k) {
                const int p = row0 + k * CP_THREADS + tid;
                const float a = fabsf(v[k][cc]);
                if (p < R && p >= cabs && a >= 0.f) {  // NaN is never a candidate
                    const unsigned ab = __float_as_uint(a);
                    if (ab > bb || bp == INT_MAX) {
                        bb = ab;
                        bp = p;
                    }
                }
            }
            const unsigned wm = __reduce_max_sync(0xffffffffu, bb);
            const int wp = (int)__reduce_min_sync(0xffffffffu, bb == wm ? (unsigned)bp : (unsigned)INT_MAX);
            if (lane == 0) {
                sh.wbits[warp] = wm;
                sh.wpos[warp] = wp;
            }
            if (wp != INT_MAX && bp == wp) {  // this lane owns the warp's candidate
                const int kw = (wp - row0) / CP_THREADS;
#pragma unroll
                for (int k = 0; k < RPT; ++k)
                    if (k == kw) {
#pragma unroll
                        for (int j = 0; j < CP_SW; ++j)
                            sh.wrow[warp][j] = v[k][j];
                    }
            }
#pragma unroll
            for (int k = 0; k < RPT; ++k)  // the row at the diagonal, for the swap
                if (row0 + k * CP_THREADS + tid == cabs) {
#pragma unroll
                    for (int j = 0; j < CP_SW; ++j)
                        sh.pubdiag[buf][j] = v[k][j];
                }
            __syncthreads();
// 2. the CTA's candidate record (warp 0), pushed into every CTA's receive slot
            //    (lane l -> CTA l), and by the diagonal's owner CTA the diagonal row
            if (warp == 0) {
                const unsigned mb = lane < CP_THREADS / 32 ? sh.wbits[lane] : 0u;
                const int mp = lane < CP_THREADS / 32 ? sh.wpos[lane] : INT_MAX;
                const unsigned cm = __reduce_max_sync(0xffffffffu, mb);
                const int cp = (int)__reduce_min_sync(0xffffffffu, mb == cm ? (unsigned)mp : (unsigned)INT_MAX);
                const unsigned own = __ballot_sync(0xffffffffu, mp == cp && mp != INT_MAX);
                const int ww = own ? __ffs(own) - 1 : 0;
                const float4* wr = reinterpret_cast<const float4*>(&sh.wrow[ww][0]);
                const float4 e0 = wr[0], e1 = wr[1], e2 = wr[2], e3 = wr[3];
                const float4 e4 = make_float4(__uint_as_float(cm), __int_as_float(cp), 0.f, 0.f);
                if (lane < CS) {
                    const uint32_t dst = cluster_addr(&sh.recv[buf][q], lane);
                    const uint32_t bar = cluster_addr(&sh.mbar[buf], lane);
                    st_async16(dst, e0, bar);
                    st_async16(dst + 16, e1, bar);
                    st_async16(dst + 32, e2, bar);
                    st_async16(dst + 48, e3, bar);
                    st_async16(dst + 64, e4, bar);
                } else if (q == cabs / RPC) {
                    const float4* dr = reinterpret_cast<const float4*>(&sh.pubdiag[buf][0]);
                    const uint32_t dst = cluster_addr(&sh.recv_diag[buf][0], lane - CS);
                    const uint32_t bar = cluster_addr(&sh.mbar[buf], lane - CS);
#pragma unroll
                    for (int u = 0; u < CP_SW / 4; ++u) st_async16(dst + 16 * u, dr[u], bar);
                }
            }
        };
        // step 3 for sub-panel column cc: wait, read the records, the winner
        auto receive = [&](const int cc) {
            const int cabs = cs0 + cc;
            const int c = cc;
            const int buf = cabs & 1;
            // 3. wait for the 16 records and the diagonal row, pick the same winner in every CTA
            if (warp == 0) {
                int ok = 1;
                if (lane == 0 && !rx_failed) {
                    ok = tc::mbar_wait(&sh.mbar[buf], (uint32_t)((cabs >> 1) & 1)) ? 1 : 0;
                    if (ok)
                        tc::mbar_arrive_expect_tx(&sh.mbar[buf], CP_RX_BYTES);  // re-arm for column cabs + 2
                    else
                        atomicExch(err, 8 /* MG_TIMEOUT */);
                }
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok) rx_failed = true;
                __syncwarp();
                float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0, q2 = q0, q3 = q0, q4 = q0;
                if (lane < CS) {
                    const float4* src = reinterpret_cast<const float4*>(&sh.recv[buf][lane]);
                    q0 = src[0];
                    q1 = src[1];
                    q2 = src[2];
                    q3 = src[3];
                    q4 = src[4];
                } else if (lane < CS + CP_SW / 4) {
                    q0 = reinterpret_cast<const float4*>(&sh.recv_diag[buf][0])[lane - CS];
                }
                const unsigned rb = lane < CS ? __float_as_uint(q4.x) : 0u;
                const int rp = lane < CS ? __float_as_int(q4.y) : INT_MAX;
                const unsigned gm = __reduce_max_sync(0xffffffffu, rb);
                const int gp = (int)__reduce_min_sync(0xffffffffu, rb == gm ? (unsigned)rp : (unsigned)INT_MAX);
                const unsigned gown = __ballot_sync(0xffffffffu, lane < CS && rp == gp);
                if (gown && lane == __ffs(gown) - 1) {
                    float4* d = reinterpret_cast<float4*>(sh.prow[buf]);
                    d[0] = q0;
                    d[1] = q1;
                    d[2] = q2;
                    d[3] = q3;
                }
                if (lane >= CS && lane < CS + CP_SW / 4) reinterpret_cast<float4*>(sh.drow[buf])[lane - CS] = q0;
                if (lane == 0) {
                    const float gv = __uint_as_float(gm);
                    const bool okp = gp >= 0 && gp < R && gv > 0.f;
                    sh.s_win[buf] = okp ? gp : cabs;
                    sh.s_pv[buf] = okp ? gv : 0.f;
                    sh.piv[cabs] = okp ? gp : cabs;
                    sh.touch[2 * c] = cabs;
                    sh.touch[2 * c + 1] = okp ? gp : cabs;
                    if (okp && gp != cabs) {
                        const int t = map[cabs];
                        map[cabs] = map[gp];
                        map[gp] = t;
                    }
                    if (!okp && q == 0) atomicCAS(info, 0, r0 + cabs + 1);
                }
            }
            __syncthreads();
        };

#pragma unroll
        for (int c = 0; c < CP_SW; ++c) {
            if (c < sw) {
                const int cabs = cs0 + c;
                const int buf = cabs & 1;
                publish(c);
                receive(c);
                // 4. interchange, scale, update (exactly zero column: nothing, as LAPACK)
                const float* ur = sh.prow[buf];
                if (sh.s_pv[buf] > 0.f) {
                    const int win = sh.s_win[buf];
                    if (win != cabs) {
#pragma unroll
                        for (int k = 0; k < RPT; ++k) {
                            const int p = row0 + k * CP_THREADS + tid;
                            if (p == cabs) {
#pragma unroll
                                for (int j = 0; j < CP_SW; ++j) v[k][j] = ur[j];
                            } else if (p == win) {
#pragma unroll
                                for (int j = 0; j < CP_SW; ++j) v[k][j] = sh.drow[buf][j];
                            }
                        }
                    }
                    const float inv = 1.f / ur[c];
                    float lk[RPT];  // multipliers of column c for my rows
                    bool ak[RPT];   // my rows below the pivot
#pragma unroll
                    for (int k = 0; k < RPT; ++k) {
                        const int p = row0 + k * CP_THREADS + tid;
                        ak[k] = p < R && p > cabs;
                        lk[k] = ak[k] ? v[k][c] * inv : 0.f;
                        if (ak[k]) v[k][c] = lk[k];
                    }
#pragma unroll
                    for (int j = c + 1; j < CP_SW; ++j) {
                        const float u = ur[j];
#pragma unroll
                        for (int k = 0; k < RPT; ++k)
                            if (ak[k]) v[k][j] = fmaf(lk[k], -u, v[k][j]);
                    }
                }
            }
        }

        // store my rows of the sub-panel (through the tile)
#pragma unroll
        for (int k = 0; k < RPT; ++k)
#pragma unroll
            for (int j = 0; j < CP_SW; ++j) tile[j * RPC + k * CP_THREADS + tid] = v[k][j];
        __syncthreads();
#pragma unroll 8
        for (int e = tid; e < CP_SW * RPC; e += CP_THREADS) {
            const int j = e / RPC, i = e - j * RPC, p = row0 + i;
            if (p < R && j < sw) P0[(size_t)(cs0 + j) * lda + p] = tile[e];
        }
        __syncthreads();  // map, touch list final for this sub-panel

        // 5. this sub-panel's interchanges on the panel's other columns
        //    (columns are dealt to the CTAs round-robin) and on pos (CTA 0)
        const int nt = 2 * sw;
        const int nother = w - sw;
        const int nmine = q < nother ? (nother - q + CS - 1) / CS : 0;
        for (int g0 = 0; g0 < nmine; g0 += CP_GCOLS) {
            const int gc = min(CP_GCOLS, nmine - g0);
            for (int e = tid; e < gc * nt; e += CP_THREADS) {
                const int jj = q + (g0 + e / nt) * CS;
                const int col = jj < cs0 ? jj : jj + sw;
                const int t = e % nt;
                sh.gbuf[e] = __ldcg(P0 + (size_t)map[sh.touch[t]] + (size_t)col * lda);
            }
            if (q == 0 && g0 == 0 && tid < nt) sh.gpos[tid] = __ldcg(pos + r0 + map[sh.touch[tid]]);
            __syncthreads();
            for (int e = tid; e < gc * nt; e += CP_THREADS) {
                const int jj = q + (g0 + e / nt) * CS;
                const int col = jj < cs0 ? jj : jj + sw;
                const int t = e % nt;
                P0[(size_t)sh.touch[t] + (size_t)col * lda] = sh.gbuf[e];
            }
            if (q == 0 && g0 == 0 && tid < nt) pos[r0 + sh.touch[tid]] = sh.gpos[tid];
            __syncthreads();
        }
        if (q == 0 && nmine == 0) {  // pos only (no other columns dealt to CTA 0)
            if (tid < nt) sh.gpos[tid] = __ldcg(pos + r0 + map[sh.touch[tid]]);
            __syncthreads();
            if (tid < nt) pos[r0 + sh.touch[tid]] = sh.gpos[tid];
        }
        __syncthreads();
        if (tid < nt) map[sh.touch[tid]] = sh.touch[tid];  // back to identity for the next sub-panel
        cluster.sync();  // swapped columns visible to the cluster

        const int nright = w - cs0 - CP_SW;
        if (nright > 0) {
            // 6. U(S, right) = L11^{-1} A(S, right), redundantly in every CTA
            for (int e = tid; e < CP_SW * CP_SW; e += CP_THREADS) {
                const int i = e % CP_SW, k = e / CP_SW;
                sh.l11[i][k] = __ldcg(P0 + (size_t)(cs0 + i) + (size_t)(cs0 + k) * lda);
            }
            for (int e = tid; e < CP_SW * nright; e += CP_THREADS) {
                const int i = e % CP_SW, jj = e / CP_SW;
                sh.ub[jj][i] = __ldcg(P0 + (size_t)(cs0 + i) + (size_t)(cs0 + CP_SW + jj) * lda);
            }
            __syncthreads();
            if (tid < nright) {
                float x[CP_SW];
#pragma unroll
                for (int i = 0; i < CP_SW; ++i) x[i] = sh.ub[tid][i];
#pragma unroll
                for (int k = 0; k < CP_SW; ++k)
#pragma unroll
                    for (int i = k + 1; i < CP_SW; ++i) x[i] = fmaf(sh.l11[i][k], -x[k], x[i]);
#pragma unroll
                for (int i = 0; i < CP_SW; ++i) sh.ub[tid][i] = x[i];
            }
            __syncthreads();
            cluster.sync();  // every CTA has read A(S, right) before CTA 0 overwrites it
            if (q == 0)
                for (int e = tid; e < CP_SW * nright; e += CP_THREADS) {
                    const int i = e % CP_SW, jj = e / CP_SW;
                    P0[(size_t)(cs0 + i) + (size_t)(cs0 + CP_SW + jj) * lda] = sh.ub[jj][i];
                }
            // 7. A(below, right) -= L(below, S) U(S, right) for my rows
            bool act[RPT];
#pragma unroll
            for (int k = 0; k < RPT; ++k) {
                const int p = row0 + k * CP_THREADS + tid;
                act[k] = p < R && p >= cs0 + CP_SW;
            }
            // columns in groups of 4, the next group's loads in flight during this group's FMAs
            constexpr int G = 4;
            const size_t ld = (size_t)lda;
            float* const C0 = P0 + (size_t)(cs0 + CP_SW) * ld;
            float cur[G][RPT], nxt[G][RPT];
#pragma unroll
            for (int g = 0; g < G; ++g)
#pragma unroll
                for (int k = 0; k < RPT; ++k)
                    cur[g][k] = (g < nright && act[k]) ? __ldcg(C0 + (size_t)g * ld + row0 + k * CP_THREADS + tid) : 0.f;
            for (int j0 = 0; j0 < nright; j0 += G) {
#pragma unroll
                for (int g = 0; g < G; ++g)
#pragma unroll
                    for (int k = 0; k < RPT; ++k) {
                        const int jj = j0 + G + g;
                        nxt[g][k] = (jj < nright && act[k]) ? __ldcg(C0 + (size_t)jj * ld + row0 + k * CP_THREADS + tid) : 0.f;
                    }
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    const int jj = j0 + g;
                    if (jj < nright) {
                        const float4* u4 = reinterpret_cast<const float4*>(&sh.ub[jj][0]);
#pragma unroll
                        for (int k4 = 0; k4 < CP_SW / 4; ++k4) {
                            const float4 u = u4[k4];
#pragma unroll
                            for (int k = 0; k < RPT; ++k) {
                                float a = cur[g][k];
                                a = fmaf(v[k][4 * k4 + 0], -u.x, a);
                                a = fmaf(v[k][4 * k4 + 1], -u.y, a);
                                a = fmaf(v[k][4 * k4 + 2], -u.z, a);
                                a = fmaf(v[k][4 * k4 + 3], -u.w, a);
                                cur[g][k] = a;
                            }
                        }
#pragma unroll
                        for (int k = 0; k < RPT; ++k)
                            if (act[k]) C0[(size_t)jj * ld + row0 + k * CP_THREADS + tid] = cur[g][k];
                    }
                }
#pragma unroll
                for (int g = 0; g < G; ++g)
#pragma unroll
                    for (int k = 0; k < RPT; ++k) cur[g][k] = nxt[g][k];
            }
        }
    }
    if (q == 0 && tid < w) piv_out[tid] = sh.piv[tid];
    cluster.sync();  // no CTA leaves while another may still read its shared memory
}

cudaLaunchConfig_t cluster_cfg(cudaStream_t st, size_t smem, cudaLaunchAttribute* at) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CP_CS);
    cfg.blockDim = dim3(CP_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = CP_CS;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cfg;
}

template <int RPT>
cudaError_t launch_cluster(cudaStream_t st, size_t smem, float* A, int lda, int m, int r0, int w, int* pos,
                           int* piv, int* info, int* err) {
    cudaLaunchAttribute at[1];
    cudaLaunchConfig_t cfg = cluster_cfg(st, smem, at);
    return cudaLaunchKernelEx(&cfg, panel_cluster_kernel<RPT>, A, lda, m, r0, w, pos, piv, info, err);
}

// Sets the kernel's attributes and returns how many such clusters fit.
template <int RPT>
int prepare(size_t smem_max) {
    auto k = panel_cluster_kernel<RPT>;
    int n = 0;
    cudaLaunchAttribute at[1];
    cudaLaunchConfig_t cfg = cluster_cfg(nullptr, smem_max, at);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max) != cudaSuccess ||
        cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace

namespace mg {

// Rows the cluster panel can take (0 if 16-CTA clusters of it do not fit
// the device; probed once per handle).
int panel_cluster_rows(mg_handle_t h) {
    constexpr int kRows = CP_CS * CP_MAX_RPT * CP_THREADS;
    if (h->panel_cluster == 0) {
        const size_t smem_max = (size_t)CP_SW * CP_MAX_RPT * CP_THREADS * sizeof(float) + (size_t)kRows * sizeof(int);
        const bool ok = prepare<1>(smem_max) > 0 && prepare<2>(smem_max) > 0 && prepare<3>(smem_max) > 0 &&
                        prepare<4>(smem_max) > 0;
        h->panel_cluster = ok ? CP_CS : -1;
    }
    return h->panel_cluster > 0 ? kRows : 0;
}

// FP32 panel of columns [r0, r0+w) over rows [r0, m) on one cluster; piv
// (device, w ints) receives the pivot rows relative to r0; pos is updated;
// info receives the first exactly-zero pivot column (1-based, atomicCAS on 0);
// err receives MG_TIMEOUT if a receive wait gave up.
// The caller checks panel_cluster_rows(h) >= m - r0 and w <= 128.
mg_status_t sgetf2_cluster(mg_handle_t h, float* A, int lda, int m, int r0, int w, int* pos, int* piv,
                           int* info, int* err) {
    const int R = m - r0;
    if (w <= 0 || w > CP_MAXW || R < w || R > panel_cluster_rows(h))
        return fail(h, MG_ERR_ARG, "sgetf2_cluster: unsupported panel %d x %d", R, w);
    const int rpt = (R + CP_CS * CP_THREADS - 1) / (CP_CS * CP_THREADS);
    const size_t smem = (size_t)CP_SW * rpt * CP_THREADS * sizeof(float) + (size_t)R * sizeof(int);
    ProfScope prof(h, "panel_f32", (double)R * w * w, 2.0 * R * w * sizeof(float));
    cudaError_t e;
    switch (rpt) {
        case 1: e = launch_cluster<1>(h->stream, smem, A, lda, m, r0, w, pos, piv, info, err); break;
        case 2: e = launch_cluster<2>(h->stream, smem, A, lda, m, r0, w, pos, piv, info, err); break;
        case 3: e = launch_cluster<3>(h->stream, smem, A, lda, m, r0, w, pos, piv, info, err); break;
        default: e = launch_cluster<4>(h->stream, smem, A, lda, m, r0, w, pos, piv, info, err); break;
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "panel_cluster_kernel launch");
    h->launches++;
    return MG_OK;
}

}  // namespace mg
