// FP32 panel factorization (getf2: partial pivoting, first index of the
// largest |a|, reciprocal scaling, fused rank-1 updates) on ONE thread-block
// cluster, for the mixed-precision LU.
//
// Why a cluster: a panel column needs one all-CTA agreement on the pivot.
// Through global memory (a grid barrier over ~128 CTAs) that costs several
// L2 round trips per column, ~4.5 us; inside a 16-CTA cluster each CTA pushes
// its candidate into every CTA's shared memory and waits on a local barrier.
// A 16-CTA cluster cannot hold a 16384 x 128 FP32 panel (8 MiB) on chip, so
// the panel is factored in sub-panels of 16 columns kept in registers (each
// of the 256 threads of a CTA owns RPT <= 4 rows x 16 columns, in a rotating
// window so that the column loop stays rolled):
//
//   for each sub-panel S = [cs0, cs0+16):
//     1. load my rows of S into registers
//     2. for each column c of S: local max |a| (warp redux), each warp's
//        winner row into shared memory -> warp 0 forms the CTA's 80-byte
//        record (row, |a| bits, position) and stores it with st.async into
//        slot [my rank] of every CTA (the diagonal row's owner also sends
//        that row), completing bytes on the receiver's mbarrier -> every warp
//        waits on the local mbarrier for 16 records + the diagonal row and
//        picks the same winner as every other warp and CTA -> swap in
//        registers -> scale by the reciprocal -> fused rank-1 update of my
//        rows' remaining columns
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
// column c+1, and every CTA sends that only after all of its warps have
// consumed their slots of column c (its one CTA barrier per column) and warp 0
// has re-armed their mbarrier (expect 1344 bytes).  The waits acquire at
// cluster scope, and the other lanes of a warp read the records only after a
// __syncwarp behind the waiting lane.  Waits are
// bounded: on a timeout the kernel records MG_TIMEOUT, skips later waits and
// runs on to the end, so every CTA executes the same cluster barriers.
// Global loads inside the kernel go to L2 (__ldcg): rows of the panel are
// rewritten by other CTAs of the cluster (the interchanges are dealt out by
// column), and an SM's L1 is not coherent with their stores.
#include <cooperative_groups.h>

#include <climits>
#include <type_traits>

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

constexpr int CP_NW = CP_THREADS / 32;  // warps per CTA
constexpr int CP_NREC = CP_CS;          // records a CTA receives per column: one per CTA

struct CpShared {
    float ub[CP_NOTHER][CP_UB_LD];  // U(S, right), [column][row of S]
    float l11[CP_SW][CP_SW + 1];
    CpRec recv[2][CP_NREC];          // the candidates for the column, by column parity
    __align__(16) float recv_diag[2][CP_SW];  // the row at the diagonal (sent by its owner)
    __align__(8) uint64_t mbar[2];            // receive barriers (transaction bytes), by parity
    uint2 wkey[2][CP_NW];                     // each warp's candidate (|a| bits, position), by parity
    int piv[CP_MAXW];
    int touch[2 * CP_SW];
    float gbuf[CP_GCOLS * 2 * CP_SW];
    int gpos[2 * CP_SW];
};

// Tournament pivoting (TOURN): per sub-panel, one exchange of candidate rows
// instead of one agreement per column.  Every CTA receives all 16 CTAs' 16
// candidates (their rows as the sub-panel started, and their positions) and
// the rows then at the sub-panel's 16 diagonal positions.
struct TsShared {
    CpRec cand[CP_CS][CP_SW];                 // [sender rank][column picked for]; pos < 0: no candidate
    __align__(16) float top[CP_SW][CP_SW];    // rows at positions cs0 .. cs0+15 as the sub-panel started
    CpRec mine[CP_SW];                        // this CTA's candidates
    float T[CP_SW][CP_SW + 1];                // the factored diagonal block
    int win[CP_SW];                           // the winners' positions (pivot order); -1: zero column
    int winslot[CP_SW];                       // their slot in the last level's candidate list
    int ok;
    __align__(8) uint64_t mbar;               // receive barrier (transaction bytes), one phase per sub-panel
};

__device__ __forceinline__ uint32_t ts_rx_bytes(int R, int cs0) {
    const int ntop = min(CP_SW, R - cs0);
    return (uint32_t)(CP_CS * CP_SW * sizeof(CpRec) + ntop * CP_SW * sizeof(float));
}

// One warp's elimination with partial pivoting over NPL rows per lane (u:
// working copies, updated in place; pos < 0: no row) across the sub-panel's
// sw <= 16 columns: per column the first largest |a| among the rows not yet
// picked (the smaller position on ties), then for the others l = a * (1/p),
// a_j := fma(l, -p_j, a_j).  pk[c] = lane * 8 + k of the row picked for
// column c (the same in every lane), or -1 if no nonzero was left.  The
// result depends only on the set of rows, not on how they sit in the warp.
template <int NPL>
__device__ __forceinline__ void warp_pick(float (&u)[NPL][CP_SW], const int (&pos)[NPL], int sw, int (&pk)[CP_SW]) {
    const int lane = threadIdx.x & 31;
    unsigned chosen = 0u;
#pragma unroll
    for (int c = 0; c < CP_SW; ++c) {
        pk[c] = -1;
        if (c < sw) {
            unsigned bb = 0u;
            int bp = INT_MAX, bk = 0;
#pragma unroll
            for (int k = 0; k < NPL; ++k) {
                if (pos[k] >= 0 && !((chosen >> k) & 1u)) {
                    const float a = fabsf(u[k][c]);
                    if (a >= 0.f) {  // NaN is never picked
                        const unsigned ab = __float_as_uint(a);
                        if (bp == INT_MAX || ab > bb || (ab == bb && pos[k] < bp)) {
                            bb = ab;
                            bp = pos[k];
                            bk = k;
                        }
                    }
                }
            }
            const unsigned wm = __reduce_max_sync(0xffffffffu, bp == INT_MAX ? 0u : bb);
            const unsigned wp =
                __reduce_min_sync(0xffffffffu, (bp != INT_MAX && bb == wm) ? (unsigned)bp : 0xffffffffu);
            if (wm != 0u && wp != 0xffffffffu) {  // the same in every lane
                const unsigned own = __ballot_sync(0xffffffffu, bp == (int)wp);
                const int ol = __ffs(own) - 1;
                const int okk = __shfl_sync(0xffffffffu, bk, ol);
                pk[c] = ol * 8 + okk;
                if (lane == ol) chosen |= 1u << bk;
                float pr[CP_SW];
#pragma unroll
                for (int j = c; j < CP_SW; ++j) {
                    float val = u[0][j];
#pragma unroll
                    for (int k = 1; k < NPL; ++k)
                        if (bk == k) val = u[k][j];
                    pr[j] = __shfl_sync(0xffffffffu, val, ol);
                }
                const float inv = 1.f / pr[c];
#pragma unroll
                for (int k = 0; k < NPL; ++k) {
                    if (pos[k] >= 0 && !((chosen >> k) & 1u)) {
                        const float l = u[k][c] * inv;
#pragma unroll
                        for (int j = c + 1; j < CP_SW; ++j) u[k][j] = fmaf(l, -pr[j], u[k][j]);
                    }
                }
            }
        }
    }
}

// A warp's tournament level over candidate records: lane l takes records
// in[l + 32 t], t < NPL (n records in all); the picks go to out[c] (the
// record as it came in; pos -1 where column c had no pick) and slot[c]
// receives the index of the picked record in `in`.
template <int NPL>
__device__ __forceinline__ void warp_level(const CpRec* in, int n, int sw, CpRec* out, int* slot) {
    const int lane = threadIdx.x & 31;
    float u[NPL][CP_SW];
    int pos[NPL];
#pragma unroll
    for (int t = 0; t < NPL; ++t) {
        const int q = lane + 32 * t;
        pos[t] = q < n ? in[q].pos : -1;
#pragma unroll
        for (int j = 0; j < CP_SW; ++j) u[t][j] = q < n ? in[q].row[j] : 0.f;
    }
    int pk[CP_SW];
    warp_pick<NPL>(u, pos, sw, pk);
#pragma unroll
    for (int c = 0; c < CP_SW; ++c) {
        const int q = pk[c] < 0 ? -1 : (pk[c] >> 3) + 32 * (pk[c] & 7);
        if (lane < CP_SW) out[c].row[lane] = q < 0 ? 0.f : in[q].row[lane];
        if (lane == 0) {
            out[c].pos = q < 0 ? -1 : in[q].pos;
            if (slot) slot[c] = q;
        }
    }
}

// Bytes each CTA receives per column: the candidate records and the diagonal row.
constexpr uint32_t CP_RX_BYTES = CP_NREC * sizeof(CpRec) + CP_SW * sizeof(float);

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

template <int RPT, bool TOURN>
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
    __shared__ __align__(16) TsShared ts;  // used by the tournament form only
    cg::cluster_group cluster = cg::this_cluster();
    const int q = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int R = m - r0;
    const int row0 = q * RPC;
    float* const P0 = A + (size_t)r0 + (size_t)r0 * lda;  // panel origin

    for (int p = tid; p < R; p += CP_THREADS) map[p] = p;
    if (tid == 0) {
        if constexpr (TOURN) {
            tc::mbar_init(&ts.mbar, 1);
            tc::fence_barrier_init();
            tc::mbar_arrive_expect_tx(&ts.mbar, ts_rx_bytes(R, 0));
        } else {
            tc::mbar_init(&sh.mbar[0], 1);
            tc::mbar_init(&sh.mbar[1], 1);
            tc::fence_barrier_init();
            tc::mbar_arrive_expect_tx(&sh.mbar[0], CP_RX_BYTES);
            tc::mbar_arrive_expect_tx(&sh.mbar[1], CP_RX_BYTES);
        }
    }
    cluster.sync();  // every CTA's receive barriers are armed before the first record is sent
    bool rx_failed = false;  // this warp: a receive wait gave up (error recorded; later waits skipped)

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

        if constexpr (!TOURN) {
            // Column loop over a rotating register window, so that every step runs
            // the same code at fixed register indices (a rolled loop: the fully
            // unrolled 16 columns are slower, instruction-fetch bound).  At step c
            // position 0 of v holds column c and positions 1 .. 15-c columns
            // c+1 .. 15; each step shifts the window left by one and puts column
            // c's multipliers (or the untouched column of a finished row) at its
            // last position.  The first 8 steps shift all 16 positions; the last
            // 8 columns are then at positions 0..7 and only those shift (half the
            // update work of a 16-wide window); the halves swap at the end.
            // Shift positions 0 .. W-1 of every row of mine left by one, n times:
            auto rotate_n = [&](auto WT, const int n) {
                constexpr int W = decltype(WT)::value;
#pragma unroll 1
                for (int r = 0; r < n; ++r)
#pragma unroll
                    for (int k = 0; k < RPT; ++k) {
                        const float v0 = v[k][0];
#pragma unroll
                        for (int j = 1; j < W; ++j) v[k][j - 1] = v[k][j];
                        v[k][W - 1] = v0;
                    }
            };
            // the warp of this CTA holding position pp (-1: not a row of this CTA)
            auto warp_of = [&](int pp) {
                const int i = pp - row0;
                return (i >= 0 && i < RPC) ? (i % CP_THREADS) >> 5 : -1;
            };
            // position pp (a row of this warp) broadcast to every lane of the warp
            auto bcast_row = [&](int pp, float(&r)[CP_SW]) {
                const int i = pp - row0, ol = i & 31, okk = i / CP_THREADS;
#pragma unroll
                for (int j = 0; j < CP_SW; ++j) {
                    float x = v[0][j];
#pragma unroll
                    for (int k = 1; k < RPT; ++k)
                        if (okk == k) x = v[k][j];
                    r[j] = __shfl_sync(0xffffffffu, x, ol);
                }
            };
            auto step = [&](auto WT, const int c) {
                constexpr int W = decltype(WT)::value;  // window width: positions 0 .. W-1 shift
                const int cabs = cs0 + c;
                const int buf = cabs & 1;
                // 1. this thread's and this warp's candidate (first largest |a|
                //    among the rows at or below the diagonal; NaN never wins)
                unsigned bb = 0u;
                int bp = INT_MAX;
#pragma unroll
                for (int k = 0; k < RPT; ++k) {
                    const int p = row0 + k * CP_THREADS + tid;
                    const float a = fabsf(v[k][0]);
                    if (p < R && p >= cabs && a >= 0.f) {
                        const unsigned ab = __float_as_uint(a);
                        if (ab > bb || bp == INT_MAX) {
                            bb = ab;
                            bp = p;
                        }
                    }
                }
                const unsigned wm = __reduce_max_sync(0xffffffffu, bb);
                const int wp = (int)__reduce_min_sync(0xffffffffu, bb == wm ? (unsigned)bp : (unsigned)INT_MAX);
                if (lane == 0) sh.wkey[buf][warp] = make_uint2(wm, (unsigned)wp);
                __syncthreads();
                // 2. every warp: the CTA's candidate from its warps' keys; the warp
                //    holding it broadcasts the row and pushes the record into slot
                //    [my rank] of every CTA (lane l -> CTA l); the warp holding the
                //    diagonal row pushes that row (lanes 16..31 -> CTA lane - 16)
                const uint2 kk = lane < CP_NW ? sh.wkey[buf][lane] : make_uint2(0u, (unsigned)INT_MAX);
                const unsigned cm = __reduce_max_sync(0xffffffffu, kk.x);
                const int cp = (int)__reduce_min_sync(0xffffffffu, kk.x == cm ? kk.y : (unsigned)INT_MAX);
                const int cw = cp == INT_MAX ? 0 : warp_of(cp);  // no candidate: warp 0 sends an empty record
                if (warp == cw) {
                    float r[CP_SW];
                    bcast_row(cp == INT_MAX ? row0 : cp, r);
                    if (lane < CS) {
                        const uint32_t dst = cluster_addr(&sh.recv[buf][q], lane);
                        const uint32_t bar = cluster_addr(&sh.mbar[buf], lane);
#pragma unroll
                        for (int u4 = 0; u4 < CP_SW / 4; ++u4)
                            st_async16(dst + 16u * u4, make_float4(r[4 * u4], r[4 * u4 + 1], r[4 * u4 + 2], r[4 * u4 + 3]),
                                       bar);
                        st_async16(dst + 64, make_float4(__uint_as_float(cm), __int_as_float(cp), 0.f, 0.f), bar);
                    }
                }
                if (warp == warp_of(cabs)) {
                    float r[CP_SW];
                    bcast_row(cabs, r);
                    if (lane >= CS) {
                        const uint32_t dst = cluster_addr(&sh.recv_diag[buf][0], lane - CS);
                        const uint32_t bar = cluster_addr(&sh.mbar[buf], lane - CS);
#pragma unroll
                        for (int u4 = 0; u4 < CP_SW / 4; ++u4)
                            st_async16(dst + 16u * u4, make_float4(r[4 * u4], r[4 * u4 + 1], r[4 * u4 + 2], r[4 * u4 + 3]),
                                       bar);
                    }
                }
                // 3. every warp: wait for the records and the diagonal row, pick the
                //    same winner (first largest |a|) as every other warp and CTA
                int ok = 1;
                if (lane == 0) {
                    ok = rx_failed ? 0 : (tc::mbar_wait_cluster(&sh.mbar[buf], (uint32_t)((cabs >> 1) & 1)) ? 1 : 0);
                    if (!ok && !rx_failed) atomicExch(err, 8 /* MG_TIMEOUT */);
                    if (ok && warp == 0) tc::mbar_arrive_expect_tx(&sh.mbar[buf], CP_RX_BYTES);  // column cabs + 2
                }
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok) rx_failed = true;
                __syncwarp();  // the other lanes' reads of the records after lane 0's acquire
                unsigned rb = 0u;
                int rp = INT_MAX, rs = 0;
#pragma unroll
                for (int t = 0; t < (CP_NREC + 31) / 32; ++t) {
                    const int idx = lane + 32 * t;
                    if (idx < CP_NREC) {
                        const uint2 kv = *reinterpret_cast<const uint2*>(&sh.recv[buf][idx].bits);
                        const int pp = (int)kv.y;
                        if (pp != INT_MAX && (rp == INT_MAX || kv.x > rb || (kv.x == rb && pp < rp))) {
                            rb = kv.x;
                            rp = pp;
                            rs = idx;
                        }
                    }
                }
                const unsigned gm = __reduce_max_sync(0xffffffffu, rb);
                const int gp = (int)__reduce_min_sync(0xffffffffu, rb == gm ? (unsigned)rp : (unsigned)INT_MAX);
                const unsigned gown = __ballot_sync(0xffffffffu, rp == gp && gp != INT_MAX);
                const int gslot = __shfl_sync(0xffffffffu, rs, gown ? __ffs(gown) - 1 : 0);
                const bool okp = gp >= 0 && gp < R && __uint_as_float(gm) > 0.f;
                if (warp == 0 && lane == 0) {
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
                // 4. interchange, scale, update, shift the window (an exactly zero
                //    column: shift only, as LAPACK leaves it)
                if (okp) {
                    float u[CP_SW];
                    {
                        const float4* u4p = reinterpret_cast<const float4*>(sh.recv[buf][gslot].row);
#pragma unroll
                        for (int u4 = 0; u4 < CP_SW / 4; ++u4) {
                            const float4 t4 = u4p[u4];
                            u[4 * u4] = t4.x;
                            u[4 * u4 + 1] = t4.y;
                            u[4 * u4 + 2] = t4.z;
                            u[4 * u4 + 3] = t4.w;
                        }
                    }
                    if (gp != cabs && (warp == warp_of(cabs) || warp == warp_of(gp))) {
#pragma unroll
                        for (int k = 0; k < RPT; ++k) {
                            const int p = row0 + k * CP_THREADS + tid;
                            if (p == cabs) {
#pragma unroll
                                for (int j = 0; j < CP_SW; ++j) v[k][j] = u[j];
                            } else if (p == gp) {
#pragma unroll
                                for (int j = 0; j < CP_SW; ++j) v[k][j] = sh.recv_diag[buf][j];
                            }
                        }
                    }
                    const float inv = 1.f / u[0];
                    const int na = CP_SW - 1 - c;  // columns right of the pivot: positions 1 .. na
#pragma unroll
                    for (int k = 0; k < RPT; ++k) {
                        const int p = row0 + k * CP_THREADS + tid;
                        const bool ak = p < R && p > cabs;
                        const float l = v[k][0] * inv;
                        const float v0 = v[k][0];
#pragma unroll
                        for (int j = 1; j < W; ++j) {
                            const float x = v[k][j];
                            v[k][j - 1] = (ak && j <= na) ? fmaf(l, -u[j], x) : x;
                        }
                        v[k][W - 1] = ak ? l : v0;
                    }
                } else {
                    rotate_n(WT, 1);
                }
            };
#pragma unroll 1
            for (int c = 0; c < min(sw, CP_SW / 2); ++c) step(std::integral_constant<int, CP_SW>{}, c);
            if (sw <= CP_SW / 2) {
                rotate_n(std::integral_constant<int, CP_SW>{}, CP_SW - sw);
            } else {
#pragma unroll 1
                for (int c = CP_SW / 2; c < sw; ++c) step(std::integral_constant<int, CP_SW / 2>{}, c);
                rotate_n(std::integral_constant<int, CP_SW / 2>{}, CP_SW - sw);
#pragma unroll
                for (int k = 0; k < RPT; ++k)
#pragma unroll
                    for (int j = 0; j < CP_SW / 2; ++j) {
                        const float t = v[k][j];
                        v[k][j] = v[k][j + CP_SW / 2];
                        v[k][j + CP_SW / 2] = t;
                    }
            }
            __syncthreads();  // piv, touch and map of this sub-panel complete
        } else {
            // ---- tournament pivoting for the sub-panel (CALU's TSLU: Grigori,
            // Demmel & Xiang, "CALU: a communication optimal LU factorization
            // algorithm", SIAM J. Matrix Anal. Appl. 2011), as a reduction
            // tree of partial-pivoting eliminations, each level passing on the
            // rows it picked as they were when the sub-panel started:
            //   L1 each warp over its own rows (RPT per lane),
            //   L2 warp 0 over the 8 warps' picks of its CTA,
            //   exchange: every CTA's 16 picks to every CTA of the cluster,
            //   L3 warp w over the picks of CTAs 2w and 2w+1, then
            //   L4 warp 0 over those 8 warps' picks: the 16 pivots, in order.
            // Every level is warp-level (shuffles and reductions, no CTA
            // barrier per column); levels L3 and L4 run identically in every CTA.
            CpRec* const wc = reinterpret_cast<CpRec*>(tile);  // the tile is free until the store
            {   // L1
                float u[RPT][CP_SW];
                int pos[RPT];
#pragma unroll
                for (int k = 0; k < RPT; ++k) {
                    const int p = row0 + k * CP_THREADS + tid;
                    pos[k] = (p < R && p >= cs0) ? p : -1;
#pragma unroll
                    for (int j = 0; j < CP_SW; ++j) u[k][j] = v[k][j];
                }
                int pk[CP_SW];
                warp_pick<RPT>(u, pos, sw, pk);
                CpRec* const mw = wc + warp * CP_SW;
#pragma unroll
                for (int c = 0; c < CP_SW; ++c) {
                    if (pk[c] < 0) {
                        if (lane == 0) mw[c].pos = -1;
                    } else if (lane == (pk[c] >> 3)) {
                        const int kw = pk[c] & 7;
#pragma unroll
                        for (int k = 0; k < RPT; ++k)
                            if (k == kw) {
#pragma unroll
                                for (int j = 0; j < CP_SW; ++j) mw[c].row[j] = v[k][j];
                                mw[c].pos = pos[k];
                            }
                    }
                }
            }
            __syncthreads();
            if (warp == 0) warp_level<4>(wc, 8 * CP_SW, sw, ts.mine, nullptr);  // L2
            __syncthreads();
            // exchange: candidates and the diagonal rows to every CTA of the cluster
            {
                const int dest = tid >> 4, c = tid & 15;
                const float4* src = reinterpret_cast<const float4*>(&ts.mine[c]);
                const uint32_t dst = cluster_addr(&ts.cand[q][c], dest);
                const uint32_t bar = cluster_addr(&ts.mbar, dest);
#pragma unroll
                for (int u4 = 0; u4 < 5; ++u4) st_async16(dst + 16u * u4, src[u4], bar);
            }
            const int ntop = min(CP_SW, R - cs0);
#pragma unroll
            for (int k = 0; k < RPT; ++k) {
                const int p = row0 + k * CP_THREADS + tid;
                if (p >= cs0 && p < cs0 + ntop) {
                    for (int dest = 0; dest < CS; ++dest) {
                        const uint32_t dst = cluster_addr(&ts.top[p - cs0][0], dest);
                        const uint32_t bar = cluster_addr(&ts.mbar, dest);
#pragma unroll
                        for (int u4 = 0; u4 < CP_SW / 4; ++u4)
                            st_async16(dst + 16u * u4,
                                       make_float4(v[k][4 * u4], v[k][4 * u4 + 1], v[k][4 * u4 + 2], v[k][4 * u4 + 3]),
                                       bar);
                    }
                }
            }
            if (tid == 0) {
                int ok = 0;
                if (!rx_failed) {
                    ok = tc::mbar_wait_cluster(&ts.mbar, (uint32_t)(s & 1)) ? 1 : 0;
                    if (!ok) atomicExch(err, 8 /* MG_TIMEOUT */);
                }
                if (ok && s + 1 < nsub) tc::mbar_arrive_expect_tx(&ts.mbar, ts_rx_bytes(R, cs0 + CP_SW));
                ts.ok = ok;
            }
            __syncthreads();
            if (!ts.ok) {
                rx_failed = true;
                for (int e = tid; e < CS * CP_SW; e += CP_THREADS) (&ts.cand[0][0])[e].pos = -1;
                __syncthreads();
            }
            warp_level<1>(&ts.cand[0][0] + warp * 32, 32, sw, wc + warp * CP_SW, nullptr);  // L3
            __syncthreads();
            if (warp == 0) {  // L4: the pivots
                float u[4][CP_SW];
                int pos[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int qq = lane + 32 * t;
                    pos[t] = wc[qq].pos;
#pragma unroll
                    for (int j = 0; j < CP_SW; ++j) u[t][j] = wc[qq].row[j];
                }
                int pk[CP_SW];
                warp_pick<4>(u, pos, sw, pk);
                if (lane < CP_SW) {
                    const int c = lane;
                    int qsel = -1;
#pragma unroll
                    for (int cc = 0; cc < CP_SW; ++cc)
                        if (cc == c) qsel = pk[cc] < 0 ? -1 : (pk[cc] >> 3) + 32 * (pk[cc] & 7);
                    ts.win[c] = (c < sw && qsel >= 0) ? wc[qsel].pos : -1;
                    ts.winslot[c] = qsel;
                }
            }
            __syncthreads();
            // T4. the interchanges: winner c moves to position cs0 + c (Mat's
            //     swap sequence, tracked in map), as partial pivoting records them
            if (tid == 0) {
                for (int c = 0; c < sw; ++c) {
                    const int cabs = cs0 + c;
                    int cur = cabs;
                    const int g = ts.win[c];
                    if (g >= 0) {
                        cur = g;
                        if (map[g] != g)
                            for (int t = 0; t < 2 * c; ++t)
                                if (map[sh.touch[t]] == g) {
                                    cur = sh.touch[t];
                                    break;
                                }
                    } else if (q == 0) {
                        atomicCAS(info, 0, r0 + cabs + 1);
                    }
                    sh.piv[cabs] = cur;
                    sh.touch[2 * c] = cabs;
                    sh.touch[2 * c + 1] = cur;
                    if (cur != cabs) {
                        const int t = map[cabs];
                        map[cabs] = map[cur];
                        map[cur] = t;
                    }
                }
            }
            __syncthreads();
            // the row (as the sub-panel started) now at each touched position
            auto row_of = [&](int r) -> const float* {
                for (int c = 0; c < sw; ++c)
                    if (ts.win[c] == r) return wc[ts.winslot[c]].row;
                // a displaced diagonal row (the interchanges move only those and
                // the winners; the clamp keeps a broken invariant in bounds)
                const int t = r - cs0;
                return ts.top[t >= 0 && t < CP_SW ? t : 0];
            };
            // T5. the diagonal block, factored without further pivoting (one warp,
            //     lane i holds row i), then every other row of mine eliminated with
            //     it: l = a * (1 / u_kk), a_j -= l u_kj, the fused operations of
            //     the partial-pivoting panel
            if (warp == 0) {
                float t[CP_SW];
                const bool rowok = lane < sw;
                const float* src = rowok ? row_of(map[cs0 + lane]) : nullptr;
#pragma unroll
                for (int j = 0; j < CP_SW; ++j) t[j] = rowok ? src[j] : 0.f;
#pragma unroll
                for (int k = 0; k < CP_SW; ++k) {
                    float rk[CP_SW];
#pragma unroll
                    for (int j = 0; j < CP_SW; ++j) rk[j] = __shfl_sync(0xffffffffu, t[j], k);
                    if (k < sw && lane > k && rowok && rk[k] != 0.f) {
                        const float l = t[k] * (1.f / rk[k]);
                        t[k] = l;
#pragma unroll
                        for (int j = 0; j < CP_SW; ++j)
                            if (j > k) t[j] = fmaf(l, -rk[j], t[j]);
                    }
                }
                if (rowok)
#pragma unroll
                    for (int j = 0; j < CP_SW; ++j) ts.T[lane][j] = t[j];
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < RPT; ++k) {
                const int p = row0 + k * CP_THREADS + tid;
                if (p >= R || p < cs0) continue;
                if (p < cs0 + sw) {
#pragma unroll
                    for (int j = 0; j < CP_SW; ++j) v[k][j] = ts.T[p - cs0][j];
                    continue;
                }
                if (map[p] != p) {  // a row moved here by the interchanges
                    const float* src = row_of(map[p]);
#pragma unroll
                    for (int j = 0; j < CP_SW; ++j) v[k][j] = src[j];
                }
#pragma unroll
                for (int c = 0; c < CP_SW; ++c) {
                    if (c < sw && ts.T[c][c] != 0.f) {
                        const float l = v[k][c] * (1.f / ts.T[c][c]);
                        v[k][c] = l;
#pragma unroll
                        for (int j = 0; j < CP_SW; ++j)
                            if (j > c) v[k][j] = fmaf(l, -ts.T[c][j], v[k][j]);
                    }
                }
            }
            __syncthreads();  // the tile (candidate records) is rewritten by the store below
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
            // columns in groups of G (G x RPT = 16 loads per thread), the next
            // group's loads in flight during this group's FMAs
            constexpr int G = 16 / RPT;
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

template <int RPT, bool TOURN>
cudaError_t launch_cluster(cudaStream_t st, size_t smem, float* A, int lda, int m, int r0, int w, int* pos,
                           int* piv, int* info, int* err) {
    cudaLaunchAttribute at[1];
    cudaLaunchConfig_t cfg = cluster_cfg(st, smem, at);
    return cudaLaunchKernelEx(&cfg, panel_cluster_kernel<RPT, TOURN>, A, lda, m, r0, w, pos, piv, info, err);
}

// Sets the kernel's attributes and returns how many such clusters fit.
template <int RPT, bool TOURN>
int prepare(size_t smem_max) {
    auto k = panel_cluster_kernel<RPT, TOURN>;
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
        const bool ok = prepare<1, false>(smem_max) > 0 && prepare<2, false>(smem_max) > 0 &&
                        prepare<3, false>(smem_max) > 0 && prepare<4, false>(smem_max) > 0 &&
                        prepare<1, true>(smem_max) > 0 && prepare<2, true>(smem_max) > 0 &&
                        prepare<3, true>(smem_max) > 0 && prepare<4, true>(smem_max) > 0;
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
                           int* info, int* err, bool tourn) {
    const int R = m - r0;
    if (w <= 0 || w > CP_MAXW || R < w || R > panel_cluster_rows(h))
        return fail(h, MG_ERR_ARG, "sgetf2_cluster: unsupported panel %d x %d", R, w);
    const int rpt = (R + CP_CS * CP_THREADS - 1) / (CP_CS * CP_THREADS);
    const size_t smem = (size_t)CP_SW * rpt * CP_THREADS * sizeof(float) + (size_t)R * sizeof(int);
    ProfScope prof(h, "panel_f32", (double)R * w * w, 2.0 * R * w * sizeof(float));
    cudaError_t e;
#define MG_LC(RPTV, TV) launch_cluster<RPTV, TV>(h->stream, smem, A, lda, m, r0, w, pos, piv, info, err)
    switch (rpt) {
        case 1: e = tourn ? MG_LC(1, true) : MG_LC(1, false); break;
        case 2: e = tourn ? MG_LC(2, true) : MG_LC(2, false); break;
        case 3: e = tourn ? MG_LC(3, true) : MG_LC(3, false); break;
        default: e = tourn ? MG_LC(4, true) : MG_LC(4, false); break;
    }
#undef MG_LC
    if (e != cudaSuccess) return cuda_fail(h, e, "panel_cluster_kernel launch");
    h->launches++;
    return MG_OK;
}

}  // namespace mg
