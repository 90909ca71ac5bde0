// Symmetric eigendecomposition EVD_Q(A, E, Q, eps, EVD_QR) of the Mat-8.1
// snapshot, results bit-identical to its AVX-512 build.
//
// Reference path (Mat-8.1): EVD_Q (EVD/EVD_Q.h:7-35) -> __EVD_Q_QR
// (EVD/__QR.h:145-169):
//  1. __EVD_Q_Householder (EVD/__QR.h:2-47): unblocked Householder
//     tridiagonalisation.  Step m takes the trailing order-N' matrix W (its
//     lower triangle), the reflector w = (x + sign(x0)||x|| e0) /
//     sqrt(cr (x0 + cr)) of its first column x, v = W22 w (per element a fused
//     chain over the columns, __mixed, plus the dot of the rest of its column,
//     __dot), h = v.w, and the rank-2 update
//     W22' = fma(w_k, fma(w_i, h, -v_i), fma(v_k, -w_i, W22_ki));
//  2. __Householder_Q2 (QR/__Householder.h:124-152): Q accumulated backwards
//     from the reflectors;
//  3. __EVD_Q_Givens (EVD/__QR.h:50-142): implicit single-shift QR sweeps on
//     the tridiagonal with absolute deflation threshold eps, every plane
//     rotation applied to two columns of Q (__ApplyGivensOnTheRight,
//     SIMD/__AVX512_double.h:1-20).
// Every dot product is Mat-8.1's __dot (SIMD/__AVX512_double.h:111-124): lane
// l of one 8-wide accumulator takes the elements l, l+8, ... in order (fused),
// then ((l0+l4)+(l2+l6)) + ((l1+l5)+(l3+l7)).
//
// GPU design:
//  - tridiagonalisation: one cooperative kernel for all steps, two bounded
//    grid barriers per step.  The trailing matrix stays in place in the
//    caller's buffer (W_m(k, i) at W[(m+i) ld + m+k]; the update of step m
//    writes W_{m+1}(k, i) over W_m(1+k, 1+i), the same address), and
//    reflector m replaces column m below the diagonal.  Phase 1: v's fused
//    chains (one thread per element, warps spread over the SMs) beside the
//    column dots (eight lanes per column); phase 2: h and the update (one warp
//    per column), where CTA 0's warp 0 updates column 0 and at once forms the
//    next reflector from it;
//  - Q: column j of Q only ever receives reflectors r = j-1, ..., 0 in that
//    order (s = -dot(w_r, Q(r+1:, j)), Q(r+1:, j) += w_r s), independent of
//    the other columns, so each column runs all its levels without any grid
//    synchronisation (eight lanes per column, four columns per warp);
//  - QR sweeps: the rotation sequence depends only on the tridiagonal, so the
//    host runs the scalar recurrence (the same operations, explicit fma) and
//    ships the rotations by sweeps, in chunks, while the GPU applies earlier
//    chunks; the application is independent per row of Q (one thread per row,
//    the carried column in a register, loads of the sweep's next columns
//    issued ahead).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "grid_sync.cuh"
#include "mg_internal.cuh"

namespace {

constexpr int TD_THREADS = 256;
constexpr int TD_WARPS = TD_THREADS / 32;
constexpr int TD_CH = 128;                           // fused-chain stage: columns per chunk
constexpr int TD_BUF = TD_CH * 32;                   // doubles per chain chunk (32 rows)
constexpr int TD_SMEM_DBL = 2 * TD_BUF + 2 * TD_CH;  // dynamic shared memory, doubles
constexpr int TD_STAGE = TD_BUF;                     // phase 2 keeps v and w on chip when nn <= this
constexpr int TD_COLREG = TD_STAGE / TD_THREADS;     // column-0 values per thread (phase 2, CTA 0)
constexpr int TD_PER = (TD_BUF + TD_THREADS - 32 - 1) / (TD_THREADS - 32);  // chunk loads per producer thread

// Mat-8.1 __dot reduction of the eight lane accumulators of an aligned group
// of eight lanes; the result is valid in the group's first lane.  All 32
// lanes must call it (they arrive from dot loops of different trip counts).
__device__ __forceinline__ double red8(double acc) {
    __syncwarp();
    const double s = __dadd_rn(acc, __shfl_down_sync(0xffffffffu, acc, 4, 8));
    const double s2 = __dadd_rn(s, __shfl_down_sync(0xffffffffu, s, 2, 8));
    return __dadd_rn(s2, __shfl_down_sync(0xffffffffu, s2, 1, 8));
}

// Lane l (0..7) of a group: the fused chain of Mat-8.1's __dot over the
// elements l, l+8, ... < len.  Loads bypass L1 (other CTAs of the same
// cooperative launch write the operands).
__device__ __forceinline__ double dot8_lane(const double* a, const double* b, int len, int l) {
    double acc = 0.0;
    int e = l;
    for (; e + 7 * 8 < len; e += 8 * 8) {
        double xa[8], xb[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            xa[u] = __ldcg(a + e + 8 * u);
            xb[u] = __ldcg(b + e + 8 * u);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) acc = fma(xa[u], xb[u], acc);
    }
    for (; e < len; e += 8) acc = fma(__ldcg(a + e), __ldcg(b + e), acc);
    return acc;
}

// Forms the reflector of the trailing matrix's first column in place (one
// warp): col[0] is the diagonal entry, col[1..nn] = x becomes w; d_out =
// col[0], e_out = -cr.  EVD/__QR.h:16-24.
__device__ void td_reflector(double* col, int nn, double* d_out, double* e_out) {
    const int lane = threadIdx.x & 31;
    // x0 is read before any lane overwrites col[1] below
    const double x0 = __ldcg(col + 1);
    double acc = 0.0;
    if (lane < 8) acc = dot8_lane(col + 1, col + 1, nn, lane);
    const double ss = __shfl_sync(0xffffffffu, red8(acc), 0);
    __syncwarp();  // every lane has read x0 and its dot operands
    double cr = sqrt(ss);
    if (x0 < 0.0) cr = -cr;
    const double w0 = __dadd_rn(x0, cr);
    const double hr = 1.0 / sqrt(__dmul_rn(cr, w0));
    for (int k = lane; k < nn; k += 32) {
        const double x = k == 0 ? w0 : __ldcg(col + 1 + k);
        col[1 + k] = __dmul_rn(x, hr);
    }
    if (lane == 0) {
        *d_out = __ldcg(col);
        *e_out = -cr;
    }
}

struct TdArgs {
    double* W;
    int ld, n;
    double* d;   // n
    double* e;   // n
    double* vc;  // n: fused-chain part of v
    double* vd;  // n: column-dot part of v
    unsigned* bar;
    int* err;
    int stage_cap;  // phase 2 keeps v, w and column 0 on chip while nn <= stage_cap (<= TD_STAGE)
};

// Stages chunk c0 .. c0+TD_CH-1 of the columns 0..ncol-1 of the trailing
// matrix's rows k0 .. k0+31 (buf[c 32 + r] = T[(c0+c) ld + k0+r], zero
// outside) and the matching reflector entries, with nthr threads (id tid).
__device__ __forceinline__ void td_chain_load(const double* T, int ld, const double* w, int nn, int k0, int ncol,
                                              int c0, double* buf, double* wb, int tid, int nthr) {
    double v[TD_PER + 2];
#pragma unroll
    for (int u = 0; u < TD_PER + 2; ++u) {
        const int idx = tid + u * nthr;
        const int c = idx >> 5, r = idx & 31;
        v[u] = (idx < TD_BUF && c0 + c < ncol && k0 + r < nn) ? __ldcg(T + (size_t)(c0 + c) * ld + k0 + r) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < TD_PER + 2; ++u) {
        const int idx = tid + u * nthr;
        if (idx < TD_BUF) buf[idx] = v[u];
    }
    if (tid < TD_CH) wb[tid] = c0 + tid < ncol ? __ldcg(w + c0 + tid) : 0.0;
}

// All steps m = 0 .. n-3 of __EVD_Q_Householder.  Cooperative launch (at
// least two CTAs); the barrier counter starts at zero.
//  phase 1: CTAs 0 .. nchc-1 run the fused chains of v, 32 elements per CTA:
//           seven warps stage the rows' columns chunk by chunk in shared
//           memory while warp 0 runs the 32 chains on the previous chunk; the
//           other CTAs' warps take the column dots, one warp per column (all
//           32 lanes load, lanes 0..7 run Mat's eight ordered chains on
//           shuffled operands);
//  phase 2: every CTA stages v and w in shared memory and computes h; CTA 0
//           updates column 0, keeps it on chip and forms the next reflector;
//           the warps of CTAs 1.. update columns 1.. (above stage_cap the same
//           steps read v, w and the column from global memory).
__global__ void __launch_bounds__(TD_THREADS) tridiag81_kernel(TdArgs a) {
    extern __shared__ __align__(16) double smem[];
    const int G = gridDim.x, cta = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int n = a.n, ld = a.ld;
    __shared__ double s_h, s_w0, s_hr;
    unsigned target = 0;
    if (cta == 0 && warp == 0) td_reflector(a.W, n - 1, a.d, a.e);
    if (!mg::grid_barrier(a.bar, target += G, a.err)) return;
    for (int m = 0; m + 2 < n; ++m) {
        const int nn = n - m - 1;
        const double* w = a.W + (size_t)m * ld + m + 1;   // reflector m
        double* T = a.W + (size_t)(m + 1) * ld + (m + 1);  // T[i ld + k] = W_m(1+k, 1+i)
        // ---- phase 1: v = W22 w
        const int nchain = (nn + 31) / 32;
        const int nchc = min(nchain, G / 2);
        if (cta < nchc) {
            // v_k = fma chain over i = 0..k of W22(k, i) w_i (EVD/__QR.h:27-29)
            double* buf = smem;
            double* wb = smem + 2 * TD_BUF;
            for (int cb = cta; cb < nchain; cb += nchc) {
                const int k0 = cb * 32, ncol = min(k0 + 32, nn);
                const int nchunk = (ncol + TD_CH - 1) / TD_CH;
                td_chain_load(T, ld, w, nn, k0, ncol, 0, buf, wb, tid, TD_THREADS);
                __syncthreads();
                double acc = 0.0;
                for (int t = 0; t < nchunk; ++t) {
                    if (warp == 0) {
                        const double* cur = buf + (t & 1) * TD_BUF;
                        const double* cw = wb + (t & 1) * TD_CH;
                        const int c0 = t * TD_CH;
                        const int clim = min(min(TD_CH, ncol - c0), k0 + lane - c0 + 1);  // columns i <= k
                        int c = 0;
                        for (; c + 8 <= clim; c += 8) {
                            double xt[8], xw[8];
#pragma unroll
                            for (int u = 0; u < 8; ++u) {
                                xt[u] = cur[(c + u) * 32 + lane];
                                xw[u] = cw[c + u];
                            }
#pragma unroll
                            for (int u = 0; u < 8; ++u) acc = fma(xt[u], xw[u], acc);
                        }
                        for (; c < clim; ++c) acc = fma(cur[c * 32 + lane], cw[c], acc);
                    } else if (t + 1 < nchunk) {
                        td_chain_load(T, ld, w, nn, k0, ncol, (t + 1) * TD_CH, buf + ((t + 1) & 1) * TD_BUF,
                                      wb + ((t + 1) & 1) * TD_CH, tid - 32, TD_THREADS - 32);
                    }
                    __syncthreads();
                }
                if (warp == 0 && k0 + lane < nn) a.vc[k0 + lane] = acc;
            }
        } else {
            // v_i += dot(W22(i+1:, i), w(i+1:)) (EVD/__QR.h:30-32), one warp per column
            const int ndw = (G - nchc) * TD_WARPS;
            for (int i = warp * (G - nchc) + (cta - nchc); i < nn; i += ndw) {
                const int len = nn - i - 1;
                const double* pa = T + (size_t)i * ld + i + 1;
                const double* pb = w + i + 1;
                double acc = 0.0;
                for (int base = 0; base < len; base += 256) {
                    double xa[8], xb[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int e = base + 32 * u + lane;
                        xa[u] = e < len ? __ldcg(pa + e) : 0.0;
                        xb[u] = e < len ? __ldcg(pb + e) : 0.0;
                    }
                    // lane l (< 8) takes the elements base + 8j + l, j = 0..31, in order
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const int src = ((j & 3) << 3) | (lane & 7);
                        const double x = __shfl_sync(0xffffffffu, xa[j >> 2], src);
                        const double y = __shfl_sync(0xffffffffu, xb[j >> 2], src);
                        if (lane < 8 && base + 8 * j + lane < len) acc = fma(x, y, acc);
                    }
                }
                const double r = red8(acc);
                if (lane == 0) a.vd[i] = r;
            }
        }
        if (!mg::grid_barrier(a.bar, target += G, a.err)) return;
        // ---- phase 2: h = v.w, then the rank-2 update (EVD/__QR.h:34-39)
        const bool staged = nn <= a.stage_cap;
        double* sv = smem;
        double* sw = smem + TD_STAGE;
        if (staged) {
            for (int k = tid; k < nn; k += TD_THREADS) {
                sv[k] = __dadd_rn(__ldcg(a.vc + k), __ldcg(a.vd + k));
                sw[k] = __ldcg(w + k);
            }
            __syncthreads();
        }
        if (warp == 0) {
            double acc = 0.0;
            if (lane < 8) {
                if (staged) {
                    int e = lane;
                    for (; e + 7 * 8 < nn; e += 8 * 8) {
                        double xv[8], xw[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            xv[u] = sv[e + 8 * u];
                            xw[u] = sw[e + 8 * u];
                        }
#pragma unroll
                        for (int u = 0; u < 8; ++u) acc = fma(xv[u], xw[u], acc);
                    }
                    for (; e < nn; e += 8) acc = fma(sv[e], sw[e], acc);
                } else {
                    int e = lane;
                    for (; e + 7 * 8 < nn; e += 8 * 8) {
                        double xv[8], xw[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int q = e + 8 * u;
                            xv[u] = __dadd_rn(__ldcg(a.vc + q), __ldcg(a.vd + q));
                            xw[u] = __ldcg(w + q);
                        }
#pragma unroll
                        for (int u = 0; u < 8; ++u) acc = fma(xv[u], xw[u], acc);
                    }
                    for (; e < nn; e += 8)
                        acc = fma(__dadd_rn(__ldcg(a.vc + e), __ldcg(a.vd + e)), __ldcg(w + e), acc);
                }
            }
            const double hh = red8(acc);
            if (lane == 0) s_h = hh;
        }
        __syncthreads();
        const double h = s_h;
        if (cta == 0) {
            if (staged) {
                // column 0 of W_{m+1}, kept in registers, then on chip for the reflector
                const double w0v = sw[0], q = fma(w0v, h, -sv[0]);
                double cv[TD_COLREG];
#pragma unroll
                for (int t = 0; t < TD_COLREG; ++t) {
                    const int k = tid + t * TD_THREADS;
                    cv[t] = 0.0;
                    if (k < nn) {
                        cv[t] = fma(sw[k], q, fma(sv[k], -w0v, __ldcg(T + k)));
                        T[k] = cv[t];
                    }
                }
                if (m + 3 < n) {
                    __syncthreads();  // v and w are no longer read
                    double* scol = smem;
#pragma unroll
                    for (int t = 0; t < TD_COLREG; ++t) {
                        const int k = tid + t * TD_THREADS;
                        if (k < nn) scol[k] = cv[t];
                    }
                    __syncthreads();
                    // the next reflector from the updated first column (EVD/__QR.h:16-24)
                    const int len = nn - 1;
                    if (warp == 0) {
                        double acc = 0.0;
                        if (lane < 8) {
                            int e = lane;
                            for (; e + 7 * 8 < len; e += 8 * 8) {
                                double xa[8];
#pragma unroll
                                for (int u = 0; u < 8; ++u) xa[u] = scol[1 + e + 8 * u];
#pragma unroll
                                for (int u = 0; u < 8; ++u) acc = fma(xa[u], xa[u], acc);
                            }
                            for (; e < len; e += 8) acc = fma(scol[1 + e], scol[1 + e], acc);
                        }
                        const double ss = red8(acc);
                        if (lane == 0) {
                            const double x0 = scol[1];
                            double cr = sqrt(ss);
                            if (x0 < 0.0) cr = -cr;
                            const double w0 = __dadd_rn(x0, cr);
                            s_w0 = w0;
                            s_hr = 1.0 / sqrt(__dmul_rn(cr, w0));
                            a.d[m + 1] = scol[0];
                            a.e[m + 1] = -cr;
                        }
                    }
                    __syncthreads();
                    const double w0 = s_w0, hr = s_hr;
                    for (int k = tid; k < len; k += TD_THREADS) T[1 + k] = __dmul_rn(k == 0 ? w0 : scol[1 + k], hr);
                }
            } else if (warp == 0) {
                const double wi = __ldcg(w), q = fma(wi, h, -__dadd_rn(__ldcg(a.vc), __ldcg(a.vd)));
                for (int k = lane; k < nn; k += 32) {
                    const double vk = __dadd_rn(__ldcg(a.vc + k), __ldcg(a.vd + k));
                    T[k] = fma(__ldcg(w + k), q, fma(vk, -wi, __ldcg(T + k)));
                }
                if (m + 3 < n) {
                    __threadfence();
                    __syncwarp();
                    td_reflector(T, nn - 1, a.d + m + 1, a.e + m + 1);
                }
            }
        } else {
            // columns 1 .. nn-1 over the warps of CTAs 1 .. G-1
            const int nw2 = (G - 1) * TD_WARPS;
            for (int i = 1 + warp * (G - 1) + (cta - 1); i < nn; i += nw2) {
                double* col = T + (size_t)i * ld;
                if (staged) {
                    const double wi = sw[i], q = fma(wi, h, -sv[i]);
                    int k = i + lane;
                    for (; k + 7 * 32 < nn; k += 8 * 32) {
                        double x[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) x[u] = __ldcg(col + k + 32 * u);
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int kk = k + 32 * u;
                            col[kk] = fma(sw[kk], q, fma(sv[kk], -wi, x[u]));
                        }
                    }
                    for (; k < nn; k += 32) col[k] = fma(sw[k], q, fma(sv[k], -wi, __ldcg(col + k)));
                } else {
                    const double wi = __ldcg(w + i);
                    const double q = fma(wi, h, -__dadd_rn(__ldcg(a.vc + i), __ldcg(a.vd + i)));
                    for (int k = i + lane; k < nn; k += 32) {
                        const double vk = __dadd_rn(__ldcg(a.vc + k), __ldcg(a.vd + k));
                        col[k] = fma(__ldcg(w + k), q, fma(vk, -wi, __ldcg(col + k)));
                    }
                }
            }
        }
        if (!mg::grid_barrier(a.bar, target += G, a.err)) return;
    }
}

// The last 2 x 2 block (EVD/__QR.h:42-44), or the 1 x 1 matrix.
__global__ void td_tail_kernel(const double* __restrict__ W, int ld, int n, double* d, double* e) {
    if (threadIdx.x != 0) return;
    if (n == 1) {
        d[0] = W[0];
        return;
    }
    const double* B = W + (size_t)(n - 2) * ld + (n - 2);
    d[n - 2] = B[0];
    d[n - 1] = B[ld + 1];
    e[n - 2] = B[1];
}

// Q (n x n, ld ldq) from the reflectors held below the diagonal of U (ld ldu):
// Q starts as the identity; column j receives reflectors r = min(j-1, n-3)
// .. 0 (QR/__Householder.h:131-145).  Eight lanes per column, four columns
// per warp.
__global__ void formq81_kernel(const double* __restrict__ U, int ldu, int n, double* __restrict__ Q, int ldq) {
    const int lane = threadIdx.x & 31, grp = lane >> 3, l = lane & 7;
    const int wid = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int j0 = wid * 4;
    if (j0 >= n) return;
    const int j = j0 + grp;
    double* q = Q + (size_t)j * ldq;
    const int rtop = min(j0 + 3 - 1, n - 3);
    for (int r = rtop; r >= 0; --r) {
        const bool act = j < n && j >= r + 1;
        const int len = n - r - 1;
        const double* u = U + (size_t)r * ldu + r + 1;
        double* qc = q + r + 1;
        double acc = 0.0;
        if (act) {
            int e = l;
            for (; e + 7 * 8 < len; e += 8 * 8) {
                double xa[8], xb[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    xa[t] = __ldg(u + e + 8 * t);
                    xb[t] = qc[e + 8 * t];
                }
#pragma unroll
                for (int t = 0; t < 8; ++t) acc = fma(xa[t], xb[t], acc);
            }
            for (; e < len; e += 8) acc = fma(__ldg(u + e), qc[e], acc);
        }
        const double s = -__shfl_sync(0xffffffffu, red8(acc), grp * 8);
        if (act)
            for (int e = l; e < len; e += 8) qc[e] = fma(__ldg(u + e), s, qc[e]);
        __syncwarp();
    }
}

// The same Q formation with a CTA's FQ_COLS columns of Q and the reflector
// (double-buffered) in shared memory, for n <= FQ_NMAX: warp 0 runs the
// columns' dot chains (eight lanes per column) while warps 1.. stage the next
// reflector; then all threads apply the axpy on chip.  Columns start as e_j;
// the kernel writes every column of Q.
constexpr int FQ_COLS = 4;
constexpr int FQ_THREADS = 128;
constexpr int FQ_NMAX = 4096;

__global__ void __launch_bounds__(FQ_THREADS) formq81_smem_kernel(const double* __restrict__ U, int ldu, int n,
                                                                  double* __restrict__ Q, int ldq) {
    extern __shared__ __align__(16) double fsm[];
    double* qs = fsm;                  // FQ_COLS x n
    double* us = fsm + FQ_COLS * n;    // 2 x n
    __shared__ double s_s[FQ_COLS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int j0 = blockIdx.x * FQ_COLS;
    for (int c = 0; c < FQ_COLS; ++c)
        for (int r = tid; r < n; r += FQ_THREADS) qs[c * n + r] = j0 + c == r ? 1.0 : 0.0;
    const int rtop = min(j0 + FQ_COLS - 2, n - 3);
    if (rtop >= 0)
        for (int e = tid; e < n - rtop - 1; e += FQ_THREADS) us[e] = __ldg(U + (size_t)rtop * ldu + rtop + 1 + e);
    __syncthreads();
    for (int r = rtop, b = 0; r >= 0; --r, b ^= 1) {
        const int len = n - r - 1;
        const double* u = us + b * n;
        if (warp == 0) {
            const int grp = lane >> 3, l = lane & 7, j = j0 + grp;
            const bool act = j < n && j >= r + 1;
            const double* qc = qs + grp * n + r + 1;
            double acc = 0.0;
            if (act) {
                int e = l;
                for (; e + 7 * 8 < len; e += 8 * 8) {
                    double xa[8], xb[8];
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        xa[t] = u[e + 8 * t];
                        xb[t] = qc[e + 8 * t];
                    }
#pragma unroll
                    for (int t = 0; t < 8; ++t) acc = fma(xa[t], xb[t], acc);
                }
                for (; e < len; e += 8) acc = fma(u[e], qc[e], acc);
            }
            const double sred = red8(acc);
            if (l == 0) s_s[grp] = act ? -sred : 0.0;
        } else if (r > 0) {
            const int rn = r - 1;
            double* un = us + (b ^ 1) * n;
            for (int e = tid - 32; e < n - rn - 1; e += FQ_THREADS - 32)
                un[e] = __ldg(U + (size_t)rn * ldu + rn + 1 + e);
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < FQ_COLS; ++c) {
            const int j = j0 + c;
            if (j < n && j >= r + 1) {
                const double sc = s_s[c];
                double* qc = qs + c * n + r + 1;
                for (int e = tid; e < len; e += FQ_THREADS) qc[e] = fma(u[e], sc, qc[e]);
            }
        }
        __syncthreads();
    }
    for (int c = 0; c < FQ_COLS; ++c)
        if (j0 + c < n)
            for (int r = tid; r < n; r += FQ_THREADS) Q[(size_t)(j0 + c) * ldq + r] = qs[c * n + r];
}

__global__ void evd_identity_kernel(double* __restrict__ Q, int ldq, int n) {
    const size_t total = (size_t)n * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % n), c = (int)(e / n);
        Q[r + (size_t)c * ldq] = r == c ? 1.0 : 0.0;
    }
}

__global__ void evd_copy_lower_kernel(const double* __restrict__ A, int lda, int n, double* __restrict__ B, int ldb) {
    const size_t total = (size_t)n * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % n), c = (int)(e / n);
        if (r >= c) B[r + (size_t)c * ldb] = A[r + (size_t)c * lda];
    }
}

// E = diag(w) (EVD/__QR.h:161-168).
__global__ void evd_diag_kernel(double* __restrict__ E, int lde, int n, const double* __restrict__ w) {
    const size_t total = (size_t)n * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % n), c = (int)(e / n);
        E[r + (size_t)c * lde] = r == c ? w[r] : 0.0;
    }
}

struct Sweep {
    int start, len, off, pad;
};

// The rotations of a chunk of sweeps applied to Q's columns: sweep (start,
// len) rotates the column pairs (start, start+1), ..., (start+len-1,
// start+len) in order, each by (c, s): x' = fma(x, c, y s),
// y' = fma(-x, s, y c) (SIMD/__AVX512_double.h:1-20).  Every row is
// independent; a warp holds 32 rows (one per lane) and carries the current
// column in a register.  One warp instruction of FP64 work keeps the SM
// sub-partition's FP64 pipe busy for many cycles whatever the active lanes,
// so a lone warp per row strip is bound by the rotation count: ROT_WARPS
// warps share each 32-row strip instead, warp w applying the sweeps
// s = w, w + ROT_WARPS, ... .  A sweep may touch a column only after every
// earlier sweep still in flight has finished with it: each warp publishes in
// shared memory (sweep << 32 | P), "columns < P are final for this sweep",
// after every batch of ROT_PF rotations, and waits (bounded) on the others'
// words before the batch.  Rows are read and written through L1 (the warps
// of one CTA share an SM).
constexpr int ROT_WARPS = 8;
constexpr int ROT_PF = 16;  // rotations per batch (the loads of a batch are in flight together)

__device__ __forceinline__ bool rot_wait(volatile unsigned long long* prog, int s, int need, int* err) {
    bool ok = true;
    if ((threadIdx.x & 31) == 0) {
        for (int q = s - 1; q >= 0 && q > s - ROT_WARPS; --q) {
            const unsigned long long want = ((unsigned long long)q << 32) | (unsigned)need;
            unsigned spins = 0;
            while (prog[q % ROT_WARPS] < want) {
                if (++spins > mg::kSpinLimit) {
                    atomicExch(err, 8 /* MG_TIMEOUT */);
                    ok = false;
                    break;
                }
                if (spins > 64) __nanosleep(32);
            }
            if (!ok) break;
        }
        __threadfence_block();
    }
    const bool all_ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    __syncwarp();  // the other lanes' loads come after lane 0 saw the flags
    return all_ok;
}

__global__ void __launch_bounds__(32 * ROT_WARPS) rot81_kernel(double* __restrict__ Q, int ldq, int n,
                                                               const Sweep* __restrict__ sw, int nsw,
                                                               const double2* __restrict__ cs, int* err) {
    __shared__ unsigned long long prog[ROT_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r = blockIdx.x * 32 + lane;
    const bool live = r < n;
    double* row = Q + (live ? r : 0);
    if (lane == 0) prog[warp] = (unsigned long long)warp << 32;  // sweep `warp`, nothing final yet
    __syncthreads();
    volatile unsigned long long* vprog = prog;
    for (int si = warp; si < nsw; si += ROT_WARPS) {
        const Sweep S = sw[si];
        const double2* p = cs + S.off;
        double x = 0.0;
        for (int k = 0; k < S.len; k += ROT_PF) {
            const int nb = min(ROT_PF, S.len - k);
            // this batch reads columns up to start + k + nb
            if (!rot_wait(vprog, si, S.start + k + nb + 1, err)) return;
            if (k == 0 && live) x = row[(size_t)S.start * ldq];
            double y[ROT_PF];
            double2 c[ROT_PF];
#pragma unroll
            for (int u = 0; u < ROT_PF; ++u) {
                y[u] = (u < nb && live) ? row[(size_t)(S.start + k + 1 + u) * ldq] : 0.0;
                c[u] = u < nb ? __ldg(p + k + u) : make_double2(0.0, 0.0);
            }
#pragma unroll
            for (int u = 0; u < ROT_PF; ++u) {
                if (u < nb) {
                    const double xn = fma(x, c[u].x, __dmul_rn(y[u], c[u].y));
                    if (live) row[(size_t)(S.start + k + u) * ldq] = xn;
                    x = fma(-x, c[u].y, __dmul_rn(y[u], c[u].x));
                }
            }
            if (k + nb == S.len && live) row[(size_t)(S.start + S.len) * ldq] = x;
            __threadfence_block();
            __syncwarp();
            if (lane == 0)
                vprog[warp] = k + nb == S.len
                                  ? (unsigned long long)(si + ROT_WARPS) << 32  // sweep done: the next one, nothing final
                                  : ((unsigned long long)si << 32) | (unsigned)(S.start + k + nb);
        }
        if (S.len == 0) {
            __syncwarp();
            if (lane == 0) vprog[warp] = (unsigned long long)(si + ROT_WARPS) << 32;
        }
    }
    if (lane == 0) vprog[warp] = ~0ull;
}

int evd_grid(mg_handle_t h, size_t total) {
    size_t g = (total + 255) / 256;
    const size_t cap = (size_t)h->num_sms * 8;
    return (int)(g < 1 ? 1 : g > cap ? cap : g);
}

// ------------------------------------------------------------------ host QR sweeps
// __EVD_Q_Givens (EVD/__QR.h:50-142) on the host.  Each plane rotation's
// (c, s) goes to the sink in order, sweep by sweep.  The reference build
// fuses t*t + 1, the first product of c2*temp + s2*temp_2 and of
// s2*temp + c2*temp_2, the added/subtracted 2*cs*b_i, the first and last
// products of -cs*temp + cs*temp_2 + (c2 - s2)*b_i, c*b_{i-1} + s*B, and in
// the shift c2^2 - 4 (a_{n-1} a_n - b_{n-1}^2) both leading products; the
// same operations are written out here with std::fma.
struct RotSink {
    virtual bool sweep(int start, int len) = 0;  // a sweep of len rotations begins at column start
    virtual void rot(double c, double s) = 0;
    virtual ~RotSink() = default;
};

inline void rot_step(double* a, double* b, int i, double t, bool first, double& c, double& s) {
    double c2, s2, cs;
    if (first) {
        s2 = 1.0 / std::fma(t, t, 1.0);
        c2 = 1.0 - s2;
        cs = t * s2;
    } else {
        c2 = 1.0 / std::fma(t, t, 1.0);
        s2 = 1.0 - c2;
        cs = t * c2;
    }
    const double temp = a[i], temp_2 = a[i + 1];
    const double cs2 = 2.0 * cs;
    a[i] = std::fma(cs2, b[i], std::fma(c2, temp, s2 * temp_2));
    a[i + 1] = std::fma(-cs2, b[i], std::fma(s2, temp, c2 * temp_2));
    b[i] = std::fma(c2 - s2, b[i], std::fma(-cs, temp, cs * temp_2));
    if (first) {
        s = std::sqrt(s2);
        c = t * s;
    } else {
        c = std::sqrt(c2);
        s = t * c;
    }
}

// Returns false when the sweep budget runs out (the reference loops on) or
// the sink fails.
bool qr_sweeps(double* a, double* b, int m, int n, double eps, long long& budget, RotSink& sink) {
    while (n > m) {
        if (std::fabs(b[m]) < eps) {
            ++m;
            continue;
        }
        if (std::fabs(b[n - 1]) < eps) {
            --n;
            continue;
        }
        for (int i = m + 1; i < n - 1; ++i) {
            if (std::fabs(b[i]) < eps) {
                if (!qr_sweeps(a, b, m, i, eps, budget, sink)) return false;
                m = i + 1;
            }
        }
        if (--budget < 0) return false;
        const double c2 = a[n - 1] + a[n];
        const double s2 = std::sqrt(std::fma(c2, c2, -(std::fma(a[n - 1], a[n], -(b[n - 1] * b[n - 1])) * 4.0)));
        const double t = (c2 - 2.0 * a[n] > 0) ? (c2 - s2) * 0.5 : (c2 + s2) * 0.5;
        if (!sink.sweep(m, n - m)) return false;
        double c, s;
        if (std::fabs(b[m]) > std::fabs(a[m] - t))
            rot_step(a, b, m, (a[m] - t) / b[m], true, c, s);
        else
            rot_step(a, b, m, b[m] / (a[m] - t), false, c, s);
        double B = s * b[m + 1];
        b[m + 1] = c * b[m + 1];
        sink.rot(c, s);
        for (int i = m + 1; i < n; ++i) {
            if (std::fabs(B) > std::fabs(b[i - 1]))
                rot_step(a, b, i, b[i - 1] / B, true, c, s);
            else
                rot_step(a, b, i, B / b[i - 1], false, c, s);
            b[i - 1] = std::fma(c, b[i - 1], s * B);
            B = s * b[i + 1];
            b[i + 1] = c * b[i + 1];
            sink.rot(c, s);
        }
    }
    return true;
}

// Counts the rotations (the eigenvalue-only host entry point).
struct CountSink final : RotSink {
    long long count = 0;
    bool sweep(int, int) override { return true; }
    void rot(double, double) override { ++count; }
};

// Streams the rotations to the GPU in chunks: two pinned staging areas and
// two device areas used in turn; a chunk is launched when the next sweep does
// not fit, while the host goes on with the recurrence.
struct GpuRotSink final : RotSink {
    mg_handle_t h;
    double* Q;
    int ldq, n;
    int* err = nullptr;    // device error word (MG_TIMEOUT if a bounded wait gave up)
    size_t cap_rot, cap_sw;
    double2* hcs[2];
    Sweep* hsw[2];
    double2* dcs[2];
    Sweep* dsw[2];
    cudaEvent_t done[2] = {nullptr, nullptr};
    bool used[2] = {false, false};
    int cur = 0;
    size_t nrot = 0, nsw = 0;
    long long total_rot = 0;
    double wait_ms = 0;  // host time spent waiting for the GPU to free a staging area
    mg_status_t st = MG_OK;

    bool flush() {
        if (nsw == 0) return true;
        cudaStream_t s = h->stream;
        cudaError_t e = cudaMemcpyAsync(dsw[cur], hsw[cur], nsw * sizeof(Sweep), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dcs[cur], hcs[cur], nrot * sizeof(double2), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            st = mg::cuda_fail(h, e, "EVD_Q rotation upload");
            return false;
        }
        rot81_kernel<<<(n + 31) / 32, 32 * ROT_WARPS, 0, s>>>(Q, ldq, n, dsw[cur], (int)nsw, dcs[cur], err);
        if ((st = mg::post_launch(h, "rot81_kernel")) != MG_OK) return false;
        if ((e = cudaEventRecord(done[cur], s)) != cudaSuccess) {
            st = mg::cuda_fail(h, e, "cudaEventRecord");
            return false;
        }
        used[cur] = true;
        cur ^= 1;
        nrot = nsw = 0;
        if (used[cur]) {
            const auto t0 = std::chrono::steady_clock::now();
            e = cudaEventSynchronize(done[cur]);
            wait_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            if (e != cudaSuccess) {
                st = mg::cuda_fail(h, e, "cudaEventSynchronize");
                return false;
            }
        }
        return true;
    }
    bool sweep(int start, int len) override {
        if (nrot + (size_t)len > cap_rot || nsw + 1 > cap_sw)
            if (!flush()) return false;
        hsw[cur][nsw++] = Sweep{start, len, (int)nrot, 0};
        return true;
    }
    void rot(double c, double s) override {
        hcs[cur][nrot++] = make_double2(c, s);
        ++total_rot;
    }
    ~GpuRotSink() override {
        for (cudaEvent_t& e : done)
            if (e) cudaEventDestroy(e);
    }
};

// An event destroyed on every return path.
struct ScopedEvent {
    cudaEvent_t e = nullptr;
    ~ScopedEvent() {
        if (e) cudaEventDestroy(e);
    }
};

// Device workspace of the tridiagonalisation: barrier + error word, d, e, vc, vd.
size_t td_ws_bytes(int n) { return 256 + 4 * mg::align_up((size_t)(n + 1) * 8, 256); }

}  // namespace

namespace mg {

// Tridiagonalises the symmetric W (n x n, ld ldw; lower triangle read) in
// place: reflector m below the diagonal of column m, d (n) / e (n - 1) into
// the device vectors.  Uses the start of h->ws.
static mg_status_t tridiag81(mg_handle_t h, int n, double* W, int ldw, double** d_out, double** e_out) {
    MG_TRY(ensure_ws(h, td_ws_bytes(n)));
    char* b = (char*)h->ws;
    const size_t vb = align_up((size_t)(n + 1) * 8, 256);
    TdArgs a;
    a.W = W;
    a.ld = ldw;
    a.n = n;
    a.bar = (unsigned*)b;
    a.err = (int*)(b + 64);
    a.d = (double*)(b + 256);
    a.e = (double*)(b + 256 + vb);
    a.vc = (double*)(b + 256 + 2 * vb);
    a.vd = (double*)(b + 256 + 3 * vb);
    cudaStream_t st = h->stream;
    MG_CHECK_CUDA(h, cudaMemsetAsync(b, 0, 256, st));
    MG_CHECK_CUDA(h, cudaMemsetAsync(a.e, 0, vb, st));
    if (n >= 3) {
        ProfScope prof(h, "tridiag81", 4.0 / 3.0 * n * (double)n * n, 8.0 * n * (double)n * n / 1.5);
        const int smem = TD_SMEM_DBL * (int)sizeof(double);
        MG_CHECK_CUDA(h, cudaFuncSetAttribute(tridiag81_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        int per_sm = 0;
        MG_CHECK_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tridiag81_kernel, TD_THREADS, smem));
        if (per_sm < 1) return fail(h, MG_ERR_CUDA, "tridiag81_kernel: no co-resident CTA");
        const int G = h->num_sms * (per_sm < 2 ? per_sm : 2);
        if (G < 2) return fail(h, MG_ERR_UNSUPPORTED, "tridiag81_kernel needs two co-resident CTAs");
        // MG_TRIDIAG_STAGE_CAP lowers the on-chip threshold of phase 2 (test hook for the global-memory path)
        a.stage_cap = TD_STAGE;
        if (const char* cap = getenv("MG_TRIDIAG_STAGE_CAP")) {
            const int c = atoi(cap);
            if (c >= 0 && c < TD_STAGE) a.stage_cap = c;
        }
        void* args[] = {&a};
        cudaError_t e = cudaLaunchCooperativeKernel((const void*)tridiag81_kernel, dim3(G), dim3(TD_THREADS), args,
                                                    (size_t)smem, st);
        if (e != cudaSuccess) return cuda_fail(h, e, "tridiag81_kernel launch");
        h->launches++;
    }
    td_tail_kernel<<<1, 32, 0, st>>>(W, ldw, n, a.d, a.e);
    MG_TRY(post_launch(h, "td_tail_kernel"));
    *d_out = a.d;
    *e_out = a.e;
    return MG_OK;
}

static mg_status_t formq81(mg_handle_t h, int n, const double* U, int ldu, double* Q, int ldq) {
    cudaStream_t st = h->stream;
    ProfScope prof(h, "formq81", 4.0 / 3.0 * n * (double)n * n, 0);
    const int fq_smem = (FQ_COLS + 2) * n * (int)sizeof(double);
    // MG_FORMQ_NMAX lowers the order up to which Q is formed on chip (test hook for the global-memory kernel)
    int nmax = FQ_NMAX;
    if (const char* v = getenv("MG_FORMQ_NMAX")) {
        const int c = atoi(v);
        if (c >= 0 && c < FQ_NMAX) nmax = c;
    }
    if (n >= 3 && n <= nmax && fq_smem <= h->max_smem_optin) {
        MG_CHECK_CUDA(h, cudaFuncSetAttribute(formq81_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              fq_smem));
        formq81_smem_kernel<<<(n + FQ_COLS - 1) / FQ_COLS, FQ_THREADS, fq_smem, st>>>(U, ldu, n, Q, ldq);
        return post_launch(h, "formq81_smem_kernel");
    }
    evd_identity_kernel<<<evd_grid(h, (size_t)n * n), 256, 0, st>>>(Q, ldq, n);
    MG_TRY(post_launch(h, "evd_identity_kernel"));
    if (n >= 3) {
        const int warps = (n + 3) / 4;
        formq81_kernel<<<(warps * 32 + 127) / 128, 128, 0, st>>>(U, ldu, n, Q, ldq);
        MG_TRY(post_launch(h, "formq81_kernel"));
    }
    return MG_OK;
}

static mg_status_t td_check(mg_handle_t h, const char* who) {
    int* hw = (int*)h->hws;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw, (char*)h->ws + 64, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hw[0]) return fail(h, MG_TIMEOUT, "%s: a grid barrier timed out", who);
    return MG_OK;
}

}  // namespace mg

extern "C" {

mg_status_t mg_dtridiag81(mg_handle_t h, int n, double* A, int lda, double* Q, int ldq, double* d, double* e) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || lda < (n > 1 ? n : 1) || ldq < (n > 1 ? n : 1) || (n > 0 && (!A || !Q || !d || (n > 1 && !e))))
        return mg::fail(h, MG_ERR_ARG, "mg_dtridiag81: bad arguments");
    if (n == 0) return MG_OK;
    MG_TRY(mg::ensure_hws(h, 64));
    double *dd, *de;
    MG_TRY(mg::tridiag81(h, n, A, lda, &dd, &de));
    MG_TRY(mg::formq81(h, n, A, lda, Q, ldq));
    cudaStream_t st = h->stream;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(d, dd, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    if (n > 1) MG_CHECK_CUDA(h, cudaMemcpyAsync(e, de, (size_t)(n - 1) * 8, cudaMemcpyDeviceToDevice, st));
    return mg::td_check(h, "mg_dtridiag81");
}

mg_status_t mg_devd_q(mg_handle_t h, int n, const double* A, int lda, double eps, double* E, int lde, double* Q,
                      int ldq, double* w) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || lda < (n > 1 ? n : 1) || lde < (n > 1 ? n : 1) || ldq < (n > 1 ? n : 1) ||
        (n > 0 && (!A || !E || !Q)) || !(eps >= 0.0))
        return mg::fail(h, MG_ERR_ARG, "mg_devd_q: bad arguments");
    if (n == 0) return MG_OK;
    cudaStream_t st = h->stream;
    // rotation chunks: two pinned staging areas and two device areas after the
    // tridiagonalisation workspace; the workspaces are sized first (growing
    // them later would move the tridiagonalisation's vectors)
    GpuRotSink sink;
    sink.h = h;
    sink.Q = Q;
    sink.ldq = ldq;
    sink.n = n;
    sink.cap_rot = (size_t)1 << 20;
    if (sink.cap_rot < (size_t)n) sink.cap_rot = (size_t)n;
    sink.cap_sw = sink.cap_rot / 8 + 64;
    const size_t chunk_bytes = mg::align_up(sink.cap_rot * sizeof(double2), 256) +
                               mg::align_up(sink.cap_sw * sizeof(Sweep), 256);
    const size_t base = mg::align_up(td_ws_bytes(n), 256);
    const size_t hv = mg::align_up((size_t)(n + 1) * 8, 256);
    const size_t hbase0 = 256 + 2 * hv;  // pinned: status word, d, e, then the chunks
    MG_TRY(mg::ensure_ws(h, base + 2 * chunk_bytes));
    MG_TRY(mg::ensure_hws(h, hbase0 + 2 * chunk_bytes));
    MG_TRY(mg::ensure_lookahead(h));
    // E is the work matrix, as in Mat (EVD/EVD_Q.h:9-10)
    if (A != E) {
        evd_copy_lower_kernel<<<evd_grid(h, (size_t)n * n), 256, 0, st>>>(A, lda, n, E, lde);
        MG_TRY(mg::post_launch(h, "evd_copy_lower_kernel"));
    }
    double *dd, *de;
    MG_TRY(mg::tridiag81(h, n, E, lde, &dd, &de));
    // d, e and the barrier status go to the host on the side stream as soon as
    // the tridiagonalisation is done: the host recurrence then runs beside
    // the Q formation (the rotations follow it on the handle's stream)
    ScopedEvent td_done;
    MG_CHECK_CUDA(h, cudaEventCreateWithFlags(&td_done.e, cudaEventDisableTiming));
    MG_CHECK_CUDA(h, cudaEventRecord(td_done.e, st));
    MG_TRY(mg::formq81(h, n, E, lde, Q, ldq));
    int* herr = (int*)h->hws;
    double* hd = (double*)((char*)h->hws + 256);
    double* he = (double*)((char*)h->hws + 256 + hv);
    {
        cudaStream_t side = h->pp_stream;
        cudaError_t e = cudaStreamWaitEvent(side, td_done.e, 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hd, dd, (size_t)n * 8, cudaMemcpyDeviceToHost, side);
        if (e == cudaSuccess && n > 1) e = cudaMemcpyAsync(he, de, (size_t)(n - 1) * 8, cudaMemcpyDeviceToHost, side);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(herr, (char*)h->ws + 64, sizeof(int), cudaMemcpyDeviceToHost, side);
        if (e == cudaSuccess) e = cudaStreamSynchronize(side);
        if (e != cudaSuccess) return mg::cuda_fail(h, e, "mg_devd_q: tridiagonal copy");
    }
    if (herr[0]) {
        cudaStreamSynchronize(st);
        return mg::fail(h, MG_TIMEOUT, "mg_devd_q: a grid barrier timed out");
    }
    std::vector<double> a(hd, hd + n), b((size_t)n + 1, 0.0);
    if (n > 1) std::copy(he, he + (n - 1), b.begin());
    b[n - 1] = 0.0;  // EVD/__QR.h:154-157
    // after the host read the status word: reset it for the rotation kernels
    sink.err = (int*)((char*)h->ws + 64);
    MG_CHECK_CUDA(h, cudaMemsetAsync(sink.err, 0, sizeof(int), st));
    for (int i = 0; i < 2; ++i) {
        char* dbase = (char*)h->ws + base + i * chunk_bytes;
        char* hbase = (char*)h->hws + hbase0 + i * chunk_bytes;
        sink.dcs[i] = (double2*)dbase;
        sink.dsw[i] = (Sweep*)(dbase + mg::align_up(sink.cap_rot * sizeof(double2), 256));
        sink.hcs[i] = (double2*)hbase;
        sink.hsw[i] = (Sweep*)(hbase + mg::align_up(sink.cap_rot * sizeof(double2), 256));
        MG_CHECK_CUDA(h, cudaEventCreateWithFlags(&sink.done[i], cudaEventDisableTiming));
    }
    long long budget = 64LL * n;
    bool ok;
    {
        mg::ProfScope prof(h, "qr_sweeps81", 0, 0);
        const auto t0 = std::chrono::steady_clock::now();
        ok = qr_sweeps(a.data(), b.data(), 0, n - 1, eps, budget, sink) && sink.flush();
        const double host_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        mg::prof_host(h, "qr_sweeps81_host", host_ms - sink.wait_ms, (double)sink.total_rot);
        mg::prof_host(h, "qr_sweeps81_wait", sink.wait_ms, 0);
    }
    mg_status_t ret = sink.st;
    // eigenvalues into E's diagonal (EVD/__QR.h:161-168) and optionally into w
    double* dw = (double*)((char*)h->ws + 256);  // d's device slot, no longer needed
    if (ret == MG_OK) {
        cudaError_t e = cudaMemcpyAsync(dw, a.data(), (size_t)n * 8, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) ret = mg::cuda_fail(h, e, "EVD_Q eigenvalue upload");
    }
    if (ret == MG_OK) {
        evd_diag_kernel<<<evd_grid(h, (size_t)n * n), 256, 0, st>>>(E, lde, n, dw);
        ret = mg::post_launch(h, "evd_diag_kernel");
    }
    if (ret == MG_OK && w) {
        cudaError_t e = cudaMemcpyAsync(w, dw, (size_t)n * 8, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) ret = mg::cuda_fail(h, e, "EVD_Q eigenvalue copy");
    }
    cudaError_t se = cudaStreamSynchronize(st);
    if (ret == MG_OK && se != cudaSuccess) ret = mg::cuda_fail(h, se, "cudaStreamSynchronize");
    if (ret != MG_OK) return ret;
    MG_TRY(mg::td_check(h, "mg_devd_q rotations"));
    if (!ok) return mg::fail(h, MG_NOT_CONVERGED, "mg_devd_q: the QR sweeps did not deflate within %d sweeps", 64 * n);
    return MG_OK;
}

// Host only: the QR sweeps of EVD_Q on a tridiagonal (EVD/__QR.h:50-142),
// eigenvalues only.  No CUDA call.
mg_status_t mg_dsteqr81_host(int n, double* d, const double* e, double eps, long long* rotations) {
    if (n < 0 || (n > 0 && !d) || (n > 1 && !e) || !(eps >= 0.0)) return MG_ERR_ARG;
    if (rotations) *rotations = 0;
    if (n == 0) return MG_OK;
    std::vector<double> b((size_t)n + 1, 0.0);
    if (n > 1) std::copy(e, e + (n - 1), b.begin());
    CountSink sink;
    long long budget = 64LL * n;
    const bool ok = qr_sweeps(d, b.data(), 0, n - 1, eps, budget, sink);
    if (rotations) *rotations = sink.count;
    return ok ? MG_OK : MG_NOT_CONVERGED;
}

}  // extern "C"
