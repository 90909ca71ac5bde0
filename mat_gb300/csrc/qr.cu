// Blocked Householder QR with the full m x m Q (Mat's QR(A, Q, R, QR_Householder)).
//
// Reference path (Mat-8.3.1/QR): QR (QR.h:8-25) -> __QR_HouseHolder_Blocked
// (__Householder_Blocked.h:215-245, 336-353), BS = 48 (AVX-512, Mat.h:77-79):
// per block of columns the panel __QR_HouseHolder_Blocked2 (:63-84: LAPACK-
// style reflectors, v0 = 1 implicit, tau = (x0 + cr)/cr, R_rr = -cr with
// cr = sign(x0)||x||), the upper-triangular T of the compact WY form
// (CalculateT, :87-103), the trailing update R2 -= V (T^T (V^T R2)) (:144-212),
// then the full Q accumulated backwards, Q_j -= V (T (V^T Q_j)) (CalculateQ,
// :248-333), and R zeroed below the diagonal (:346-352).
//
// GPU design (results bit-identical to Mat's AVX-512 build for the blocked
// path):
//  - every dot product is computed by one warp in the reduction order of
//    Mat's AVX-512 __dot (Calculate/__AVX512_double.h:110-133): lane p holds
//    partial sum p (= Mat's accumulator q = p/8, lane p%8), fused over
//    elements 32t + p, then the remaining full 8-blocks into lanes 0..7, the
//    lane-wise (a0+a1)+(a2+a3), the fused tail and the 8->4->2->1 sum;
//  - the panel is one cooperative kernel with one CTA per panel column and
//    two bounded grid barriers per reflector (after the reflector, after the
//    columns it updates);
//  - T: four lanes per inner product V_l^T V_i in the order of Mat's generic
//    __dot (CalculateT passes const pointers, which selects that template),
//    then the k^2/2 recurrence;
//  - the trailing update and the Q accumulation: three FP64 DMMA GEMMs on an
//    explicit unit-lower V (ones on the diagonal, zeros above), whose
//    per-element fused chains follow Mat's packed GEMMs.
// Matrices with min(m, n) <= 2*BS use Mat's unblocked normalisation
// (QR/__HouseHolder.h:179-208) there; this implementation factors them as a
// single panel of the blocked algorithm, which agrees to rounding.
#include <cmath>

#include "grid_sync.cuh"
#include "mg_internal.cuh"

namespace {

constexpr int QR_BS = 48;  // Mat-8.3.1/Mat.h:77-79 (AVX-512)
constexpr int QR_THREADS = 512;  // one CTA per panel column: its loops over the column keep many loads in flight

// Mat's AVX-512 __dot(a, b, len), computed by one full warp; every lane returns
// the result.  Loads bypass L1 (the operands may have been written by other
// CTAs of the same cooperative launch).
__device__ double warp_dot_mat(const double* __restrict__ a, const double* __restrict__ b, int len) {
    const int lane = threadIdx.x & 31;
    const int nb = len / 8;
    double acc = 0.0;
    int i = 0;
    // four 8-lane accumulators over strides of 32 elements: lane p <- elements 32t + p;
    // loads run PF steps ahead of the (ordered) fused chain
    constexpr int PF = 16;
    for (; i + 4 * PF <= nb; i += 4 * PF) {
        double xa[PF], xb[PF];
#pragma unroll
        for (int u = 0; u < PF; ++u) {
            xa[u] = __ldcg(a + (i + 4 * u) * 8 + lane);
            xb[u] = __ldcg(b + (i + 4 * u) * 8 + lane);
        }
#pragma unroll
        for (int u = 0; u < PF; ++u) acc = fma(xa[u], xb[u], acc);
    }
    for (; i <= nb - 4; i += 4) acc = fma(__ldcg(a + i * 8 + lane), __ldcg(b + i * 8 + lane), acc);
    // remaining full 8-blocks into the first accumulator (lanes 0..7)
    for (; i < nb; ++i)
        if (lane < 8) acc = fma(__ldcg(a + i * 8 + lane), __ldcg(b + i * 8 + lane), acc);
    const double x1 = __shfl_down_sync(0xffffffffu, acc, 8);
    const double x2 = __shfl_down_sync(0xffffffffu, acc, 16);
    const double x3 = __shfl_down_sync(0xffffffffu, acc, 24);
    double s = (acc + x1) + (x2 + x3);  // meaningful in lanes 0..7
    const int rem = len - nb * 8;
    if (lane < rem) s = fma(__ldcg(a + nb * 8 + lane), __ldcg(b + nb * 8 + lane), s);
    const double s4 = __shfl_down_sync(0xffffffffu, s, 4);
    const double h4 = s + s4;  // lanes 0..3
    const double h2 = h4 + __shfl_down_sync(0xffffffffu, h4, 2);  // lanes 0..1
    const double r = h2 + __shfl_down_sync(0xffffffffu, h2, 1);   // lane 0
    return __shfl_sync(0xffffffffu, r, 0);
}

// The same __dot(a, b, len) computed by a whole CTA of QR_THREADS threads:
// all threads stage the operands through shared memory in chunks of
// QR_DOT_CH elements (each thread keeps its chunk loads in flight together),
// and warp 0 runs the 32 ordered fused chains of warp_dot_mat on them (lane
// p <- elements 32t + p), then the identical tail and reduction.  One warp
// streaming both operands from L2 alone kept too few loads in flight (about
// 64 us for a 16384-element dot).  Call from every thread of the CTA; every
// thread returns the result.  sbuf holds 2 * QR_DOT_CH doubles.
constexpr int QR_DOT_CH = 2048;

__device__ double block_dot_mat(const double* __restrict__ a, const double* __restrict__ b, int len,
                                double* sbuf, double* s_out) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb = len / 8;
    const int nmain = 32 * (nb / 4);  // elements of the 32-strided fused chains
    double acc = 0.0;
    for (int c0 = 0; c0 < nmain; c0 += QR_DOT_CH) {
        const int cn = min(QR_DOT_CH, nmain - c0);
        __syncthreads();  // the previous chunk is consumed
        {
            constexpr int PER = QR_DOT_CH / QR_THREADS;
            double ta[PER], tb[PER];
#pragma unroll
            for (int u = 0; u < PER; ++u) {
                const int e = tid + u * QR_THREADS;
                ta[u] = e < cn ? __ldcg(a + c0 + e) : 0.0;
                tb[u] = e < cn ? __ldcg(b + c0 + e) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < PER; ++u) {
                const int e = tid + u * QR_THREADS;
                sbuf[e] = ta[u];
                sbuf[QR_DOT_CH + e] = tb[u];
            }
        }
        __syncthreads();
        if (warp == 0) {
            // eight shared loads ahead of the ordered chain (cn is a multiple of 32)
            int t = lane;
            for (; t + 7 * 32 < cn; t += 8 * 32) {
                double xa[8], xb[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    xa[u] = sbuf[t + 32 * u];
                    xb[u] = sbuf[QR_DOT_CH + t + 32 * u];
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) acc = fma(xa[u], xb[u], acc);
            }
            for (; t < cn; t += 32) acc = fma(sbuf[t], sbuf[QR_DOT_CH + t], acc);
        }
    }
    if (warp == 0) {
        int i = nb / 4 * 4;
        // remaining full 8-blocks into the first accumulator (lanes 0..7)
        for (; i < nb; ++i)
            if (lane < 8) acc = fma(__ldcg(a + i * 8 + lane), __ldcg(b + i * 8 + lane), acc);
        const double x1 = __shfl_down_sync(0xffffffffu, acc, 8);
        const double x2 = __shfl_down_sync(0xffffffffu, acc, 16);
        const double x3 = __shfl_down_sync(0xffffffffu, acc, 24);
        double sx = (acc + x1) + (x2 + x3);
        const int rem = len - nb * 8;
        if (lane < rem) sx = fma(__ldcg(a + nb * 8 + lane), __ldcg(b + nb * 8 + lane), sx);
        const double s4 = __shfl_down_sync(0xffffffffu, sx, 4);
        const double h4 = sx + s4;
        const double h2 = h4 + __shfl_down_sync(0xffffffffu, h4, 2);
        const double r = h2 + __shfl_down_sync(0xffffffffu, h2, 1);
        if (lane == 0) *s_out = r;
    }
    __syncthreads();
    return *s_out;
}

struct QrPanelWs {
    unsigned* bar;
    int* err;
};

// Panel of b columns at P (h rows, ld ldr).  CTA c owns column c.
__global__ void __launch_bounds__(QR_THREADS) qr_panel_kernel(double* __restrict__ P, int ldr, int h, int b,
                                                               double* __restrict__ tau, QrPanelWs ws) {
    __shared__ double s_q, s_hr, s_dot;
    __shared__ int s_skip;
    __shared__ double sbuf[2 * QR_DOT_CH];
    const int c = blockIdx.x;
    unsigned phase = 0;
    for (int r = 0; r < b; ++r) {
        const int len = h - r;
        double* w = P + r + (size_t)r * ldr;
        if (c == r) {
            const double ss = block_dot_mat(w, w, len, sbuf, &s_dot);
            {
                if (threadIdx.x == 0) {
                    double cr = sqrt(ss);
                    if (cr == 0.0) {
                        tau[r] = 0.0;
                        s_skip = 1;
                    } else {
                        const double x0 = __ldcg(w);
                        if (x0 < 0.0) cr = -cr;
                        const double w0 = x0 + cr;
                        s_hr = 1.0 / w0;
                        w[0] = -cr;
                        tau[r] = w0 / cr;
                        s_skip = 0;
                    }
                }
            }
            __syncthreads();
            if (!s_skip) {
                const double hr = s_hr;
                for (int i0 = 1 + threadIdx.x; i0 < len; i0 += 8 * blockDim.x) {
                    double x[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int i = i0 + u * blockDim.x;
                        x[u] = i < len ? w[i] : 0.0;
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int i = i0 + u * blockDim.x;
                        if (i < len) w[i] = x[u] * hr;
                    }
                }
            }
        }
        if (!mg::grid_barrier(ws.bar, (++phase) * gridDim.x, ws.err)) return;
        // apply H_r to the columns right of it (Mat skips them when the column was zero)
        if (c > r && __ldcg(tau + r) != 0.0) {
            double* col = P + r + (size_t)c * ldr;
            {
                const double d = __ldcg(col) + block_dot_mat(w + 1, col + 1, len - 1, sbuf, &s_dot);
                if (threadIdx.x == 0) s_q = -d * __ldcg(tau + r);
            }
            __syncthreads();
            const double q = s_q;
            for (int i0 = threadIdx.x; i0 < len; i0 += 8 * blockDim.x) {
                double xv[8], xc[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int i = i0 + u * blockDim.x;
                    xv[u] = i == 0 ? 1.0 : (i < len ? __ldcg(w + i) : 0.0);
                    xc[u] = i < len ? col[i] : 0.0;
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int i = i0 + u * blockDim.x;
                    if (i < len) col[i] = fma(xv[u], q, xc[u]);
                }
            }
        }
        if (!mg::grid_barrier(ws.bar, (++phase) * gridDim.x, ws.err)) return;
    }
}

// Mat's generic __dot template as the reference build evaluates it (used by
// CalculateT, QR/__Householder_Blocked.h:95, whose operands are const): four
// partial sums over i mod 4, the first floor(n4/32)*32 elements multiplied
// and added separately (vectorised in the reference build), the rest fused,
// ((t0 + t1) + t2) + t3, then a fused tail.  Computed by four consecutive
// lanes (one partial sum each); lane q0 of the group returns the result.
__device__ double quad_dot_generic(const double* __restrict__ a, const double* __restrict__ b, int len, int q) {
    const int n4 = 4 * (len / 4), nv = (n4 / 32) * 32;
    double t = 0.0;
    int i = q;
    constexpr int PF = 16;  // loads run PF steps ahead of the (ordered) chain
    for (; i + 4 * (PF - 1) < nv; i += 4 * PF) {
        double xa[PF], xb[PF];
#pragma unroll
        for (int u = 0; u < PF; ++u) {
            xa[u] = __ldcg(a + i + 4 * u);
            xb[u] = __ldcg(b + i + 4 * u);
        }
#pragma unroll
        for (int u = 0; u < PF; ++u) t = __dadd_rn(t, __dmul_rn(xa[u], xb[u]));
    }
    for (; i < nv; i += 4) t = __dadd_rn(t, __dmul_rn(__ldcg(a + i), __ldcg(b + i)));
    for (; i + 4 * (PF - 1) < n4; i += 4 * PF) {
        double xa[PF], xb[PF];
#pragma unroll
        for (int u = 0; u < PF; ++u) {
            xa[u] = __ldcg(a + i + 4 * u);
            xb[u] = __ldcg(b + i + 4 * u);
        }
#pragma unroll
        for (int u = 0; u < PF; ++u) t = fma(xa[u], xb[u], t);
    }
    for (; i < n4; i += 4) t = fma(__ldcg(a + i), __ldcg(b + i), t);
    // lanes q = 0..3 of a group of four consecutive lanes
    const unsigned full = 0xffffffffu;
    const double t1 = __shfl_down_sync(full, t, 1);
    const double t2 = __shfl_down_sync(full, t, 2);
    const double t3 = __shfl_down_sync(full, t, 3);
    double ans = ((t + t1) + t2) + t3;  // meaningful in lane q == 0
    if (q == 0)
        for (int j = n4; j < len; ++j) ans = fma(__ldcg(a + j), __ldcg(b + j), ans);
    return ans;
}

// s[l + i*b] = V_l[i] + dot(V_l[i+1..], V_i[i+1..]) for l < i; eight pairs per
// warp, four lanes per pair.
__global__ void qr_t_dots_kernel(const double* __restrict__ P, int ldr, int h, int b, double* __restrict__ S) {
    const int lane = threadIdx.x & 31, q = lane & 3;
    const int gp = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;  // pair index
    const int npairs = b * (b - 1) / 2;
    const bool active = gp < npairs;
    int i = 1, l = 0;
    if (active) {
        int base = 0;
        while (base + i <= gp) {
            base += i;
            ++i;
        }
        l = gp - base;
    }
    const double* vl = P + (size_t)l * ldr;
    const double* vi = P + (size_t)i * ldr;
    const int len = active ? h - i - 1 : 0;
    const double d = quad_dot_generic(vl + i + 1, vi + i + 1, len, q);
    if (active && q == 0) S[l + (size_t)i * b] = __ldcg(vl + i) + d;
}

// T (b x b, ld b, upper) from S and tau (Mat's CalculateT recurrence).
__global__ void qr_t_kernel(const double* __restrict__ S, const double* __restrict__ tau, int b, double* __restrict__ T) {
    // S and T staged in shared memory; thread r owns row r of T, so every
    // w_r = sum_c T(r, c) S(c, i) is one fused chain over c in ascending order
    // (the order of Mat's loop) while the rows proceed in parallel.
    __shared__ double ss[QR_BS * QR_BS], st[QR_BS * QR_BS], stau[QR_BS];
    const int r = threadIdx.x;
    for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
        ss[e] = S[e];
        st[e] = 0.0;
    }
    if (r < b) stau[r] = tau[r];
    __syncthreads();
    if (r == 0) st[0] = stau[0];
    __syncthreads();
    for (int i = 1; i < b; ++i) {
        if (r < i) {
            double w = 0.0;
            for (int c = r; c < i; ++c) w = fma(st[r + c * b], ss[c + i * b], w);
            st[r + i * b] = w * -stau[i];
        } else if (r == i) {
            st[i + i * b] = stau[i];
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < b * b; e += blockDim.x) T[e] = st[e];
}

// Explicit unit-lower V (h x b, ld h) from the reflectors stored below the diagonal of P.
__global__ void qr_expand_v_kernel(const double* __restrict__ P, int ldr, int h, int b, double* __restrict__ V) {
    const size_t total = (size_t)h * b;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % h), c = (int)(e / h);
        V[e] = r > c ? P[r + (size_t)c * ldr] : (r == c ? 1.0 : 0.0);
    }
}

__global__ void identity_kernel(double* __restrict__ Q, int ldq, int m) {
    const size_t total = (size_t)m * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % m), c = (int)(e / m);
        Q[r + (size_t)c * ldq] = r == c ? 1.0 : 0.0;
    }
}

__global__ void zero_below_kernel(double* __restrict__ R, int ldr, int m, int n) {
    const size_t total = (size_t)m * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % m), c = (int)(e / m);
        if (r > c) R[r + (size_t)c * ldr] = 0.0;
    }
}

__global__ void copy_kernel(const double* __restrict__ A, int lda, int m, int n, double* __restrict__ B, int ldb) {
    const size_t total = (size_t)m * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % m), c = (int)(e / m);
        B[r + (size_t)c * ldb] = A[r + (size_t)c * lda];
    }
}

struct QrWs {
    unsigned* bar;
    int* err;
    double* tau;  // k
    double* T;    // ceil(k/BS) blocks of BS*BS
    double* S;    // BS*BS
    double* V;    // m*BS
    double* W;    // BS*max(m,n)
    double* W2;   // BS*max(m,n)
};

size_t carve_qr(mg_handle_t h, int m, int n, QrWs* w) {
    const int k = m < n ? m : n;
    const int nblk = (k + QR_BS - 1) / QR_BS;
    const int mx = m > n ? m : n;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = mg::align_up(off + bytes, 256);
        return o;
    };
    const size_t o0 = take(256);
    const size_t oTau = take((size_t)k * 8);
    const size_t oT = take((size_t)nblk * QR_BS * QR_BS * 8);
    const size_t oS = take((size_t)QR_BS * QR_BS * 8);
    const size_t oV = take((size_t)m * QR_BS * 8);
    const size_t oW = take((size_t)QR_BS * mx * 8);
    const size_t oW2 = take((size_t)QR_BS * mx * 8);
    if (w) {
        char* b = (char*)h->ws;
        w->bar = (unsigned*)(b + o0);
        w->err = (int*)(b + o0 + 64);
        w->tau = (double*)(b + oTau);
        w->T = (double*)(b + oT);
        w->S = (double*)(b + oS);
        w->V = (double*)(b + oV);
        w->W = (double*)(b + oW);
        w->W2 = (double*)(b + oW2);
    }
    return off;
}

int grid_cap(mg_handle_t h, size_t total) {
    size_t g = (total + 255) / 256;
    const size_t cap = (size_t)h->num_sms * 8;
    return (int)(g < 1 ? 1 : g > cap ? cap : g);
}

// ---------------------------------------------------------- unblocked path
// Mat's QR for min(m, n) <= 2*BS (QR/__HouseHolder.h:179-208 and
// __HouseHolder_Q1 :48-79): reflector r is w = x / sqrt(cr (x0 + cr)) with
// x0 += cr (so H = I - w w^T), applied as col -= w (w^T col) to columns r..n-1
// (R's entries below the diagonal keep the rounding-level values this leaves);
// Q is then built backwards: with T2 the (m-r-1)-square trailing block,
// column i >= 1 of the new (m-r)-square block is [w0 t; w[1..] t + T2(:, i-1)]
// with t = -w[1..]^T T2(:, i-1), and column 0 is -w0 w + e0.  Mat runs this in
// place inside Q's buffer; every new column depends only on w and T2(:, i-1),
// which no earlier column overwrites, so the columns are computed in parallel
// from a separate T2 buffer with the same per-element operations.
__global__ void qru_reflector_kernel(const double* __restrict__ R, int ldr, int m, int r, double* __restrict__ w,
                                     int* __restrict__ skip) {
    __shared__ double s_hr;
    __shared__ int s_skip;
    const int len = m - r;
    const double* x = R + r + (size_t)r * ldr;
    for (int i = threadIdx.x; i < len; i += blockDim.x) w[i] = x[i];
    __syncthreads();
    if (threadIdx.x < 32) {
        const double ss = warp_dot_mat(w, w, len);
        if (threadIdx.x == 0) {
            double cr = sqrt(ss);
            if (cr == 0.0) {
                s_skip = 1;
            } else {
                if (w[0] < 0.0) cr = -cr;
                const double w0 = w[0] + cr;
                w[0] = w0;
                s_hr = 1.0 / sqrt(cr * w0);
                s_skip = 0;
            }
            *skip = s_skip;
        }
    }
    __syncthreads();
    if (!s_skip)
        for (int i = threadIdx.x; i < len; i += blockDim.x) w[i] = w[i] * s_hr;
}

// col -= w (w^T col) for columns r..n-1 of R, one warp per column.
__global__ void qru_apply_kernel(double* __restrict__ R, int ldr, int m, int n, int r, const double* __restrict__ w,
                                 const int* __restrict__ skip) {
    if (*skip) return;
    const int c = r + (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= n) return;
    const int len = m - r;
    double* col = R + r + (size_t)c * ldr;
    const double d = -warp_dot_mat(w, col, len);
    for (int i = lane; i < len; i += 32) col[i] = fma(w[i], d, col[i]);
}

// Columns i >= 1 of the new block B1 (r1 x r1) from T2 (r2 = r1 - 1 square), one warp per column.
__global__ void qru_q1_kernel(const double* __restrict__ w, int r1, const double* __restrict__ T2,
                              double* __restrict__ B1) {
    const int i = 1 + (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= r1) return;
    const int r2 = r1 - 1;
    const double* src = T2 + (size_t)(i - 1) * r2;
    const double temp = -warp_dot_mat(w + 1, src, r2);
    double* dst = B1 + (size_t)i * r1;
    if (lane == 0) dst[0] = w[0] * temp;
    for (int e = lane; e < r2; e += 32) dst[1 + e] = fma(w[1 + e], temp, __ldcg(src + e));
}

// Column 0 of B1: -w0 w, then + 1 on the diagonal.
__global__ void qru_q1_col0_kernel(const double* __restrict__ w, int r1, double* __restrict__ B1) {
    const double q = -w[0];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < r1; e += gridDim.x * blockDim.x) {
        const double v = w[e] * q;
        B1[e] = e == 0 ? v + 1.0 : v;
    }
}

}  // namespace

namespace mg {

// In place on R (m x n, ld ldr): R above the diagonal, reflectors below;
// tau and the T blocks in the workspace carved by carve_qr.
static mg_status_t dgeqrf_blocked(mg_handle_t h, int m, int n, double* R, int ldr, QrWs& w) {
    const int k = m < n ? m : n;
    cudaStream_t st = h->stream;
    for (int j = 0; j < k; j += QR_BS) {
        const int b = QR_BS < k - j ? QR_BS : k - j;
        const int hh = m - j;
        double* P = R + j + (size_t)j * ldr;
        {
            ProfScope prof(h, "qr_panel", 4.0 * hh * (double)b * b, 16.0 * hh * (double)b);
            MG_CHECK_CUDA(h, cudaMemsetAsync(w.bar, 0, sizeof(unsigned), st));
            double* tau_j = w.tau + j;
            QrPanelWs pws{w.bar, w.err};
            void* args[] = {&P, &ldr, (void*)&hh, (void*)&b, &tau_j, &pws};
            cudaError_t e;
            if (b > 1)
                e = cudaLaunchCooperativeKernel((const void*)qr_panel_kernel, dim3(b), dim3(QR_THREADS), args, 0, st);
            else
                e = cudaLaunchKernel((const void*)qr_panel_kernel, dim3(1), dim3(QR_THREADS), args, 0, st);
            if (e != cudaSuccess) return cuda_fail(h, e, "qr_panel_kernel launch");
            h->launches++;
        }
        double* Tj = w.T + (size_t)(j / QR_BS) * QR_BS * QR_BS;
        {
            ProfScope prof(h, "qr_t", 2.0 * hh * (double)b * b / 2, 8.0 * hh * (double)b);
            const int npairs = b * (b - 1) / 2;
            if (npairs > 0) {
                qr_t_dots_kernel<<<(npairs * 4 + 255) / 256, 256, 0, st>>>(P, ldr, hh, b, w.S);
                MG_TRY(post_launch(h, "qr_t_dots_kernel"));
            }
            qr_t_kernel<<<1, 64, 0, st>>>(w.S, w.tau + j, b, Tj);
            MG_TRY(post_launch(h, "qr_t_kernel"));
        }
        if (j + b < n) {
            const int nc = n - j - b;
            double* R2 = R + j + (size_t)(j + b) * ldr;
            qr_expand_v_kernel<<<grid_cap(h, (size_t)hh * b), 256, 0, st>>>(P, ldr, hh, b, w.V);
            MG_TRY(post_launch(h, "qr_expand_v_kernel"));
            // W = V^T R2; W2 = T^T W; R2 -= V W2.  The first product (48 outputs per
            // column, K = hh) is bound by the length of its fused K chains, not by
            // its width: a look-ahead that updates the next panel's columns first
            // put a second chain on the critical path and was slower.
            {
                ProfScope p1(h, "qr_vtr", 2.0 * b * (double)nc * hh, 0);
                MG_TRY(dgemm_launch(h, 1, 0, b, nc, hh, 1.0, w.V, hh, R2, ldr, 0.0, w.W, b, 0));
            }
            {
                ProfScope p2(h, "qr_tw", 2.0 * b * (double)nc * b, 0);
                MG_TRY(dgemm_launch(h, 1, 0, b, nc, b, 1.0, Tj, b, w.W, b, 0.0, w.W2, b, 0));
            }
            {
                ProfScope p3(h, "qr_vw", 2.0 * hh * (double)nc * b, 0);
                MG_TRY(dgemm_launch(h, 0, 0, hh, nc, b, -1.0, w.V, hh, w.W2, b, 1.0, R2, ldr, 0));
            }
        }
    }
    return MG_OK;
}

// Q (m x m) = H_0 H_1 ... H_{k-1}, accumulated backwards from the identity.
// When block j is applied, Q differs from the identity only in rows and
// columns >= j, so the block update is restricted to Q(j:m, j:m): the
// skipped columns would receive exact zeros (fused chains over zero
// entries), so the result is the one of the full-width update.
static mg_status_t dorgqr_full(mg_handle_t h, int m, int n, const double* R, int ldr, double* Q, int ldq, QrWs& w) {
    const int k = m < n ? m : n;
    cudaStream_t st = h->stream;
    identity_kernel<<<grid_cap(h, (size_t)m * m), 256, 0, st>>>(Q, ldq, m);
    MG_TRY(post_launch(h, "identity_kernel"));
    if (k == 0) return MG_OK;
    const int last = ((k - 1) / QR_BS) * QR_BS;
    for (int j = last; j >= 0; j -= QR_BS) {
        const int b = QR_BS < k - j ? QR_BS : k - j;
        const int hh = m - j;
        const double* P = R + j + (size_t)j * ldr;
        const double* Tj = w.T + (size_t)(j / QR_BS) * QR_BS * QR_BS;
        double* Qj = Q + j + (size_t)j * ldq;
        const int nq = m - j;
        qr_expand_v_kernel<<<grid_cap(h, (size_t)hh * b), 256, 0, st>>>(P, ldr, hh, b, w.V);
        MG_TRY(post_launch(h, "qr_expand_v_kernel"));
        // W = V^T Q_j; W2 = T W; Q_j -= V W2   (Q_j = Q(j:m, j:m))
        MG_TRY(dgemm_launch(h, 1, 0, b, nq, hh, 1.0, w.V, hh, Qj, ldq, 0.0, w.W, b, 0));
        MG_TRY(dgemm_launch(h, 0, 0, b, nq, b, 1.0, Tj, b, w.W, b, 0.0, w.W2, b, 0));
        MG_TRY(dgemm_launch(h, 0, 0, hh, nq, b, -1.0, w.V, hh, w.W2, b, 1.0, Qj, ldq, 0));
    }
    return MG_OK;
}

// Mat's unblocked QR (min(m, n) <= 2*BS): R in place (ld ldr), Q (m x m, ld ldq).
static mg_status_t dqr_unblocked(mg_handle_t h, int m, int n, double* R, int ldr, double* Q, int ldq) {
    const int k = m < n ? m : n;
    cudaStream_t st = h->stream;
    // workspace: the k reflectors (packed, lengths m, m-1, ...), two m x m blocks, a flag per reflector
    const size_t wlen = (size_t)k * m, mm = (size_t)m * m;
    MG_TRY(ensure_ws(h, (wlen + 2 * mm) * sizeof(double) + (size_t)(k + 64) * sizeof(int) + 1024));
    double* wv = (double*)h->ws;
    double* B[2] = {wv + wlen, wv + wlen + mm};
    int* skip = (int*)(B[1] + mm);
    for (int r = 0; r < k; ++r) {
        double* w = wv + (size_t)r * m;
        qru_reflector_kernel<<<1, 256, 0, st>>>(R, ldr, m, r, w, skip + r);
        MG_TRY(post_launch(h, "qru_reflector_kernel"));
        const int cols = n - r;
        qru_apply_kernel<<<(cols * 32 + 255) / 256, 256, 0, st>>>(R, ldr, m, n, r, w, skip + r);
        MG_TRY(post_launch(h, "qru_apply_kernel"));
    }
    // T2 = identity of order m - k
    int cur = 0;
    const int r2 = m - k;
    if (r2 > 0) {
        identity_kernel<<<grid_cap(h, (size_t)r2 * r2), 256, 0, st>>>(B[cur], r2, r2);
        MG_TRY(post_launch(h, "identity_kernel"));
    }
    for (int r = k - 1; r >= 0; --r) {
        const int r1 = m - r;
        const double* w = wv + (size_t)r * m;
        double* B1 = B[cur ^ 1];
        if (r1 > 1) {
            qru_q1_kernel<<<((r1 - 1) * 32 + 255) / 256, 256, 0, st>>>(w, r1, B[cur], B1);
            MG_TRY(post_launch(h, "qru_q1_kernel"));
        }
        qru_q1_col0_kernel<<<grid_cap(h, (size_t)r1), 256, 0, st>>>(w, r1, B1);
        MG_TRY(post_launch(h, "qru_q1_col0_kernel"));
        cur ^= 1;
    }
    MG_CHECK_CUDA(h, cudaMemcpy2DAsync(Q, (size_t)ldq * sizeof(double), B[cur], (size_t)m * sizeof(double),
                                       (size_t)m * sizeof(double), m, cudaMemcpyDeviceToDevice, st));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
    return MG_OK;
}

}  // namespace mg

extern "C" {

mg_status_t mg_dgeqrf(mg_handle_t h, int m, int n, double* A, int lda, double* tau, double* T) {
    if (!h) return MG_ERR_ARG;
    if (m < 0 || n < 0 || lda < (m > 1 ? m : 1) || ((size_t)m * n && (!A || !tau || !T)))
        return mg::fail(h, MG_ERR_ARG, "mg_dgeqrf: bad arguments");
    const int k = m < n ? m : n;
    if (k == 0) return MG_OK;
    MG_TRY(mg::ensure_ws(h, carve_qr(h, m, n, nullptr)));
    MG_TRY(mg::ensure_hws(h, 64));
    QrWs w;
    carve_qr(h, m, n, &w);
    MG_CHECK_CUDA(h, cudaMemsetAsync(w.bar, 0, 256, h->stream));
    MG_TRY(mg::dgeqrf_blocked(h, m, n, A, lda, w));
    const int nblk = (k + QR_BS - 1) / QR_BS;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(tau, w.tau, (size_t)k * 8, cudaMemcpyDeviceToDevice, h->stream));
    MG_CHECK_CUDA(h, cudaMemcpyAsync(T, w.T, (size_t)nblk * QR_BS * QR_BS * 8, cudaMemcpyDeviceToDevice, h->stream));
    int* hw = (int*)h->hws;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw, w.err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hw[0]) return mg::fail(h, MG_TIMEOUT, "dgeqrf: a panel grid barrier timed out");
    return MG_OK;
}

mg_status_t mg_dqr(mg_handle_t h, int m, int n, const double* A, int lda, double* Q, int ldq, double* R, int ldr) {
    if (!h) return MG_ERR_ARG;
    if (m < 0 || n < 0 || lda < (m > 1 ? m : 1) || ldq < (m > 1 ? m : 1) || ldr < (m > 1 ? m : 1) ||
        ((size_t)m * n && (!A || !Q || !R)))
        return mg::fail(h, MG_ERR_ARG, "mg_dqr: bad arguments");
    if (m == 0) return MG_OK;
    if ((m < n ? m : n) <= 2 * QR_BS) {  // Mat's unblocked variant (QR/__HouseHolder.h:179-208)
        if (A != R) {
            copy_kernel<<<grid_cap(h, (size_t)m * n), 256, 0, h->stream>>>(A, lda, m, n, R, ldr);
            MG_TRY(mg::post_launch(h, "copy_kernel"));
        }
        return mg::dqr_unblocked(h, m, n, R, ldr, Q, ldq);
    }
    MG_TRY(mg::ensure_ws(h, carve_qr(h, m, n, nullptr)));
    MG_TRY(mg::ensure_hws(h, 64));
    QrWs w;
    carve_qr(h, m, n, &w);
    cudaStream_t st = h->stream;
    MG_CHECK_CUDA(h, cudaMemsetAsync(w.bar, 0, 256, st));
    if (A != R) {
        copy_kernel<<<grid_cap(h, (size_t)m * n), 256, 0, st>>>(A, lda, m, n, R, ldr);
        MG_TRY(mg::post_launch(h, "copy_kernel"));
    }
    MG_TRY(mg::dgeqrf_blocked(h, m, n, R, ldr, w));
    MG_TRY(mg::dorgqr_full(h, m, n, R, ldr, Q, ldq, w));
    zero_below_kernel<<<grid_cap(h, (size_t)m * n), 256, 0, st>>>(R, ldr, m, n);
    MG_TRY(mg::post_launch(h, "zero_below_kernel"));
    int* hw = (int*)h->hws;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw, w.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
    if (hw[0]) return mg::fail(h, MG_TIMEOUT, "dqr: a panel grid barrier timed out");
    return MG_OK;
}

}  // extern "C"
