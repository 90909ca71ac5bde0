// Blocked right-looking Cholesky (Mat's LLT), LDL^T (Mat's LDLT) and the
// Cholesky solve.
//
// Reference path (Mat-8.3.1/LU/__LLT.h): LLT (:212-246) copies the lower
// triangle and calls __LLT (:94-150), BS = 48 (AVX-512, Mat.h:73-75): per
// block column the unblocked __LLT2 on the diagonal block (:3-13), the
// right-side solve __Solve_direct_XLT on the blocks below (:30-40), and the
// trailing update C -= L21 * L21^T (__times_A_BT_LLT, :59-91) on full
// blocks from the diagonal down; matrices of at most 2*BS columns use __LLT2
// alone; the strict upper triangle is zeroed at the end.
//
// GPU kernels keep Mat's per-element operation sequence (so results are
// bit-identical): the diagonal block by one CTA with one thread per row;
// X := X L^{-T} by one thread per row of the panel (rows are independent);
// the trailing update by the FP64 DMMA GEMM in its in-place C -= A B^T mode
// restricted to tiles that meet the lower triangle.  The same kernels,
// templated on the element type, give the FP32 Cholesky (mg_spotrf) with the
// FP32 SIMT GEMM for the trailing update.
#include "mg_internal.cuh"

namespace {

constexpr int LLT_BS = 48;        // Mat-8.3.1/Mat.h:73-75 (AVX-512)
constexpr int LLT2_MAX = 2 * LLT_BS;
constexpr int LLT2_THREADS = 256;  // lanes over rows, 8 warps over the columns of each column step

// Unblocked Cholesky of the k x k block at L (k <= 96), in place, lower part.
// Column jj: t = 1/sqrt(L(jj,jj)); L(r,jj) *= t for r >= jj; then for
// i > jj: L(r,i) = fma(L(r,jj), -L(i,jj), L(r,i)) for r >= i.
template <typename T>
__global__ void llt2_kernel(T* __restrict__ L, int ldl, int k, int col0, int* __restrict__ info) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    T* s = reinterpret_cast<T*>(s_raw);  // column-major k x k with stride LLT2_MAX
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        const int r = e % k, c = e / k;
        s[r + c * LLT2_MAX] = L[r + (size_t)c * ldl];
    }
    __syncthreads();
    for (int jj = 0; jj < k; ++jj) {
        const T d = s[jj + jj * LLT2_MAX];
        const T t = T(1) / sqrt(d);
        if (threadIdx.x == 0 && !(d > T(0))) atomicCAS(info, 0, col0 + jj + 1);
        __syncthreads();  // every thread has read d before row jj is scaled
        for (int r = jj + threadIdx.x; r < k; r += blockDim.x) s[r + jj * LLT2_MAX] = s[r + jj * LLT2_MAX] * t;
        __syncthreads();
        // the trailing triangle, every element once (the same single fma per
        // element as a row-at-a-time loop), lanes over the rows of a column and
        // the CTA's warps over the columns; not one thread per row, whose
        // longest row was the column step's chain (one warp alone: 3.4x slower)
        {
            const int tr = threadIdx.x & 31, tc = threadIdx.x >> 5, ncg = blockDim.x >> 5;
            for (int i = jj + 1 + tc; i < k; i += ncg) {
                const T lij = s[i + jj * LLT2_MAX];
                for (int rr = i + tr; rr < k; rr += 32)
                    s[rr + i * LLT2_MAX] = fma(s[rr + jj * LLT2_MAX], -lij, s[rr + i * LLT2_MAX]);
            }
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        const int rr = e % k, c = e / k;
        if (rr >= c) L[rr + (size_t)c * ldl] = s[rr + c * LLT2_MAX];
    }
}

// X (rows x k) := X * Lkk^{-T} (Mat's __Solve_direct_XLT), one thread per row:
// for j: x_j *= 1/L(j,j); x_kk = fma(x_j, -L(kk,j), x_kk) for kk > j.  The
// row sits in registers as a rotating window so that the column loop stays
// rolled at fixed register indices (the fully unrolled k = 96 loop spilled to
// the stack and was instruction-fetch bound): at step j, position 0 holds x_j
// and positions 1 .. k-1-j hold x_{j+1} .. x_{k-1}; each step shifts the
// window by one and parks the finished x_j at the end.
constexpr int XLT_THREADS = 128;
template <typename T, int KB>
constexpr size_t xlt_smem_bytes() { return ((size_t)KB * KB + KB) * sizeof(T); }

template <typename T, int KB = LLT_BS>
__global__ void __launch_bounds__(XLT_THREADS) xlt_kernel(const T* __restrict__ Ld, int ldl, T* __restrict__ X, int ldx,
                                                         int rows, int k) {
    extern __shared__ __align__(16) unsigned char xlt_raw[];
    T* const sl = reinterpret_cast<T*>(xlt_raw);  // [KB][KB]: L(i, j) at i + j * KB
    T* const sinv = sl + KB * KB;                 // [KB]
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        const int i = e % k, j = e / k;
        sl[i + j * KB] = Ld[i + (size_t)j * ldl];
    }
    __syncthreads();
    for (int j = threadIdx.x; j < k; j += blockDim.x) sinv[j] = T(1) / sl[j + j * KB];
    __syncthreads();
    const int r = blockIdx.x * XLT_THREADS + threadIdx.x;
    if (r >= rows) return;
    T x[KB];
#pragma unroll
    for (int j = 0; j < KB; ++j) x[j] = j < k ? X[r + (size_t)j * ldx] : T(0);
#pragma unroll 1
    for (int j = 0; j < k; ++j) {
        const T xj = x[0] * sinv[j];
        const T* lj = sl + j * KB + j;  // lj[d] = L(j + d, j)
        const int na = k - 1 - j;       // positions 1 .. na still to update
#pragma unroll
        for (int d = 1; d < KB; ++d) x[d - 1] = d <= na ? fma(xj, -lj[d], x[d]) : x[d];
        x[KB - 1] = xj;
    }
#pragma unroll 1
    for (int j = k; j < KB; ++j) {  // k < KB: finish the rotation
        const T x0 = x[0];
#pragma unroll
        for (int d = 1; d < KB; ++d) x[d - 1] = x[d];
        x[KB - 1] = x0;
    }
#pragma unroll
    for (int j = 0; j < KB; ++j)
        if (j < k) X[r + (size_t)j * ldx] = x[j];
}

template <typename T, int KB = LLT_BS>
mg_status_t launch_xlt(mg_handle_t h, cudaStream_t st, const T* Ld, int ldl, T* X, int ldx, int rows, int k) {
    constexpr size_t smem = xlt_smem_bytes<T, KB>();
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(xlt_kernel<T, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    xlt_kernel<T, KB><<<(rows + XLT_THREADS - 1) / XLT_THREADS, XLT_THREADS, smem, st>>>(Ld, ldl, X, ldx, rows, k);
    return mg::post_launch(h, "xlt_kernel");
}

// Unblocked LDL^T of the k x k block at L (k <= 96), in place, lower part
// (Mat's __LDLT2, LU/__LLT.h:16-27).  Column jj: d = L(jj,jj) (to d_out);
// L(r,jj) *= 1/d for r >= jj (the diagonal becomes d * (1/d)); then for
// i > jj: L(r,i) = fma(L(r,jj), (-L(i,jj)) d, L(r,i)) for r >= i.  info =
// first exactly zero d (1-based).
__global__ void ldlt2_kernel(double* __restrict__ L, int ldl, int k, int col0, double* __restrict__ d_out,
                             int* __restrict__ info) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    double* s = reinterpret_cast<double*>(s_raw);  // column-major k x k with stride LLT2_MAX
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        const int r = e % k, c = e / k;
        s[r + c * LLT2_MAX] = L[r + (size_t)c * ldl];
    }
    __syncthreads();
    const int r = threadIdx.x;
    for (int jj = 0; jj < k; ++jj) {
        const double d = s[jj + jj * LLT2_MAX];
        const double t = 1.0 / d;
        if (r == 0) {
            d_out[col0 + jj] = d;
            if (d == 0.0) atomicCAS(info, 0, col0 + jj + 1);
        }
        __syncthreads();  // every thread has read d before row jj is scaled
        if (r >= jj && r < k) s[r + jj * LLT2_MAX] = __dmul_rn(s[r + jj * LLT2_MAX], t);
        __syncthreads();
        if (r > jj && r < k) {
            const double lrj = s[r + jj * LLT2_MAX];
            for (int i = jj + 1; i <= r; ++i)
                s[r + i * LLT2_MAX] = fma(lrj, __dmul_rn(-s[i + jj * LLT2_MAX], d), s[r + i * LLT2_MAX]);
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        const int rr = e % k, c = e / k;
        if (rr >= c) L[rr + (size_t)c * ldl] = s[rr + c * LLT2_MAX];
    }
}

// The end of Mat's __Solve_direct_XDLT (LU/__LLT.h:53-55) and the packing
// of the trailing update's B operand (__pack_BT_block_d,
// Mul/__pack_double.h:241-282): P(r,p) *= 1/d_p, then W(r,p) = P(r,p) d_p.
__global__ void ldlt_scale_kernel(double* __restrict__ P, int ldp, int rows, int k, const double* __restrict__ d,
                                  double* __restrict__ W, int ldw) {
    const size_t total = (size_t)rows * k;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % rows), p = (int)(e / rows);
        const double x = __dmul_rn(P[r + (size_t)p * ldp], 1.0 / d[p]);
        P[r + (size_t)p * ldp] = x;
        W[r + (size_t)p * ldw] = __dmul_rn(x, d[p]);
    }
}

template <typename T>
__global__ void zero_upper_kernel(T* __restrict__ L, int ldl, int n) {
    const size_t total = (size_t)n * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % n), c = (int)(e / n);
        if (r < c) L[r + (size_t)c * ldl] = T(0);
    }
}

// Forward / back substitution with L (lower, non-unit) for the Cholesky solve,
// blocked by 64 rows like the LU narrow solve: per element a chain over k in
// ascending (L z = b) or descending (L^T x = z) order.
constexpr int CS_B = 64;

template <typename T>
__global__ void chol_fwd_diag_kernel(int n, int nrhs, const T* __restrict__ L, int ldl, T* __restrict__ X,
                                     int ldx, int b0, int b1) {
    const int bs = b1 - b0;
    for (int k = b0; k < b1; ++k) {
        for (int j = threadIdx.x; j < nrhs; j += blockDim.x) X[k + (size_t)j * ldx] /= L[k + (size_t)k * ldl];
        __syncthreads();
        for (int q = threadIdx.x; q < bs * nrhs; q += blockDim.x) {
            const int r = b0 + q % bs, j = q / bs;
            if (r > k) X[r + (size_t)j * ldx] = fma(L[r + (size_t)k * ldl], -X[k + (size_t)j * ldx], X[r + (size_t)j * ldx]);
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void chol_fwd_update_kernel(int n, int nrhs, const T* __restrict__ L, int ldl, T* __restrict__ X,
                                       int ldx, int b0, int b1) {
    __shared__ T xs[4][CS_B];
    const int bs = b1 - b0;
    for (int j0 = 0; j0 < nrhs; j0 += 4) {
        const int nj = min(4, nrhs - j0);
        __syncthreads();
        for (int q = threadIdx.x; q < bs * nj; q += blockDim.x) xs[q / bs][q % bs] = X[b0 + q % bs + (size_t)(j0 + q / bs) * ldx];
        __syncthreads();
        for (int r = b1 + blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
            T acc[4];
            for (int j = 0; j < nj; ++j) acc[j] = X[r + (size_t)(j0 + j) * ldx];
            for (int k = 0; k < bs; ++k) {
                const T l = L[r + (size_t)(b0 + k) * ldl];
                for (int j = 0; j < nj; ++j) acc[j] = fma(l, -xs[j][k], acc[j]);
            }
            for (int j = 0; j < nj; ++j) X[r + (size_t)(j0 + j) * ldx] = acc[j];
        }
    }
}

// L^T x = z: row i of L^T is column i of L.
template <typename T>
__global__ void chol_bwd_diag_kernel(int n, int nrhs, const T* __restrict__ L, int ldl, T* __restrict__ X,
                                     int ldx, int b0, int b1) {
    const int bs = b1 - b0;
    for (int k = b1 - 1; k >= b0; --k) {
        for (int j = threadIdx.x; j < nrhs; j += blockDim.x) X[k + (size_t)j * ldx] /= L[k + (size_t)k * ldl];
        __syncthreads();
        for (int q = threadIdx.x; q < bs * nrhs; q += blockDim.x) {
            const int i = b0 + q % bs, j = q / bs;
            if (i < k) X[i + (size_t)j * ldx] = fma(L[k + (size_t)i * ldl], -X[k + (size_t)j * ldx], X[i + (size_t)j * ldx]);
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void chol_bwd_update_kernel(int n, int nrhs, const T* __restrict__ L, int ldl, T* __restrict__ X,
                                       int ldx, int b0, int b1) {
    // rows i < b0: x_i -= sum_{k in block} L(k,i) x_k  (k descending); one warp per row i
    __shared__ T xs[4][CS_B];
    const int bs = b1 - b0;
    const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    for (int j0 = 0; j0 < nrhs; j0 += 4) {
        const int nj = min(4, nrhs - j0);
        __syncthreads();
        for (int q = threadIdx.x; q < bs * nj; q += blockDim.x) xs[q / bs][q % bs] = X[b0 + q % bs + (size_t)(j0 + q / bs) * ldx];
        __syncthreads();
        for (int i = blockIdx.x * warps + (threadIdx.x >> 5); i < b0; i += gridDim.x * warps) {
            if (lane < nj) {
                T acc = X[i + (size_t)(j0 + lane) * ldx];
                const T* lp = L + (size_t)i * ldl + b0;  // L(b0.., i): contiguous in column i
                for (int k = bs - 1; k >= 0; --k) acc = fma(lp[k], -xs[lane][k], acc);
                X[i + (size_t)(j0 + lane) * ldx] = acc;
            }
        }
    }
}

// The Cholesky factor L (lower, fp32) rewritten as the packed LU of the same
// matrix, L L^T = (L D^-1)(D L^T) with D = diag(L), so that the mixed
// solve's LU refinement applies to it unchanged: pass 1 writes U(r, c) =
// L(r, r) L(c, r) on and above the diagonal (reading the lower triangle),
// pass 2 the unit-lower part L(r, c) / L(c, c) below it.  d holds diag(L).
__global__ void chol_diag_kernel(const float* __restrict__ L, int ldl, int n, float* __restrict__ d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = L[i + (size_t)i * ldl];
}
__global__ void chol_to_lu_upper_kernel(float* __restrict__ A, int lda, int n, const float* __restrict__ d) {
    const size_t total = (size_t)n * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % n), c = (int)(e / n);
        if (r <= c) A[r + (size_t)c * lda] = d[r] * A[c + (size_t)r * lda];
    }
}
__global__ void chol_to_lu_lower_kernel(float* __restrict__ A, int lda, int n, const float* __restrict__ d) {
    const size_t total = (size_t)n * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % n), c = (int)(e / n);
        if (r > c) A[r + (size_t)c * lda] = A[r + (size_t)c * lda] / d[c];
    }
}

// FP32 Cholesky of a diagonal block of the mixed SPD factorization (k <= 64)
// together with G = L^{-T}, in one sweep with one CTA barrier per column.
// Right-looking Cholesky is a sequence of column operations on A (column c
// -= (a_cj / a_jj) column j for every c > j, then column j scaled by
// 1 / sqrt(a_jj)) that turns A into A L^{-T} = L; the same operations
// applied to an identity stacked below A turn it into L^{-T}.  The 128 x 64
// stack [A; I] sits in registers: warp w owns columns w, w+16, w+32, w+48,
// lane l rows l and l+32 of each half.  Per column j the warp that owns it
// publishes the column (both halves; A's rows above j as zeros) to shared
// memory, every thread applies the operation to the columns after j that it
// owns (a window over its four rotated once per 16 columns, so that register
// indices stay static in a rolled loop).  The scaling of each column by
// 1 / sqrt(a_jj) waits until the sweep is over (a column is the source of
// the operations of its own step only), which keeps the square root off
// the chain from one column to the next.  A block narrower than 64 (the
// last one) is padded with the identity.  info:
// first non-positive pivot (1-based, from col0).  With ntop > 0 the kernel
// also forms Xt = P G for the first ntop rows P of the block column below
// (ld ldd, rows ntop .. 63 of Xt zero), into xtop (64 x 64, ld 64), in the
// same per-element order as xlt_split64_kernel (fmaf over k from 0), so
// that Xt equals those rows of the block column's solve bit for bit.
constexpr int CI_NB = 64;
constexpr int CI_THREADS = 512;
constexpr int CI_GP = CI_NB + 4;  // pitch of G (row-major) in shared memory: 16-byte rows

__global__ void __launch_bounds__(CI_THREADS) chol_inv64_kernel(float* __restrict__ D, int ldd, int k, int col0,
                                                              float* __restrict__ G, int* __restrict__ info,
                                                              int ntop, float* __restrict__ xtop) {
    __shared__ float colv[2][2 * CI_NB];
    __shared__ float piv[CI_NB];                       // a_jj at step j
    __shared__ __align__(16) float gsm[CI_NB * CI_GP];  // G(k, c) at k * CI_GP + c
    __shared__ float psm[CI_NB * CI_NB];               // P(r, k) at r + 64 k
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (ntop > 0) {
#pragma unroll
        for (int u = 0; u < CI_NB * CI_NB / CI_THREADS; ++u) {
            const int e = threadIdx.x + CI_THREADS * u, r = e & 63, c = e >> 6;
            psm[e] = r < ntop ? D[CI_NB + r + (size_t)c * ldd] : 0.f;
        }
    }
    float a[4][4];  // [stacked row lane + 32 q: q < 2 in A, q >= 2 in I][window position]
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = lane + 32 * (q & 1);
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const int c = w + 16 * m;
            a[q][m] = i == c ? 1.f : 0.f;
            if (q < 2 && i < k && c < k && i >= c) a[q][m] = D[i + (size_t)c * ldd];
        }
    }
#pragma unroll 1
    for (int jm = 0; jm < 4; ++jm) {
        const int nlive = 3 - jm;  // window positions 1 .. nlive hold columns after this group of 16
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) {
            const int j = 16 * jm + jj;
            float* const cv = colv[jj & 1];
            if (w == jj) {
#pragma unroll
                for (int q = 0; q < 4; ++q) cv[lane + 32 * q] = (q < 2 && lane + 32 * q < j) ? 0.f : a[q][0];
            }
            __syncthreads();  // the column is published; the buffer of column j-1 stays readable
            const float d = cv[j];
            if (threadIdx.x == 0) {
                piv[j] = d;
                if (j < k && !(d > 0.f)) atomicCAS(info, 0, col0 + j + 1);
            }
            const float rd = __frcp_rn(d);
            float t[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) t[q] = -cv[lane + 32 * q] * rd;
            if (w > jj) {  // window position 0 is column w + 16 jm, after j
                const float ck = cv[w + 16 * jm];
#pragma unroll
                for (int q = 0; q < 4; ++q) a[q][0] = fmaf(t[q], ck, a[q][0]);
            }
#pragma unroll
            for (int m = 1; m < 4; ++m) {
                if (m <= nlive) {
                    const float ck = cv[w + 16 * (jm + m)];
#pragma unroll
                    for (int q = 0; q < 4; ++q) a[q][m] = fmaf(t[q], ck, a[q][m]);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {  // rotate the window: the next group's column first
            const float t0 = a[q][0];
            a[q][0] = a[q][1];
            a[q][1] = a[q][2];
            a[q][2] = a[q][3];
            a[q][3] = t0;
        }
    }
    __syncthreads();  // every pivot recorded
#pragma unroll
    for (int m = 0; m < 4; ++m) {  // the deferred scaling of column c by 1 / sqrt(a_cc)
        const int c = w + 16 * m;
        const float sd = sqrtf(piv[c]), rs = __frcp_rn(sd);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = lane + 32 * (q & 1);
            if (q >= 2 || i > c)
                a[q][m] *= rs;
            else if (i == c)
                a[q][m] = sd;
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int i = lane + 32 * (q & 1);
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const int c = w + 16 * m;
            if (q < 2) {
                if (i < k && c < k && i >= c) D[i + (size_t)c * ldd] = a[q][m];
            } else {
                const float g = i <= c ? a[q][m] : 0.f;
                G[i + CI_NB * c] = g;
                gsm[i * CI_GP + c] = g;
            }
        }
    }
    if (ntop <= 0) return;
    __syncthreads();
    // Xt = P G: thread r = t % 64 and the 8 columns 8 (t / 64) ..
    const int r = threadIdx.x & 63, c0 = (threadIdx.x >> 6) * 8;
    float acc[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) acc[u] = 0.f;
#pragma unroll 4
    for (int kk = 0; kk < CI_NB; ++kk) {
        const float x = psm[r + CI_NB * kk];
        const float4 g0 = *reinterpret_cast<const float4*>(gsm + kk * CI_GP + c0);
        const float4 g1 = *reinterpret_cast<const float4*>(gsm + kk * CI_GP + c0 + 4);
        const float g[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
#pragma unroll
        for (int u = 0; u < 8; ++u) acc[u] = fmaf(x, g[u], acc[u]);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) xtop[r + CI_NB * (c0 + u)] = acc[u];
}

}  // namespace

namespace mg {

template <typename T>
mg_status_t potrf_impl(mg_handle_t h, int n, T* L, int ldl, int* info_out) {
    if (info_out) *info_out = 0;
    if (n == 0) return MG_OK;
    MG_TRY(ensure_hws(h, 64));
    int* dinfo = h->status;
    MG_CHECK_CUDA(h, cudaMemsetAsync(dinfo, 0, sizeof(int), h->stream));
    cudaStream_t st = h->stream;
    const size_t s2 = (size_t)LLT2_MAX * LLT2_MAX * sizeof(T);
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(llt2_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2));
    if (n <= 2 * LLT_BS) {
        llt2_kernel<T><<<1, LLT2_THREADS, s2, st>>>(L, ldl, n, 0, dinfo);
        MG_TRY(post_launch(h, "llt2_kernel"));
    } else {
        // Look-ahead of one block column: after step j's panel solve, the next
        // block column is updated first (near update), its diagonal block and
        // panel solve run on the high-priority side stream, and the rest of
        // the trailing matrix (far update) on the low-priority one; step
        // j+48's near update waits for the far update.  Every lower element
        // still receives step j's fused chain over 48 columns in order.
        MG_TRY(ensure_lookahead(h));
        auto diag_and_panel = [&](int j) -> mg_status_t {
            const int nb = n - j < LLT_BS ? n - j : LLT_BS;
            T* D = L + j + (size_t)j * ldl;
            llt2_kernel<T><<<1, LLT2_THREADS, s2, h->stream>>>(D, ldl, nb, j, dinfo);
            MG_TRY(post_launch(h, "llt2_kernel"));
            if (j + LLT_BS < n) {
                const int rows = n - (j + LLT_BS);
                MG_TRY(launch_xlt<T>(h, h->stream, D, ldl, L + (j + LLT_BS) + (size_t)j * ldl, ldl, rows, LLT_BS));
            }
            return MG_OK;
        };
        bool far_pending = false, have = false;
        for (int j = 0; j < n; j += LLT_BS) {
            if (!have) MG_TRY(diag_and_panel(j));
            have = false;
            if (j + LLT_BS >= n) break;
            const int rows = n - (j + LLT_BS);
            T* P = L + (j + LLT_BS) + (size_t)j * ldl;
            T* C = L + (j + LLT_BS) + (size_t)(j + LLT_BS) * ldl;
            if (far_pending) MG_CHECK_CUDA(h, cudaStreamWaitEvent(st, h->la_ev[1], 0));
            far_pending = false;
            const int nb1 = rows < LLT_BS ? rows : LLT_BS;  // the next block column
            if (rows > nb1) {
                MG_TRY(gemm_of(h, 0, 1, rows, nb1, LLT_BS, T(-1), P, ldl, P, ldl, T(1), C, ldl, 1));
                MG_CHECK_CUDA(h, cudaEventRecord(h->la_ev[0], st));
                MG_CHECK_CUDA(h, cudaStreamWaitEvent(h->pp_stream, h->la_ev[0], 0));
                {
                    OnStream on(h, h->pp_stream);
                    MG_TRY(diag_and_panel(j + LLT_BS));
                    MG_CHECK_CUDA(h, cudaEventRecord(h->pp_ev[0], h->pp_stream));
                }
                MG_CHECK_CUDA(h, cudaStreamWaitEvent(st, h->pp_ev[0], 0));
                have = true;
                MG_CHECK_CUDA(h, cudaStreamWaitEvent(h->la_stream, h->la_ev[0], 0));
                {
                    OnStream on(h, h->la_stream);
                    MG_TRY(gemm_of(h, 0, 1, rows - nb1, rows - nb1, LLT_BS, T(-1), P + nb1, ldl, P + nb1, ldl, T(1),
                                   C + nb1 + (size_t)nb1 * ldl, ldl, 1));
                    MG_CHECK_CUDA(h, cudaEventRecord(h->la_ev[1], h->la_stream));
                }
                far_pending = true;
            } else {
                // C(i.., i..) -= P P^T on the trailing matrix, lower tiles only
                MG_TRY(gemm_of(h, 0, 1, rows, rows, LLT_BS, T(-1), P, ldl, P, ldl, T(1), C, ldl, 1));
            }
        }
        if (far_pending) MG_CHECK_CUDA(h, cudaStreamWaitEvent(st, h->la_ev[1], 0));
    }
    zero_upper_kernel<T><<<h->num_sms * 8, 256, 0, st>>>(L, ldl, n);
    MG_TRY(post_launch(h, "zero_upper_kernel"));
    int* hw = (int*)h->hws;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
    if (sizeof(T) == 4) {  // the FP32 trailing updates may have run on the tensor cores
        int terr = 0;
        MG_TRY(tc_sgemm_error(h, &terr));
        if (terr) return fail(h, MG_TIMEOUT, "potrf: a tensor-core update's bounded wait gave up");
    }
    if (info_out) *info_out = hw[0];
    if (hw[0]) return fail(h, MG_NOT_SPD, "potrf: non-positive pivot at column %d", hw[0]);
    return MG_OK;
}
template mg_status_t potrf_impl<double>(mg_handle_t, int, double*, int, int*);
template mg_status_t potrf_impl<float>(mg_handle_t, int, float*, int, int*);

mg_status_t dpotrf_impl(mg_handle_t h, int n, double* L, int ldl, int* info_out) {
    return potrf_impl<double>(h, n, L, ldl, info_out);
}

// FP32 Cholesky for the mixed SPD solve (no counterpart in Mat, whose LLT,
// LU/__LLT.h:94-150, is FP64): right-looking, blocks of 64 columns.  Per
// block: the diagonal block's Cholesky and its inverse transpose G = L^{-T}
// in one CTA, with the product of G and the first 64 rows of the block
// column below (chol_inv64_kernel); then one kernel for the block column X
// := X G, the split of X into `nterms` BF16 terms and, in FP32, the update
// of the next block column by X and those first rows (xlt_split64_kernel);
// then the rest of the trailing update, C -= X X^T on the tensor cores from
// the one split, which serves as both operands (the B operand's rows are
// X's rows; fp32 accumulation, lower-order products first), restricted to
// the tiles that meet the lower triangle, on the side stream with one SM
// left free, where the next diagonal block's kernel runs beside it.  The
// next block column's kernel waits for it (it holds the other SMs and reads
// the split that kernel rewrites).  `split` holds bf16x_split_bytes(n, 64,
// nterms), `gblk` 2 x 64 x 64 floats.  info: first non-positive pivot (the
// fp32 factorization of an SPD matrix can break down near singularity).
mg_status_t spotrf_mixed(mg_handle_t h, int n, float* L, int ldl, int nterms, void* split, float* gblk,
                         int* gemm_err, int* info_out) {
    constexpr int NB = CI_NB;
    if (info_out) *info_out = 0;
    if (n == 0) return MG_OK;
    MG_TRY(ensure_hws(h, 64));
    MG_TRY(ensure_lookahead(h));
    int* dinfo = h->status;
    cudaStream_t st = h->stream;
    MG_CHECK_CUDA(h, cudaMemsetAsync(dinfo, 0, sizeof(int), st));
    float* const xtop = gblk + NB * NB;
    bool far_pending = false;
    for (int j = 0; j < n; j += NB) {
        const int nb = n - j < NB ? n - j : NB;
        const int rows = n - (j + nb);
        const int ntop = rows < NB ? rows : NB;  // the next block column
        float* D = L + j + (size_t)j * ldl;
        {
            ProfScope prof(h, "potrf_diag_f32", (double)nb * nb * nb + 2.0 * ntop * nb * nb, 8.0 * nb * nb);
            chol_inv64_kernel<<<1, CI_THREADS, 0, st>>>(D, ldl, nb, j, gblk, dinfo, ntop, xtop);
            MG_TRY(post_launch(h, "chol_inv64_kernel"));
        }
        if (rows == 0) break;
        float* P = L + (j + nb) + (size_t)j * ldl;
        float* C = L + (j + nb) + (size_t)(j + nb) * ldl;
        if (far_pending) MG_CHECK_CUDA(h, cudaStreamWaitEvent(st, h->la_ev[1], 0));
        far_pending = false;
        {
            ProfScope prof(h, "trsm_split_f32", 2.0 * rows * nb * (nb + ntop),
                           16.0 * rows * nb + 2.0 * nterms * rows * nb);
            MG_TRY(bf16x_xlt_split64(h, gblk, P, ldl, rows, nterms, split, xtop, ntop, C));
        }
        if (rows > ntop) {
            MG_CHECK_CUDA(h, cudaEventRecord(h->la_ev[0], st));
            MG_CHECK_CUDA(h, cudaStreamWaitEvent(h->la_stream, h->la_ev[0], 0));
            {
                OnStream on(h, h->la_stream);
                const size_t term = (size_t)rows * NB;  // elements per split term
                const uint16_t* xs = (const uint16_t*)split + (size_t)ntop * NB;  // rows ntop .. of the split
                MG_TRY(bf16x_gemm_presplit(h, nterms, rows - ntop, rows - ntop, nb, -1.0f, xs, xs, 1.0f,
                                           C + ntop + (size_t)ntop * ldl, ldl, gemm_err, term, term, h->num_sms - 1,
                                           true, true, true, true));
                MG_CHECK_CUDA(h, cudaEventRecord(h->la_ev[1], h->la_stream));
            }
            far_pending = true;
        }
    }
    if (far_pending) MG_CHECK_CUDA(h, cudaStreamWaitEvent(st, h->la_ev[1], 0));
    int* hw = (int*)h->hws;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
    if (info_out) *info_out = hw[0];
    if (hw[0]) return fail(h, MG_NOT_SPD, "spotrf_mixed: non-positive pivot at column %d", hw[0]);
    return MG_OK;
}

mg_status_t chol_to_lu_f32(mg_handle_t h, int n, float* A, int lda, float* dscratch) {
    const int grid = h->num_sms * 8;
    chol_diag_kernel<<<(n + 255) / 256, 256, 0, h->stream>>>(A, lda, n, dscratch);
    MG_TRY(post_launch(h, "chol_diag_kernel"));
    chol_to_lu_upper_kernel<<<grid, 256, 0, h->stream>>>(A, lda, n, dscratch);
    MG_TRY(post_launch(h, "chol_to_lu_upper_kernel"));
    chol_to_lu_lower_kernel<<<grid, 256, 0, h->stream>>>(A, lda, n, dscratch);
    return post_launch(h, "chol_to_lu_lower_kernel");
}

// In-place Mat LDLT on the lower triangle of L (ld ldl): unit-like lower
// factor (diagonal d_j * (1/d_j), as Mat leaves it), strict upper part
// zeroed, d (device, n) the diagonal of D.
mg_status_t dldlt_impl(mg_handle_t h, int n, double* L, int ldl, double* d, int* info_out) {
    if (info_out) *info_out = 0;
    if (n == 0) return MG_OK;
    MG_TRY(ensure_hws(h, 64));
    if (n > 2 * LLT_BS) MG_TRY(ensure_ws(h, (size_t)(n - LLT_BS) * LLT_BS * sizeof(double)));
    int* dinfo = h->status;
    MG_CHECK_CUDA(h, cudaMemsetAsync(dinfo, 0, sizeof(int), h->stream));
    cudaStream_t st = h->stream;
    const size_t s2 = (size_t)LLT2_MAX * LLT2_MAX * sizeof(double);
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(ldlt2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2));
    if (n <= 2 * LLT_BS) {
        ldlt2_kernel<<<1, 128, s2, st>>>(L, ldl, n, 0, d, dinfo);
        MG_TRY(post_launch(h, "ldlt2_kernel"));
    } else {
        double* W = (double*)h->ws;
        for (int j = 0; j < n; j += LLT_BS) {
            const int nb = n - j < LLT_BS ? n - j : LLT_BS;
            double* D = L + j + (size_t)j * ldl;
            ldlt2_kernel<<<1, 128, s2, st>>>(D, ldl, nb, j, d, dinfo);
            MG_TRY(post_launch(h, "ldlt2_kernel"));
            if (j + LLT_BS < n) {
                const int rows = n - (j + LLT_BS);
                double* P = L + (j + LLT_BS) + (size_t)j * ldl;
                MG_TRY(launch_xlt<double>(h, st, D, ldl, P, ldl, rows, LLT_BS));
                int blocks = (int)(((size_t)rows * LLT_BS + 255) / 256);
                if (blocks > h->num_sms * 8) blocks = h->num_sms * 8;
                ldlt_scale_kernel<<<blocks, 256, 0, st>>>(P, ldl, rows, LLT_BS, d + j, W, rows);
                MG_TRY(post_launch(h, "ldlt_scale_kernel"));
                // C(i.., i..) -= P (P D)^T on the trailing matrix, lower tiles only
                MG_TRY(dgemm_launch(h, 0, 1, rows, rows, LLT_BS, -1.0, P, ldl, W, rows, 1.0,
                                    L + (j + LLT_BS) + (size_t)(j + LLT_BS) * ldl, ldl, 1));
            }
        }
    }
    zero_upper_kernel<double><<<h->num_sms * 8, 256, 0, st>>>(L, ldl, n);
    MG_TRY(post_launch(h, "zero_upper_kernel"));
    int* hw = (int*)h->hws;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
    if (info_out) *info_out = hw[0];
    if (hw[0]) return fail(h, MG_SINGULAR, "ldlt: zero pivot at column %d", hw[0]);
    return MG_OK;
}

// L x = b (forward substitution), in place on X.
template <typename T>
mg_status_t chol_lower_solve(mg_handle_t h, int n, int nrhs, const T* L, int ldl, T* X, int ldx) {
    if (n == 0 || nrhs == 0) return MG_OK;
    cudaStream_t st = h->stream;
    for (int b0 = 0; b0 < n; b0 += CS_B) {
        const int b1 = b0 + CS_B < n ? b0 + CS_B : n;
        chol_fwd_diag_kernel<T><<<1, 256, 0, st>>>(n, nrhs, L, ldl, X, ldx, b0, b1);
        MG_TRY(post_launch(h, "chol_fwd_diag_kernel"));
        if (b1 < n) {
            int blocks = (n - b1 + 127) / 128;
            if (blocks > h->num_sms) blocks = h->num_sms;
            chol_fwd_update_kernel<T><<<blocks, 128, 0, st>>>(n, nrhs, L, ldl, X, ldx, b0, b1);
            MG_TRY(post_launch(h, "chol_fwd_update_kernel"));
        }
    }
    return MG_OK;
}
template mg_status_t chol_lower_solve<double>(mg_handle_t, int, int, const double*, int, double*, int);
template mg_status_t chol_lower_solve<float>(mg_handle_t, int, int, const float*, int, float*, int);

// L^T x = b (back substitution), in place on X.
template <typename T>
mg_status_t chol_lower_t_solve(mg_handle_t h, int n, int nrhs, const T* L, int ldl, T* X, int ldx) {
    if (n == 0 || nrhs == 0) return MG_OK;
    cudaStream_t st = h->stream;
    const int last = ((n - 1) / CS_B) * CS_B;
    for (int b0 = last; b0 >= 0; b0 -= CS_B) {
        const int b1 = b0 + CS_B < n ? b0 + CS_B : n;
        chol_bwd_diag_kernel<T><<<1, 256, 0, st>>>(n, nrhs, L, ldl, X, ldx, b0, b1);
        MG_TRY(post_launch(h, "chol_bwd_diag_kernel"));
        if (b0 > 0) {
            int blocks = (b0 + 7) / 8;
            if (blocks > h->num_sms * 4) blocks = h->num_sms * 4;
            chol_bwd_update_kernel<T><<<blocks, 256, 0, st>>>(n, nrhs, L, ldl, X, ldx, b0, b1);
            MG_TRY(post_launch(h, "chol_bwd_update_kernel"));
        }
    }
    return MG_OK;
}
template mg_status_t chol_lower_t_solve<double>(mg_handle_t, int, int, const double*, int, double*, int);
template mg_status_t chol_lower_t_solve<float>(mg_handle_t, int, int, const float*, int, float*, int);

mg_status_t dpotrs_impl(mg_handle_t h, int n, int nrhs, const double* L, int ldl, double* X, int ldx) {
    MG_TRY(chol_lower_solve<double>(h, n, nrhs, L, ldl, X, ldx));
    return chol_lower_t_solve<double>(h, n, nrhs, L, ldl, X, ldx);
}

}  // namespace mg

extern "C" {

mg_status_t mg_dpotrf(mg_handle_t h, int n, double* A, int lda, int* info) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || lda < (n > 1 ? n : 1) || (n && !A)) return mg::fail(h, MG_ERR_ARG, "mg_dpotrf: bad arguments");
    return mg::dpotrf_impl(h, n, A, lda, info);
}

mg_status_t mg_dpotrs(mg_handle_t h, int n, int nrhs, const double* L, int ldl, double* B, int ldb) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || nrhs < 0 || ldl < (n > 1 ? n : 1) || ldb < (n > 1 ? n : 1) || ((size_t)n * nrhs && (!L || !B)))
        return mg::fail(h, MG_ERR_ARG, "mg_dpotrs: bad arguments");
    return mg::dpotrs_impl(h, n, nrhs, L, ldl, B, ldb);
}

mg_status_t mg_dldlt(mg_handle_t h, int n, double* A, int lda, double* d, int* info) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || lda < (n > 1 ? n : 1) || (n && (!A || !d))) return mg::fail(h, MG_ERR_ARG, "mg_dldlt: bad arguments");
    return mg::dldlt_impl(h, n, A, lda, d, info);
}

mg_status_t mg_spotrf(mg_handle_t h, int n, float* A, int lda, int* info) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || lda < (n > 1 ? n : 1) || (n && !A)) return mg::fail(h, MG_ERR_ARG, "mg_spotrf: bad arguments");
    return mg::potrf_impl<float>(h, n, A, lda, info);
}

}  // extern "C"
