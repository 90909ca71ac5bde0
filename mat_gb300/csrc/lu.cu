// Blocked right-looking LU with partial pivoting (Mat's PLU) and the narrow
// Solve_direct on top of it.
//
// Reference path (Mat-8.3.1): PLU (LU/__PLU.h:152-190) -> __PLU (:93-149):
// per BS=60 block column, the panel __PLU2_piv (:54-90: left-looking column
// updates, __MaxAbs + first-index tie-break, row swaps, reciprocal scaling),
// __laswp_trailing (:3-19), the unit-lower TRSM __Solve_direct_LX
// (LU/__Base.h:95-208) on the block row, and the packed trailing update
// A22 -= L21*U12 (__mulAB_packed_n, Mul/Mul.h:240-263).
//
// GPU design:
//  - panel: one cooperative kernel, each CTA holding a slab of the panel's
//    rows in shared memory; per column one bounded grid barrier: every CTA
//    publishes (max |a|, first row, that row) and the row at the diagonal,
//    then all CTAs pick the same winner (largest |a|, smallest row on ties),
//    swap, scale by the reciprocal and apply the rank-1 update to their rows.
//    Right-looking within the panel performs exactly the fused operations of
//    Mat's left-looking loop in the same order, so the panel is bit-exact.
//  - laswp: the panel's interchanges on the columns left and right of it.
//  - trsm: one thread per right-hand column, reproducing Mat's AVX-512
//    operation order (four partial sums per row for 8-column groups,
//    column-oriented fused updates for the ragged columns).
//  - trailing update: the FP64 GEMM in its in-place "C -= A*B" mode.
//  Block size 60 = Mat's AVX-512 __BlockSize_LU, so the blocking (and with it
//  every rounding) follows the reference.
#include <climits>
#include <vector>

#include "grid_sync.cuh"
#include "mg_internal.cuh"

namespace {

constexpr int LU_BS = 60;           // Mat-8.3.1/Mat.h:69-71 (AVX-512)
constexpr int PANEL_MAX_NB = 256;   // FP64 unblocked path: s <= 1.5*BS = 90; mixed LU: 128
constexpr int PANEL_THREADS = 256;

struct PanelWs {
    unsigned* bar;  // grid barrier counter
    int* err;       // MG_TIMEOUT flag
    int* info;      // first zero-pivot column (1-based), 0 if none
};

// Exchange area layout (bytes), per panel launch.
template <typename T>
struct PanelXchg {
    T* cand_val;   // [2][P]
    int* cand_row; // [2][P]
    T* cand_rows;  // [2][P][nb]
    T* diag_row;   // [2][nb]
};

template <typename T>
__device__ __forceinline__ T ld_cg(const T* p) {
    return __ldcg(p);
}

template <typename T>
__device__ __forceinline__ void better(T& v, int& i, T ov, int oi) {
    if (ov > v || (ov == v && oi < i)) {
        v = ov;
        i = oi;
    }
}

// Panel factorization of columns [r0, r0+nb) over rows [r0, m).
template <typename T>
__global__ void __launch_bounds__(PANEL_THREADS, 1)
    panel_kernel(T* __restrict__ A, int lda, int m, int r0, int nb, int rpc, int nopiv, int* __restrict__ pos,
                 int* __restrict__ piv, PanelWs ws, PanelXchg<T> x) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* slab = reinterpret_cast<T*>(smem_raw);  // slab[c * rpc + i]
    __shared__ T prow[PANEL_MAX_NB];
    __shared__ T red_v[PANEL_THREADS / 32];
    __shared__ int red_i[PANEL_THREADS / 32];
    __shared__ int s_win, s_wcta, s_best_row;
    __shared__ T s_piv;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int b = blockIdx.x, P = gridDim.x;
    const int R = m - r0;
    const int row_lo = b * rpc;
    const int row_hi = min(R, row_lo + rpc);
    const int nrows = max(0, row_hi - row_lo);

    for (int e = tid; e < nrows * nb; e += blockDim.x) {
        const int c = e / nrows, i = e - c * nrows;
        slab[c * rpc + i] = A[(size_t)(r0 + row_lo + i) + (size_t)(r0 + c) * lda];
    }
    __syncthreads();

    for (int c = 0; c < nb; ++c) {
        const int buf = c & 1;
        // 1. local candidate: largest |a| in column c over rows >= c, smallest
        //    row on ties (nopiv: the diagonal row only, Mat's LU)
        T best = T(-1);
        int brow = INT_MAX;
        for (int i = tid; i < nrows; i += blockDim.x) {
            const int lr = row_lo + i;
            if (lr < c || (nopiv && lr != c)) continue;
            better(best, brow, fabs(slab[c * rpc + i]), lr);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const T ov = __shfl_down_sync(0xffffffffu, best, off);
            const int oi = __shfl_down_sync(0xffffffffu, brow, off);
            better(best, brow, ov, oi);
        }
        if (lane == 0) {
            red_v[warp] = best;
            red_i[warp] = brow;
        }
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < PANEL_THREADS / 32; ++w) better(best, brow, red_v[w], red_i[w]);
            s_best_row = brow;
            __stcg(x.cand_val + buf * P + b, best);
            __stcg(x.cand_row + buf * P + b, brow);
        }
        __syncthreads();
        // 2. publish the candidate row and (by its owner) the diagonal row
        {
            const int br = s_best_row;
            if (br != INT_MAX)
                for (int j = tid; j < nb; j += blockDim.x)
                    __stcg(x.cand_rows + ((size_t)buf * P + b) * nb + j, slab[j * rpc + (br - row_lo)]);
            if (c >= row_lo && c < row_hi)
                for (int j = tid; j < nb; j += blockDim.x)
                    __stcg(x.diag_row + buf * nb + j, slab[j * rpc + (c - row_lo)]);
        }
        if (!mg::grid_barrier(ws.bar, (unsigned)(c + 1) * P, ws.err)) return;
        // 3. the winner, identically in every CTA
        if (warp == 0) {
            T v = T(-1);
            int r = INT_MAX, wc = -1;
            for (int q = lane; q < P; q += 32) {
                const T ov = ld_cg(x.cand_val + buf * P + q);
                const int orow = ld_cg(x.cand_row + buf * P + q);
                if (ov > v || (ov == v && orow < r)) {
                    v = ov;
                    r = orow;
                    wc = q;
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const T ov = __shfl_down_sync(0xffffffffu, v, off);
                const int orow = __shfl_down_sync(0xffffffffu, r, off);
                const int owc = __shfl_down_sync(0xffffffffu, wc, off);
                if (ov > v || (ov == v && orow < r)) {
                    v = ov;
                    r = orow;
                    wc = owc;
                }
            }
            if (lane == 0) {
                s_win = r;
                s_wcta = wc;
                s_piv = v;
            }
        }
        __syncthreads();
        const int win = s_win;
        if (!(s_piv > T(0))) {
            // exactly zero column: no interchange, no scaling (LAPACK semantics)
            if (b == 0 && tid == 0) {
                piv[c] = c;
                atomicCAS(ws.info, 0, r0 + c + 1);
            }
            continue;
        }
        for (int j = tid; j < nb; j += blockDim.x) prow[j] = ld_cg(x.cand_rows + ((size_t)buf * P + s_wcta) * nb + j);
        __syncthreads();
        // 4. interchange rows c and win
        if (win != c) {
            if (c >= row_lo && c < row_hi)
                for (int j = tid; j < nb; j += blockDim.x) slab[j * rpc + (c - row_lo)] = prow[j];
            if (win >= row_lo && win < row_hi)
                for (int j = tid; j < nb; j += blockDim.x)
                    slab[j * rpc + (win - row_lo)] = ld_cg(x.diag_row + buf * nb + j);
        }
        if (b == 0 && tid == 0) {
            piv[c] = win;
            if (win != c) {
                const int t = pos[r0 + c];
                pos[r0 + c] = pos[r0 + win];
                pos[r0 + win] = t;
            }
        }
        __syncthreads();
        // 5. scale by the reciprocal and update the rows below (fused, Mat's order)
        const T inv = T(1) / prow[c];
        for (int i = tid; i < nrows; i += blockDim.x) {
            const int lr = row_lo + i;
            if (lr <= c) continue;
            const T l = slab[c * rpc + i] * inv;
            slab[c * rpc + i] = l;
            for (int j = c + 1; j < nb; ++j) slab[j * rpc + i] = fma(l, -prow[j], slab[j * rpc + i]);
        }
        __syncthreads();
    }

    for (int e = tid; e < nrows * nb; e += blockDim.x) {
        const int c = e / nrows, i = e - c * nrows;
        A[(size_t)(r0 + row_lo + i) + (size_t)(r0 + c) * lda] = slab[c * rpc + i];
    }
}

// Interchanges rows r0+k <-> r0+piv[k] (k = 0..kc-1, in order) on columns
// [0, c_left) and [c_right, n).
template <typename T>
__global__ void laswp_kernel(T* __restrict__ A, int lda, int r0, int kc, const int* __restrict__ piv, int c_left,
                             int c_right, int n) {
    __shared__ int sp[PANEL_MAX_NB];
    for (int k = threadIdx.x; k < kc; k += blockDim.x) sp[k] = piv[k];
    __syncthreads();
    const int nl = c_left, nr = max(0, n - c_right);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nl + nr; q += gridDim.x * blockDim.x) {
        const int col = q < nl ? q : c_right + (q - nl);
        T* cp = A + (size_t)col * lda + r0;
        for (int k = 0; k < kc; ++k) {
            const int j = sp[k];
            if (j != k) {
                const T t = cp[k];
                cp[k] = cp[j];
                cp[j] = t;
            }
        }
    }
}

// X (k x n) := L^{-1} X with L unit lower (k <= PANEL_MAX_NB), one thread per
// column, Mat's AVX-512 operation order (LU/__Base.h:95-208): columns of full
// 8-groups use four partial sums s0..s3 over j = 0,4,8.. / 1,5,.. etc. and
// x_i = s0 + (s1 + (s2 + s3)); the remaining n % 8 columns use fused
// column updates x[i..] += L[i..][i-1] * (-x[i-1]), skipped when x[i-1] == 0.
template <typename T>
__global__ void trsm_llnu_kernel(int k, int n, const T* __restrict__ L, int ldl, T* __restrict__ X, int ldx) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sL = reinterpret_cast<T*>(smem_raw);       // [k][k] column-major
    T* sx = sL + k * k;                           // [k][blockDim]
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) sL[e] = L[(e % k) + (size_t)(e / k) * ldl];
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = blockDim.x, t = threadIdx.x;
    if (col < n)
        for (int i = 0; i < k; ++i) sx[i * nt + t] = X[i + (size_t)col * ldx];
    __syncthreads();
    if (col >= n) return;
    const int n8 = (n / 8) * 8;
    if (col < n8) {
        for (int i = 0; i < k; ++i) {
            T s0 = sx[i * nt + t], s1 = 0, s2 = 0, s3 = 0;
            int j = 0;
            for (; j + 4 <= i; j += 4) {
                s0 = fma(-sL[i + (j + 0) * k], sx[(j + 0) * nt + t], s0);
                s1 = fma(-sL[i + (j + 1) * k], sx[(j + 1) * nt + t], s1);
                s2 = fma(-sL[i + (j + 2) * k], sx[(j + 2) * nt + t], s2);
                s3 = fma(-sL[i + (j + 3) * k], sx[(j + 3) * nt + t], s3);
            }
            for (; j < i; ++j) s0 = fma(-sL[i + j * k], sx[j * nt + t], s0);
            sx[i * nt + t] = s0 + (s1 + (s2 + s3));
        }
    } else {
        for (int i = 1; i < k; ++i) {
            const T a = sx[(i - 1) * nt + t];
            if (a == T(0)) continue;
            for (int r = i; r < k; ++r) sx[r * nt + t] = fma(sL[r + (i - 1) * k], -a, sx[r * nt + t]);
        }
    }
    for (int i = 0; i < k; ++i) X[i + (size_t)col * ldx] = sx[i * nt + t];
}

// X (k x n) := U^{-1} X with U upper (k <= PANEL_MAX_NB), one thread per
// column, Mat's order for every column (LU/__Base.h:209-293 and :51-92 give
// the same arithmetic): for i = k-1..0, x_i /= U(i,i), then
// x_j = fma(U(j,i), -x_i, x_j) for j < i.
template <typename T>
__global__ void trsm_lunn_kernel(int k, int n, const T* __restrict__ U, int ldu, T* __restrict__ X, int ldx) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sU = reinterpret_cast<T*>(smem_raw);       // [k][k] column-major
    T* sx = sU + k * k;                           // [k][blockDim]
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) sU[e] = U[(e % k) + (size_t)(e / k) * ldu];
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = blockDim.x, t = threadIdx.x;
    if (col < n)
        for (int i = 0; i < k; ++i) sx[i * nt + t] = X[i + (size_t)col * ldx];
    __syncthreads();
    if (col >= n) return;
    for (int i = k - 1; i >= 0; --i) {
        const T xi = sx[i * nt + t] / sU[i + i * k];
        sx[i * nt + t] = xi;
        for (int j = 0; j < i; ++j) sx[j * nt + t] = fma(sU[j + i * k], -xi, sx[j * nt + t]);
    }
    for (int i = 0; i < k; ++i) X[i + (size_t)col * ldx] = sx[i * nt + t];
}

__global__ void iota_kernel(int* p, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}

// ------------------------------------------------------------ narrow solve
// Forward substitution with unit L, Mat's narrow order (LU/__Solve_direct.h:125-130):
// x[r] receives fma(L(r,k), -x[k], x[r]) for k = 0..r-1 ascending.  Blocked by
// 64 columns: the diagonal block by one CTA, the rows below in parallel.
constexpr int TRSV_B = 64;

template <typename TM, typename T>
__global__ void trsv_lower_diag_kernel(int n, int nrhs, const TM* __restrict__ L, int ldl, T* __restrict__ X,
                                       int ldx, int b0, int b1) {
    // one CTA; threads over rows of the block x rhs
    const int bs = b1 - b0;
    for (int k = b0; k < b1; ++k) {
        for (int q = threadIdx.x; q < bs * nrhs; q += blockDim.x) {
            const int r = b0 + q % bs, j = q / bs;
            if (r > k) {
                T* x = X + (size_t)j * ldx;
                x[r] = fma((T)L[r + (size_t)k * ldl], -x[k], x[r]);
            }
        }
        __syncthreads();
    }
}

template <typename TM, typename T>
__global__ void trsv_lower_update_kernel(int n, int nrhs, const TM* __restrict__ L, int ldl, T* __restrict__ X,
                                         int ldx, int b0, int b1) {
    __shared__ T xs[4][TRSV_B];
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
                const T l = (T)L[r + (size_t)(b0 + k) * ldl];
                for (int j = 0; j < nj; ++j) acc[j] = fma(l, -xs[j][k], acc[j]);
            }
            for (int j = 0; j < nj; ++j) X[r + (size_t)(j0 + j) * ldx] = acc[j];
        }
    }
}

// Back substitution, Mat's narrow order (:132-139): for r = n-1..0:
// x[r] /= U(r,r); x[i] = fma(U(i,r), -x[r], x[i]) for i < r.
template <typename TM, typename T>
__global__ void trsv_upper_diag_kernel(int n, int nrhs, const TM* __restrict__ U, int ldu, T* __restrict__ X,
                                       int ldx, int b0, int b1) {
    const int bs = b1 - b0;
    for (int r = b1 - 1; r >= b0; --r) {
        for (int j = threadIdx.x; j < nrhs; j += blockDim.x) X[r + (size_t)j * ldx] /= (T)U[r + (size_t)r * ldu];
        __syncthreads();
        for (int q = threadIdx.x; q < bs * nrhs; q += blockDim.x) {
            const int i = b0 + q % bs, j = q / bs;
            if (i < r) {
                T* x = X + (size_t)j * ldx;
                x[i] = fma((T)U[i + (size_t)r * ldu], -x[r], x[i]);
            }
        }
        __syncthreads();
    }
}

template <typename TM, typename T>
__global__ void trsv_upper_update_kernel(int n, int nrhs, const TM* __restrict__ U, int ldu, T* __restrict__ X,
                                         int ldx, int b0, int b1) {
    __shared__ T xs[4][TRSV_B];
    const int bs = b1 - b0;
    for (int j0 = 0; j0 < nrhs; j0 += 4) {
        const int nj = min(4, nrhs - j0);
        __syncthreads();
        for (int q = threadIdx.x; q < bs * nj; q += blockDim.x) xs[q / bs][q % bs] = X[b0 + q % bs + (size_t)(j0 + q / bs) * ldx];
        __syncthreads();
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < b0; i += gridDim.x * blockDim.x) {
            T acc[4];
            for (int j = 0; j < nj; ++j) acc[j] = X[i + (size_t)(j0 + j) * ldx];
            for (int k = bs - 1; k >= 0; --k) {
                const T u = (T)U[i + (size_t)(b0 + k) * ldu];
                for (int j = 0; j < nj; ++j) acc[j] = fma(u, -xs[j][k], acc[j]);
            }
            for (int j = 0; j < nj; ++j) X[i + (size_t)(j0 + j) * ldx] = acc[j];
        }
    }
}

// X[i, j] = B[pos[i], j]
template <typename T>
__global__ void permute_rows_kernel(int n, int nrhs, const int* __restrict__ pos, const T* __restrict__ B, int ldb,
                                    T* __restrict__ X, int ldx) {
    const size_t total = (size_t)n * nrhs;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        X[i + (size_t)j * ldx] = B[pos[i] + (size_t)j * ldb];
    }
}

}  // namespace

namespace mg {

// Workspace carve-up for one getrf call (device): barrier/err/info words,
// piv[PANEL_MAX_NB], exchange buffers sized for num_sms CTAs.
template <typename T>
static constexpr size_t getrf_ws_bytes(int num_sms, int nbmax = PANEL_MAX_NB) {
    return 256 + 4 * (size_t)nbmax + 2 * (size_t)num_sms * sizeof(T) + 2 * (size_t)num_sms * sizeof(int) +
           2 * (size_t)num_sms * nbmax * sizeof(T) + 2 * (size_t)nbmax * sizeof(T) + 1024;
}

template <typename T>
struct GetrfCtx {
    PanelWs ws;
    PanelXchg<T> x;
    int* piv;
};

template <typename T>
static GetrfCtx<T> carve(void* base, int num_sms, int nbmax = PANEL_MAX_NB) {
    char* p = (char*)base;
    GetrfCtx<T> c;
    c.ws.bar = (unsigned*)p;
    c.ws.err = (int*)(p + 64);
    c.ws.info = (int*)(p + 128);
    p += 256;
    c.piv = (int*)p;
    p += align_up(4 * (size_t)nbmax, 256);
    c.x.cand_val = (T*)p;
    p += align_up(2 * (size_t)num_sms * sizeof(T), 256);
    c.x.cand_row = (int*)p;
    p += align_up(2 * (size_t)num_sms * sizeof(int), 256);
    c.x.cand_rows = (T*)p;
    p += align_up(2 * (size_t)num_sms * nbmax * sizeof(T), 256);
    c.x.diag_row = (T*)p;
    return c;
}

// The cooperative panel keeps an R x nb slab in the shared memory of P CTAs
// (one CTA up to 64 KiB of slab, else P = min(SMs, ceil(R / 128))); it
// fits when each CTA's ceil(R / P) rows x nb fit its opt-in shared memory.
template <typename T>
static cudaError_t panel_geometry(const mg_handle_s* h, int R, int nb, int* P_out, int* rpc_out, bool* fits) {
    cudaFuncAttributes fa;
    const cudaError_t e = cudaFuncGetAttributes(&fa, panel_kernel<T>);
    if (e != cudaSuccess) return e;
    const size_t cap = (size_t)h->max_smem_optin - fa.sharedSizeBytes - 256;
    int P;
    if ((size_t)R * nb * sizeof(T) <= 64 * 1024) {
        P = 1;
    } else {
        P = (R + 127) / 128;
        if (P > h->num_sms) P = h->num_sms;
    }
    *P_out = P;
    *rpc_out = (R + P - 1) / P;
    *fits = (size_t)*rpc_out * nb * sizeof(T) <= cap;
    return cudaSuccess;
}

template <typename T>
static mg_status_t launch_panel(mg_handle_t h, GetrfCtx<T>& c, T* A, int lda, int m, int r0, int nb, int* pos,
                                int nopiv = 0) {
    const int R = m - r0;
    auto kern = panel_kernel<T>;
    int P = 1, rpc = R;
    bool fits = false;
    MG_CHECK_CUDA(h, panel_geometry<T>(h, R, nb, &P, &rpc, &fits));
    if (!fits) {
        return fail(h, MG_ERR_UNSUPPORTED, "panel of %d rows x %d columns exceeds shared memory of %d CTAs", R, nb,
                    h->num_sms);
    }
    const size_t smem = (size_t)rpc * nb * sizeof(T);
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ProfScope prof(h, sizeof(T) == 8 ? "panel_f64" : "panel_f32", (double)R * nb * nb,
                   2.0 * R * nb * sizeof(T));
    MG_CHECK_CUDA(h, cudaMemsetAsync(c.ws.bar, 0, sizeof(unsigned), h->stream));
    void* args[] = {&A, &lda, &m, &r0, &nb, &rpc, &nopiv, &pos, &c.piv, &c.ws, &c.x};
    cudaError_t e;
    if (P > 1)
        e = cudaLaunchCooperativeKernel((const void*)kern, dim3(P), dim3(PANEL_THREADS), args, smem, h->stream);
    else
        e = cudaLaunchKernel((const void*)kern, dim3(1), dim3(PANEL_THREADS), args, smem, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "panel_kernel launch");
    h->launches++;
    return MG_OK;
}

template <typename T>
static mg_status_t launch_laswp(mg_handle_t h, T* A, int lda, int r0, int kc, const int* piv, int c_left,
                                int c_right, int n) {
    const int cols = c_left + (n > c_right ? n - c_right : 0);
    if (cols <= 0 || kc <= 0) return MG_OK;
    const int threads = 128;
    int blocks = (cols + threads - 1) / threads;
    ProfScope prof(h, "laswp", 0.0, 4.0 * kc * cols * sizeof(T));
    laswp_kernel<T><<<blocks, threads, 0, h->stream>>>(A, lda, r0, kc, piv, c_left, c_right, n);
    return post_launch(h, "laswp_kernel");
}

template <typename T>
static mg_status_t launch_trsm_llnu(mg_handle_t h, int k, int n, const T* L, int ldl, T* X, int ldx) {
    if (n <= 0 || k <= 0) return MG_OK;
    const int threads = 64;
    const size_t smem = ((size_t)k * k + (size_t)k * threads) * sizeof(T);
    auto kern = trsm_llnu_kernel<T>;
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ProfScope prof(h, sizeof(T) == 8 ? "trsm_f64" : "trsm_f32", (double)k * k * n, 2.0 * k * n * sizeof(T));
    kern<<<(n + threads - 1) / threads, threads, smem, h->stream>>>(k, n, L, ldl, X, ldx);
    return post_launch(h, "trsm_llnu_kernel");
}

template <typename T>
static mg_status_t launch_trsm_lunn(mg_handle_t h, int k, int n, const T* U, int ldu, T* X, int ldx) {
    if (n <= 0 || k <= 0) return MG_OK;
    const int threads = 64;
    const size_t smem = ((size_t)k * k + (size_t)k * threads) * sizeof(T);
    auto kern = trsm_lunn_kernel<T>;
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ProfScope prof(h, sizeof(T) == 8 ? "trsm_f64" : "trsm_f32", (double)k * k * n, 2.0 * k * n * sizeof(T));
    kern<<<(n + threads - 1) / threads, threads, smem, h->stream>>>(k, n, U, ldu, X, ldx);
    return post_launch(h, "trsm_lunn_kernel");
}


// In-place PLU given an exchange area `c` (no allocation); hstat receives the
// error and info words (two host ints).  Returns MG_OK, MG_SINGULAR (info =
// first zero-pivot column, 1-based) or an error.
//
// Blocked path with a look-ahead of one panel (lookahead != 0): after the
// block-row solve of step k, the next panel's 60 columns are updated first
// (near update) and panel k+1 starts right behind it, while the rest of
// the trailing matrix (far update) runs on the handle's low-priority side
// stream; step k+1's interchanges wait for it.  Every element of the
// trailing matrix still receives one fused chain over the step's 60
// columns in the same order, so the factors are those of the plain loop.
static mg_status_t dgetrf_run(mg_handle_t h, int m, int n, double* A, int lda, int* pos, GetrfCtx<double>& c,
                              int* hstat, int* info_out, int nopiv = 0, int lookahead = 0) {
    if (info_out) *info_out = 0;
    MG_CHECK_CUDA(h, cudaMemsetAsync(c.ws.bar, 0, 256, h->stream));  // barrier, error and info words
    iota_kernel<<<(m + 255) / 256, 256, 0, h->stream>>>(pos, m);
    MG_TRY(post_launch(h, "iota_kernel"));

    const int s = m < n ? m : n;
    if (s <= LU_BS * 3 / 2) {
        // Mat's unblocked __PLU2 (LU/__PLU.h:22-51): one panel over all s
        // columns, interchanges on every column.
        MG_TRY(launch_panel<double>(h, c, A, lda, m, 0, s, pos, nopiv));
        if (!nopiv) MG_TRY(launch_laswp<double>(h, A, lda, 0, s, c.piv, 0, s, n));
        if (n > s) {
            MG_TRY(launch_trsm_llnu<double>(h, s, n - s, A, lda, A + (size_t)s * lda, lda));
        }
    } else {
        if (lookahead) MG_TRY(ensure_lookahead(h));
        const cudaStream_t S = h->stream;
        bool far_pending = false;  // a far update was issued on the side stream (event la_ev[1])
        int r = 0;
        bool have_panel = false;   // panel r already factored (by the look-ahead)
        for (; r + LU_BS <= s; r += LU_BS) {
            if (!have_panel) MG_TRY(launch_panel<double>(h, c, A, lda, m, r, LU_BS, pos, nopiv));
            have_panel = false;
            if (far_pending) MG_CHECK_CUDA(h, cudaStreamWaitEvent(S, h->la_ev[1], 0));
            far_pending = false;
            if (!nopiv) MG_TRY(launch_laswp<double>(h, A, lda, r, LU_BS, c.piv, r, r + LU_BS, n));
            if (r + LU_BS < s) {
                const int nt = n - (r + LU_BS);
                const int mt = m - (r + LU_BS);
                double* A12 = A + r + (size_t)(r + LU_BS) * lda;
                const double* L21 = A + (r + LU_BS) + (size_t)r * lda;
                double* A22 = A + (r + LU_BS) + (size_t)(r + LU_BS) * lda;
                MG_TRY(launch_trsm_llnu<double>(h, LU_BS, nt, A + r + (size_t)r * lda, lda, A12, lda));
                const int r1 = r + LU_BS;  // the next panel's first column
                const bool next_full = r1 + LU_BS <= s;
                if (lookahead && next_full && nt > LU_BS) {
                    MG_TRY(dgemm_launch(h, 0, 0, mt, LU_BS, LU_BS, -1.0, L21, lda, A12, lda, 1.0, A22, lda, 0));
                    MG_CHECK_CUDA(h, cudaEventRecord(h->la_ev[0], S));
                    // the next panel on the high-priority side stream: its grid
                    // takes SMs ahead of the far update's tiles as they free up
                    MG_CHECK_CUDA(h, cudaStreamWaitEvent(h->pp_stream, h->la_ev[0], 0));
                    {
                        OnStream on(h, h->pp_stream);
                        MG_TRY(launch_panel<double>(h, c, A, lda, m, r1, LU_BS, pos, nopiv));
                        MG_CHECK_CUDA(h, cudaEventRecord(h->pp_ev[0], h->pp_stream));
                    }
                    MG_CHECK_CUDA(h, cudaStreamWaitEvent(S, h->pp_ev[0], 0));
                    have_panel = true;
                    MG_CHECK_CUDA(h, cudaStreamWaitEvent(h->la_stream, h->la_ev[0], 0));
                    {
                        OnStream on(h, h->la_stream);
                        MG_TRY(dgemm_launch(h, 0, 0, mt, nt - LU_BS, LU_BS, -1.0, L21, lda,
                                            A12 + (size_t)LU_BS * lda, lda, 1.0, A22 + (size_t)LU_BS * lda, lda, 0));
                        MG_CHECK_CUDA(h, cudaEventRecord(h->la_ev[1], h->la_stream));
                    }
                    far_pending = true;
                } else {
                    MG_TRY(dgemm_launch(h, 0, 0, mt, nt, LU_BS, -1.0, L21, lda, A12, lda, 1.0, A22, lda, 0));
                }
            }
        }
        if (far_pending) MG_CHECK_CUDA(h, cudaStreamWaitEvent(S, h->la_ev[1], 0));
        if (r < s) {
            const int rem = s - r;
            MG_TRY(launch_panel<double>(h, c, A, lda, m, r, rem, pos, nopiv));
            if (!nopiv) MG_TRY(launch_laswp<double>(h, A, lda, r, rem, c.piv, r, n, n));
        }
    }
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hstat, c.ws.err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hstat + 1, c.ws.info, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hstat[0]) return fail(h, MG_TIMEOUT, "dgetrf: a panel grid barrier timed out");
    if (info_out) *info_out = hstat[1];
    if (hstat[1]) return fail(h, MG_SINGULAR, "dgetrf: exactly zero pivot column %d", hstat[1]);
    return MG_OK;
}

size_t dgetrf_ws_bytes(int num_sms) { return getrf_ws_bytes<double>(num_sms); }

// In-place PLU; pos (device, m ints) receives Mat's permutation.
mg_status_t dgetrf_impl(mg_handle_t h, int m, int n, double* A, int lda, int* pos, int* info_out) {
    if (info_out) *info_out = 0;
    if (m == 0 || n == 0) return MG_OK;
    MG_TRY(ensure_ws(h, getrf_ws_bytes<double>(h->num_sms)));
    MG_TRY(ensure_hws(h, 64));
    GetrfCtx<double> c = carve<double>(h->ws, h->num_sms);
    return dgetrf_run(h, m, n, A, lda, pos, c, (int*)h->hws, info_out, 0, 1);
}

// In-place LU without pivoting (Mat's LU, LU/__LU.h:71-108) of a square
// n x n A: the PLU pipeline with the diagonal as every pivot (the panel's
// candidate is the diagonal row; no interchanges).  Mat's panel stops at an
// exactly zero pivot; here info records it and the factorization goes on.
mg_status_t dlu_nopiv_impl(mg_handle_t h, int n, double* A, int lda, int* info_out) {
    if (info_out) *info_out = 0;
    if (n == 0) return MG_OK;
    const size_t base = align_up(getrf_ws_bytes<double>(h->num_sms), 256);
    MG_TRY(ensure_ws(h, base + (size_t)n * sizeof(int)));
    MG_TRY(ensure_hws(h, 64));
    GetrfCtx<double> c = carve<double>(h->ws, h->num_sms);
    int* pos = (int*)((char*)h->ws + base);
    return dgetrf_run(h, n, n, A, lda, pos, c, (int*)h->hws, info_out, 1);
}

// ----------------------------------------------------------- mixed (fp32)
size_t sgetrf_xchg_bytes(int num_sms) { return getrf_ws_bytes<float>(num_sms); }

// FP32 panel: one 16-CTA cluster (panel_f32.cu) when the panel is too tall
// for one CTA's shared memory and fits the cluster; else the cooperative grid
// (or, for short panels, the single-CTA) kernel.  Same factors either way.
static mg_status_t launch_panel_f32(mg_handle_t h, GetrfCtx<float>& c, float* A, int lda, int m, int r0, int w,
                                    int* pos, bool tourn = false) {
    const int R = m - r0;
    if ((size_t)R * w * sizeof(float) > 64 * 1024 && R >= w && R <= panel_cluster_rows(h))
        return sgetf2_cluster(h, A, lda, m, r0, w, pos, c.piv, c.ws.info, c.ws.err, tourn);
    return launch_panel<float>(h, c, A, lda, m, r0, w, pos);
}


// FP32 blocked right-looking LU with partial pivoting for the mixed solve,
// with a look-ahead of one panel.  Step k on the handle's stream S:
//
//   [wait for the far update of step k-1] interchanges of panel k on the
//   columns to its right -> U12 = L11^{-1} A12 and its split terms (one
//   kernel) -> update of the next panel's columns (near update) -> panel
//   k+1 -> its interchanges on the columns to its left -> split of its L21
//   (into the buffer of parity k+1)
//
// while a low-priority side stream runs the far update (the trailing
// columns beyond the next panel) of step k on num_sms - 16 CTAs as soon as
// the near update is done.  The panel is queued directly behind the near
// update on S and submitted before the far update, so its 16-CTA cluster
// takes its SMs before the far update's persistent grid fills the rest.  A
// panel too tall for the cluster (the cooperative grid) is not overlapped.
//
// The trailing updates run on the BF16 tensor cores with `nterms` split
// terms (fp32 accumulation).  `xchg` holds sgetrf_xchg_bytes(); splitA and
// splitA2 / splitB hold bf16x_split_bytes(n, nb, nterms).  The block-row
// solve U12 = L11^{-1} A12 is one FP32 substitution kernel that also writes
// U12's split terms (bf16x_trsm_split).
mg_status_t sgetrf_mixed(mg_handle_t h, int n, float* A, int lda, int* pos, int nb, int nterms, void* xchg,
                         void* splitA, void* splitA2, void* splitB, int* gemm_err, int* info_out, bool tourn) {
    if (info_out) *info_out = 0;
    if (n == 0) return MG_OK;
    if (nb > PANEL_MAX_NB || nb > 128) return fail(h, MG_ERR_ARG, "sgetrf_mixed: block size %d > 128", nb);
    MG_TRY(ensure_hws(h, 64));
    MG_TRY(ensure_lookahead(h));
    GetrfCtx<float> c = carve<float>(xchg, h->num_sms);
    const cudaStream_t S = h->stream, S2 = h->la_stream;
    MG_CHECK_CUDA(h, cudaMemsetAsync(xchg, 0, 256, S));
    iota_kernel<<<(n + 255) / 256, 256, 0, S>>>(pos, n);
    MG_TRY(post_launch(h, "iota_kernel"));
    void* const splitL[2] = {splitA, splitA2};
    const bool cluster_ok = panel_cluster_rows(h) > 0;
    const int nsteps = (n + nb - 1) / nb;

    // panel k, then everything that depends only on it
    auto panel = [&](int k) -> mg_status_t {
        const int r = k * nb, w = nb < n - r ? nb : n - r;
        return launch_panel_f32(h, c, A, lda, n, r, w, pos, tourn);
    };
    // after panel k, on the side stream P (off the critical path): its
    // interchanges on the columns to its left and the split of its L21; the
    // next near update waits for them (event pp_ev[1]), and so, through it,
    // does the panel that next overwrites the pivot list
    bool pp_pending = false;
    auto after_panel = [&](int k) -> mg_status_t {
        const int r = k * nb, w = nb < n - r ? nb : n - r;
        MG_CHECK_CUDA(h, cudaEventRecord(h->pp_ev[0], S));
        MG_CHECK_CUDA(h, cudaStreamWaitEvent(h->pp_stream, h->pp_ev[0], 0));
        {
            OnStream on(h, h->pp_stream);
            MG_TRY(launch_laswp<float>(h, A, lda, r, w, c.piv, r, n, n));  // columns [0, r)
            if (r + w < n) {
                const int nt = n - (r + w);
                ProfScope prof(h, "split", 0.0, 2.0 * nt * w * (4.0 + 2.0 * nterms));
                MG_TRY(bf16x_split<float>(h, true, A + (r + w) + (size_t)r * lda, lda, nt, w, nterms, splitL[k & 1]));
            }
            MG_CHECK_CUDA(h, cudaEventRecord(h->pp_ev[1], h->pp_stream));
        }
        pp_pending = true;
        return MG_OK;
    };
    auto wait_after_panel = [&]() -> mg_status_t {
        if (pp_pending) MG_CHECK_CUDA(h, cudaStreamWaitEvent(S, h->pp_ev[1], 0));
        pp_pending = false;
        return MG_OK;
    };
    // a panel overlaps the previous trailing update only on the cluster path
    auto overlappable = [&](int k) {
        const int r = k * nb, R = n - r, w = nb < R ? nb : R;
        return cluster_ok && (size_t)R * w * sizeof(float) > 64 * 1024 && R >= w && R <= panel_cluster_rows(h);
    };

    MG_TRY(panel(0));
    MG_TRY(after_panel(0));
    bool far_pending = false;  // a far update was issued on S2 (event la_ev[1])
    for (int k = 0; k < nsteps; ++k) {
        const int r = k * nb, w = nb < n - r ? nb : n - r;
        if (r + w >= n) break;
        const int nt = n - (r + w);
        const int kp = bf16x_kpad(w);  // row length of this step's split terms
        if (far_pending) MG_CHECK_CUDA(h, cudaStreamWaitEvent(S, h->la_ev[1], 0));
        far_pending = false;
        MG_TRY(launch_laswp<float>(h, A, lda, r, w, c.piv, 0, r + w, n));  // columns [r + w, n)
        float* A12 = A + r + (size_t)(r + w) * lda;
        {
            ProfScope prof(h, "trsm_f32", (double)w * w * (double)nt, 8.0 * w * (double)nt);
            MG_TRY(bf16x_trsm_split(h, A + r + (size_t)r * lda, lda, A12, nt, w, nterms, splitB));
        }
        MG_TRY(wait_after_panel());
        const void* L21 = splitL[k & 1];
        float* A22 = A + (r + w) + (size_t)(r + w) * lda;
        const int w1 = nb < nt ? nb : nt;  // the next panel's columns
        MG_TRY(bf16x_gemm_presplit(h, nterms, nt, w1, w, -1.0f, L21, splitB, 1.0f, A22, lda, gemm_err, 0,
                                   (size_t)nt * kp, 0, false, true, false, true));  // the next panel: kept in L2
        const bool ov = overlappable(k + 1);
        const void* Brest = (const char*)splitB + (size_t)w1 * kp * 2;
        if (nt > w1 && ov) {
            // the panel is submitted before the far update, so that its
            // cluster is placed while the GPU is still free of the far
            // update's persistent grid
            MG_CHECK_CUDA(h, cudaEventRecord(h->la_ev[0], S));
            MG_TRY(panel(k + 1));
            MG_CHECK_CUDA(h, cudaStreamWaitEvent(S2, h->la_ev[0], 0));
            {
                OnStream on(h, S2);
                MG_TRY(bf16x_gemm_presplit(h, nterms, nt, nt - w1, w, -1.0f, L21, Brest, 1.0f,
                                           A22 + (size_t)w1 * lda, lda, gemm_err, 0, (size_t)nt * kp,
                                           h->num_sms - 16, true, true));
                MG_CHECK_CUDA(h, cudaEventRecord(h->la_ev[1], S2));
            }
            far_pending = true;
        } else {
            if (nt > w1)
                MG_TRY(bf16x_gemm_presplit(h, nterms, nt, nt - w1, w, -1.0f, L21, Brest, 1.0f,
                                           A22 + (size_t)w1 * lda, lda, gemm_err, 0, (size_t)nt * kp, 0, true,
                                           true));
            MG_TRY(panel(k + 1));
        }
        MG_TRY(after_panel(k + 1));
    }
    if (far_pending) MG_CHECK_CUDA(h, cudaStreamWaitEvent(S, h->la_ev[1], 0));
    MG_TRY(wait_after_panel());
    int* hw = (int*)h->hws;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw, c.ws.err, sizeof(int), cudaMemcpyDeviceToHost, S));
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw + 1, c.ws.info, sizeof(int), cudaMemcpyDeviceToHost, S));
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw + 2, gemm_err, sizeof(int), cudaMemcpyDeviceToHost, S));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(S));
    if (hw[0] || hw[2]) return fail(h, MG_TIMEOUT, "sgetrf_mixed: a bounded device wait timed out");
    if (info_out) *info_out = hw[1];
    if (hw[1]) return fail(h, MG_SINGULAR, "sgetrf_mixed: exactly zero pivot column %d", hw[1]);
    return MG_OK;
}

// Mat's narrow substitutions (LU/__Solve_direct.h:118-139) on in-place
// factors of element type TM, in FP64: blocks of TRSV_B rows, the block's
// triangle on one CTA, the rows outside it by a grid.
template <typename TM>
static mg_status_t narrow_subst(mg_handle_t h, int n, int nrhs, const TM* LU, int lda, double* X, int ldx) {
    const int ublocks = h->num_sms;
    for (int b0 = 0; b0 < n; b0 += TRSV_B) {
        const int b1 = b0 + TRSV_B < n ? b0 + TRSV_B : n;
        trsv_lower_diag_kernel<TM, double><<<1, 256, 0, h->stream>>>(n, nrhs, LU, lda, X, ldx, b0, b1);
        MG_TRY(post_launch(h, "trsv_lower_diag_kernel"));
        if (b1 < n) {
            int blocks = (n - b1 + 127) / 128;
            if (blocks > ublocks) blocks = ublocks;
            trsv_lower_update_kernel<TM, double><<<blocks, 128, 0, h->stream>>>(n, nrhs, LU, lda, X, ldx, b0, b1);
            MG_TRY(post_launch(h, "trsv_lower_update_kernel"));
        }
    }
    const int last = ((n - 1) / TRSV_B) * TRSV_B;
    for (int b0 = last; b0 >= 0; b0 -= TRSV_B) {
        const int b1 = b0 + TRSV_B < n ? b0 + TRSV_B : n;
        trsv_upper_diag_kernel<TM, double><<<1, 256, 0, h->stream>>>(n, nrhs, LU, lda, X, ldx, b0, b1);
        MG_TRY(post_launch(h, "trsv_upper_diag_kernel"));
        if (b0 > 0) {
            int blocks = (b0 + 127) / 128;
            if (blocks > ublocks) blocks = ublocks;
            trsv_upper_update_kernel<TM, double><<<blocks, 128, 0, h->stream>>>(n, nrhs, LU, lda, X, ldx, b0, b1);
            MG_TRY(post_launch(h, "trsv_upper_update_kernel"));
        }
    }
    return MG_OK;
}

// X := A^{-1} B given the in-place factors, pos from dgetrf_impl, in the
// operation order of Mat's Solve_direct (LU/__Solve_direct.h:146-220):
//  * nrhs <= 4: the narrow scalar substitutions (:112-139);
//  * n <= 90:   one unit-lower and one upper TRSM over the whole matrix (:166-190);
//  * otherwise: __Solve_direct_LU_X (:1-66), blocks of 60 rows: forward, the
//    block's TRSM then X(below) -= L(below, block) X(block); backward from
//    the last block, X(above) -= U(above, block) X(block).  The products are
//    the fused-chain DGEMM (alpha -1, beta 1), whose per-element order is
//    that of Mat's packed kernels whatever their NC / MC tiling.
// Mat's 8-column TRSM buffers hold 60 rows, so its one-block case with
// 60 < n <= 90 and 8 or more right-hand sides writes past them (a crash in
// the reference build); here that case computes the same arithmetic as
// the rows that fit.
mg_status_t dgetrs_impl(mg_handle_t h, int n, int nrhs, const double* LU, int lda, const int* pos,
                        const double* B, int ldb, double* X, int ldx) {
    if (n == 0 || nrhs == 0) return MG_OK;
    {
        const size_t total = (size_t)n * nrhs;
        int blocks = (int)((total + 255) / 256);
        if (blocks > h->num_sms * 8) blocks = h->num_sms * 8;
        permute_rows_kernel<double><<<blocks, 256, 0, h->stream>>>(n, nrhs, pos, B, ldb, X, ldx);
        MG_TRY(post_launch(h, "permute_rows_kernel"));
    }
    if (nrhs > 4) {
        if (n <= LU_BS * 3 / 2) {
            MG_TRY(launch_trsm_llnu<double>(h, n, nrhs, LU, lda, X, ldx));
            return launch_trsm_lunn<double>(h, n, nrhs, LU, lda, X, ldx);
        }
        for (int r = 0; r < n; r += LU_BS) {
            const int l = n - r < LU_BS ? n - r : LU_BS;
            MG_TRY(launch_trsm_llnu<double>(h, l, nrhs, LU + r + (size_t)r * lda, lda, X + r, ldx));
            if (r + l < n)
                MG_TRY(dgemm_launch(h, 0, 0, n - r - l, nrhs, l, -1.0, LU + (r + l) + (size_t)r * lda, lda, X + r,
                                    ldx, 1.0, X + r + l, ldx, 0));
        }
        for (int r = ((n - 1) / LU_BS) * LU_BS; r >= 0; r -= LU_BS) {
            const int l = n - r < LU_BS ? n - r : LU_BS;
            MG_TRY(launch_trsm_lunn<double>(h, l, nrhs, LU + r + (size_t)r * lda, lda, X + r, ldx));
            if (r > 0)
                MG_TRY(dgemm_launch(h, 0, 0, r, nrhs, l, -1.0, LU + (size_t)r * lda, lda, X + r, ldx, 1.0, X, ldx,
                                    0));
        }
        return MG_OK;
    }
    return narrow_subst<double>(h, n, nrhs, LU, lda, X, ldx);
}

// X := U^{-1} X in FP64 for an upper triangle held in fp32 (the mixed QR's R).
mg_status_t upper_solve_f32_factors(mg_handle_t h, int n, int nrhs, const float* U, int ldu, double* X, int ldx) {
    if (n == 0 || nrhs == 0) return MG_OK;
    const int ublocks = h->num_sms;
    const int last = ((n - 1) / TRSV_B) * TRSV_B;
    for (int b0 = last; b0 >= 0; b0 -= TRSV_B) {
        const int b1 = b0 + TRSV_B < n ? b0 + TRSV_B : n;
        trsv_upper_diag_kernel<float, double><<<1, 256, 0, h->stream>>>(n, nrhs, U, ldu, X, ldx, b0, b1);
        MG_TRY(post_launch(h, "trsv_upper_diag_kernel"));
        if (b0 > 0) {
            int blocks = (b0 + 127) / 128;
            if (blocks > ublocks) blocks = ublocks;
            trsv_upper_update_kernel<float, double><<<blocks, 128, 0, h->stream>>>(n, nrhs, U, ldu, X, ldx, b0, b1);
            MG_TRY(post_launch(h, "trsv_upper_update_kernel"));
        }
    }
    return MG_OK;
}

// X := (LU)^{-1} P B in FP64 arithmetic for factors held in fp32 (the mixed
// LU's, whose pos follows Mat's convention): the same narrow substitution
// kernels with each fp32 factor entry widened exactly to fp64.  This is a
// fixed linear operator M^{-1}, M = P^T L U, as GMRES-IR's preconditioner
// needs.
mg_status_t lu_solve_f32_factors(mg_handle_t h, int n, int nrhs, const float* LU, int lda, const int* pos,
                                 const double* B, int ldb, double* X, int ldx) {
    if (n == 0 || nrhs == 0) return MG_OK;
    const size_t total = (size_t)n * nrhs;
    int blocks = (int)((total + 255) / 256);
    if (blocks > h->num_sms * 8) blocks = h->num_sms * 8;
    permute_rows_kernel<double><<<blocks, 256, 0, h->stream>>>(n, nrhs, pos, B, ldb, X, ldx);
    MG_TRY(post_launch(h, "permute_rows_kernel"));
    return narrow_subst<float>(h, n, nrhs, LU, lda, X, ldx);
}

// ------------------------------------------------ allocation-free variant
// Some callers of this LU cannot allocate device memory at call time: code
// that runs inside another system's memory pool or under a fixed memory
// budget (an engine embedding the solver next to its own allocator), callers
// that must not stall the whole device (cudaMalloc / cudaFree synchronise
// it, and the handle's workspace grows through them), and plugin hosts that
// forbid device allocation outright.  mg_dgetrf_noalloc serves them: its
// panel exchange area, pivot list, barrier counter and status words live in
// one file-scope device array of fixed size, shared by every call in the
// process on that device.
constexpr int kNoAllocMaxSms = 256;      // exchange slots for up to this many panel CTAs
constexpr int kNoAllocMaxNb = 96;        // widest panel of the FP64 PLU (blocks of 60; <= 90 unblocked)
constexpr int kNoAllocMaxRows = 65536;   // rows whose panel slab fits the SMs' shared memory
constexpr size_t kNoAllocScratchBytes = getrf_ws_bytes<double>(kNoAllocMaxSms, kNoAllocMaxNb);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {nullptr};

// Device address of g_noalloc_scratch on the current device (looked up once per device).
cudaError_t noalloc_scratch(int dev, void** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return cudaSuccess;
}
}  // namespace

}  // namespace mg

extern "C" {

mg_status_t mg_dgetrf(mg_handle_t h, int m, int n, double* A, int lda, int* pos, int* info) {
    if (!h) return MG_ERR_ARG;
    if (m < 0 || n < 0 || lda < (m > 1 ? m : 1) || ((size_t)m * n && (!A || !pos)))
        return mg::fail(h, MG_ERR_ARG, "mg_dgetrf: bad arguments (m=%d n=%d lda=%d)", m, n, lda);
    return mg::dgetrf_impl(h, m, n, A, lda, pos, info);
}

mg_status_t mg_sgetf2_ex(mg_handle_t h, int flags, int m, int n, float* A, int lda, int* pos, int* info) {
    if (info) *info = 0;
    if (!h) return MG_ERR_ARG;
    if (m < 0 || n < 0 || n > 128 || lda < (m > 1 ? m : 1) || ((size_t)m * n && (!A || !pos)))
        return mg::fail(h, MG_ERR_ARG, "mg_sgetf2_ex: bad arguments (m=%d n=%d lda=%d, n must be <= 128)", m, n, lda);
    if (m == 0 || n == 0) return MG_OK;
    const int w = n < m ? n : m;
    MG_TRY(mg::ensure_ws(h, mg::getrf_ws_bytes<float>(h->num_sms)));
    MG_TRY(mg::ensure_hws(h, 64));
    mg::GetrfCtx<float> c = mg::carve<float>(h->ws, h->num_sms);
    MG_CHECK_CUDA(h, cudaMemsetAsync(c.ws.bar, 0, 256, h->stream));
    iota_kernel<<<(m + 255) / 256, 256, 0, h->stream>>>(pos, m);
    MG_TRY(mg::post_launch(h, "iota_kernel"));
    MG_TRY(mg::launch_panel_f32(h, c, A, lda, m, 0, w, pos, (flags & MG_PANEL_TOURNAMENT) != 0));
    if (w < n) {  // columns right of a short panel (m < n): interchanges only
        MG_TRY(mg::launch_laswp<float>(h, A, lda, 0, w, c.piv, 0, w, n));
    }
    int* hw = (int*)h->hws;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw, c.ws.err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hw + 1, c.ws.info, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (hw[0]) return mg::fail(h, MG_TIMEOUT, "mg_sgetf2: a panel grid barrier timed out");
    if (info) *info = hw[1];
    if (hw[1]) return mg::fail(h, MG_SINGULAR, "mg_sgetf2: exactly zero pivot column %d", hw[1]);
    return MG_OK;
}

mg_status_t mg_sgetf2(mg_handle_t h, int m, int n, float* A, int lda, int* pos, int* info) {
    return mg_sgetf2_ex(h, 0, m, n, A, lda, pos, info);
}

mg_status_t mg_sgetrf(mg_handle_t h, int n, float* A, int lda, int* pos, int* info) {
    if (info) *info = 0;
    if (!h) return MG_ERR_ARG;
    if (n < 0 || lda < (n > 1 ? n : 1) || (n && (!A || !pos)))
        return mg::fail(h, MG_ERR_ARG, "mg_sgetrf: bad arguments (n=%d lda=%d)", n, lda);
    if (n == 0) return MG_OK;
    constexpr int nb = 128, nterms = 3;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = mg::align_up(off + bytes, 1024);
        return o;
    };
    const size_t oX = take(mg::sgetrf_xchg_bytes(h->num_sms));
    const size_t oSA = take(mg::bf16x_split_bytes(n, nb, nterms));
    const size_t oSA2 = take(mg::bf16x_split_bytes(n, nb, nterms));
    const size_t oSB = take(mg::bf16x_split_bytes(n, nb, nterms));
    const size_t oE = take(64);
    MG_TRY(mg::ensure_ws(h, off));
    char* b = (char*)h->ws;
    int* gerr = (int*)(b + oE);
    MG_CHECK_CUDA(h, cudaMemsetAsync(gerr, 0, 64, h->stream));
    return mg::sgetrf_mixed(h, n, A, lda, pos, nb, nterms, b + oX, b + oSA, b + oSA2, b + oSB, gerr, info);
}

mg_status_t mg_dgetrf_noalloc(void* cuda_stream, int m, int n, double* A, int lda, int* pos, int* info) {
    if (info) *info = 0;
    if (m < 0 || n < 0 || lda < (m > 1 ? m : 1) || ((size_t)m * n && (!A || !pos))) return MG_ERR_ARG;
    if (m > mg::kNoAllocMaxRows) return MG_ERR_UNSUPPORTED;  // beyond the fixed scratch / panel capacity
    if (m == 0 || n == 0) return MG_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MG_ERR_CUDA;
    void* scratch = nullptr;
    if (mg::noalloc_scratch(dev, &scratch) != cudaSuccess) return MG_ERR_CUDA;
    mg_handle_s h;  // a handle on the stack: no workspace, no pinned memory
    h.stream = (cudaStream_t)cuda_stream;
    h.device = dev;
    if (cudaDeviceGetAttribute(&h.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&h.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return MG_ERR_CUDA;
    if (h.num_sms > mg::kNoAllocMaxSms) return MG_ERR_UNSUPPORTED;
    // the first (tallest) panel decides whether the slab fits: refuse before any launch
    const int s = m < n ? m : n;
    int P = 1, rpc = m;
    bool fits = false;
    if (mg::panel_geometry<double>(&h, m, s <= LU_BS * 3 / 2 ? s : LU_BS, &P, &rpc, &fits) != cudaSuccess)
        return MG_ERR_CUDA;
    if (!fits) return MG_ERR_UNSUPPORTED;
    mg::GetrfCtx<double> c = mg::carve<double>(scratch, h.num_sms, mg::kNoAllocMaxNb);
    int hstat[2] = {0, 0};
    return mg::dgetrf_run(&h, m, n, A, lda, pos, c, hstat, info);
}

mg_status_t mg_dlu(mg_handle_t h, int n, double* A, int lda, int* info) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || lda < (n > 1 ? n : 1) || (n && !A)) return mg::fail(h, MG_ERR_ARG, "mg_dlu: bad arguments");
    return mg::dlu_nopiv_impl(h, n, A, lda, info);
}

mg_status_t mg_dgetrs(mg_handle_t h, int n, int nrhs, const double* LU, int lda, const int* pos, const double* B,
                      int ldb, double* X, int ldx) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || nrhs < 0 || lda < (n > 1 ? n : 1) || ldb < (n > 1 ? n : 1) || ldx < (n > 1 ? n : 1))
        return mg::fail(h, MG_ERR_ARG, "mg_dgetrs: bad arguments");
    if ((size_t)n * nrhs && (!LU || !pos || !B || !X)) return mg::fail(h, MG_ERR_ARG, "mg_dgetrs: null pointer");
    if (B == X && ldb != ldx) return mg::fail(h, MG_ERR_ARG, "mg_dgetrs: in-place B needs ldb == ldx");
    if (B == X) return mg::fail(h, MG_ERR_ARG, "mg_dgetrs: B and X must not alias");
    return mg::dgetrs_impl(h, n, nrhs, LU, lda, pos, B, ldb, X, ldx);
}

mg_status_t mg_dgesv(mg_handle_t h, int n, int nrhs, const double* A, int lda, const double* B, int ldb, double* X,
                     int ldx, int* info) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || nrhs < 0 || lda < (n > 1 ? n : 1) || ldb < (n > 1 ? n : 1) || ldx < (n > 1 ? n : 1))
        return mg::fail(h, MG_ERR_ARG, "mg_dgesv: bad arguments");
    if (info) *info = 0;
    if (n == 0 || nrhs == 0) return MG_OK;
    // Solve_direct takes A by value (LU/__Solve_direct.h:146): factor a copy.
    const size_t abytes = mg::align_up((size_t)n * n * sizeof(double), 256);
    const size_t pbytes = mg::align_up((size_t)n * sizeof(int), 256);
    // the copy lives after the getrf workspace
    const size_t base = mg::align_up(mg::getrf_ws_bytes<double>(h->num_sms), 256);
    MG_TRY(mg::ensure_ws(h, base + abytes + pbytes));
    double* Acopy = (double*)((char*)h->ws + base);
    int* pos = (int*)((char*)h->ws + base + abytes);
    MG_CHECK_CUDA(h, cudaMemcpy2DAsync(Acopy, (size_t)n * sizeof(double), A, (size_t)lda * sizeof(double),
                                       (size_t)n * sizeof(double), n, cudaMemcpyDeviceToDevice, h->stream));
    mg_status_t s = mg::dgetrf_impl(h, n, n, Acopy, n, pos, info);
    if (s != MG_OK && s != MG_SINGULAR) return s;
    MG_TRY(mg::dgetrs_impl(h, n, nrhs, Acopy, n, pos, B, ldb, X, ldx));
    return s;
}

mg_status_t mg_ddet(mg_handle_t h, int n, const double* A, int lda, double* det) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || lda < (n > 1 ? n : 1) || !det || (n && !A)) return mg::fail(h, MG_ERR_ARG, "mg_ddet: bad arguments");
    *det = 1.0;
    if (n == 0) return MG_OK;
    // Mat's Det (LU/__Det.h:30-101): the PLU factors, the parity of the row
    // permutation, then the product sign * U(0,0) * U(1,1) * ... in order.
    const size_t abytes = mg::align_up((size_t)n * n * sizeof(double), 256);
    const size_t pbytes = mg::align_up((size_t)n * sizeof(int), 256);
    const size_t base = mg::align_up(mg::getrf_ws_bytes<double>(h->num_sms), 256);
    MG_TRY(mg::ensure_ws(h, base + abytes + pbytes));
    MG_TRY(mg::ensure_hws(h, (size_t)n * (sizeof(double) + sizeof(int)) + 64));
    double* Acopy = (double*)((char*)h->ws + base);
    int* pos = (int*)((char*)h->ws + base + abytes);
    MG_CHECK_CUDA(h, cudaMemcpy2DAsync(Acopy, (size_t)n * sizeof(double), A, (size_t)lda * sizeof(double),
                                       (size_t)n * sizeof(double), n, cudaMemcpyDeviceToDevice, h->stream));
    int info = 0;
    mg_status_t s = mg::dgetrf_impl(h, n, n, Acopy, n, pos, &info);
    if (s != MG_OK && s != MG_SINGULAR) return s;
    double* hd = (double*)h->hws;
    int* hp = (int*)(hd + n);
    MG_CHECK_CUDA(h, cudaMemcpy2DAsync(hd, sizeof(double), Acopy, (size_t)(n + 1) * sizeof(double), sizeof(double), n,
                                       cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hp, pos, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    std::vector<char> seen((size_t)n, 0);
    long long swaps = 0;
    for (int i = 0; i < n; ++i) {
        if (seen[i]) continue;
        int len = 0;
        for (int j = i; !seen[j]; j = hp[j]) {
            seen[j] = 1;
            ++len;
        }
        swaps += len - 1;
    }
    double d = (swaps & 1) ? -1.0 : 1.0;
    for (int i = 0; i < n; ++i) d = d * hd[i];
    *det = d;
    return MG_OK;
}

}  // extern "C"
