// Matrix inverse in Mat's operation order (Mat-8.3.1/LU/__Inv.h):
//
//   PLU of a copy (lu.cu); every column i of U scaled by t_i = 1 / u_ii
//   (rows above the diagonal; :117-122) and X = diag(t); X := X U^{-1} and
//   X := X L^{-1} with unit triangles; columns permuted, Ainv(:, pos[i]) =
//   X(:, i) (:124-142, the swap chains of __Inv_swap are that permutation).
//   n <= 90: one block (__Inv_small, :164-205).  Larger: __Inv_X_LU
//   (:4-77), blocks of 60 columns; forward, the rows 0 .. r+l-1 of column
//   block r are solved against its diagonal block of U, then
//   X(0:r+l, r+60:) -= X(0:r+l, r:r+l) U(r:r+l, r+60:); backward from the last
//   block, all rows of column block r are solved against L's diagonal block,
//   then X(:, 0:r) -= X(:, r:r+l) L(r:r+l, 0:r).  The products are the
//   fused-chain DGEMM (alpha -1, beta 1), the order of Mat's packed kernels.
//
// The right solves act on each row of X independently: one thread per row,
// the row and the triangle in shared memory.  Their arithmetic is that of
// Mat's AVX-512 __Solve_direct_XU / _XL (LU/__Base.h:541-662, 8-column
// groups) as the reference build evaluates it, with g++ contracting the
// intrinsic products into the sums: inside an 8-column group, fused column
// updates; from the group to a later column, eight products summed as
// fma(x0, q0, x1 q1), fma(x2, q2, x3 q3), ... added as a tree for rows in the
// 8-row vector part of their 60-row block, and as the chain q1 x1, then
// fma(q0, x0, .), fma(q2, x2, .) .. fma(q7, x7, .) for the rows of its
// scalar tail.  Plain products and sums use __dmul_rn / __dadd_rn so that
// nvcc does not contract them differently.
#include "mg_internal.cuh"

namespace {

constexpr int INV_BS = 60;       // Mat-8.3.1/Mat.h:71-73 (AVX-512)
constexpr int INV_THREADS = 64;  // rows per CTA of the row solves

// Column scaling of U and X = diag(1 / u_ii); X is zero on entry.
__global__ void inv_scale_kernel(int n, double* __restrict__ A, int lda, double* __restrict__ X, int ldx) {
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        double* col = A + (size_t)i * lda;
        const double t = 1.0 / col[i];
        for (int j = threadIdx.x; j < i; j += blockDim.x) col[j] = __dmul_rn(col[j], t);
        if (threadIdx.x == 0) X[i + (size_t)i * ldx] = t;
    }
}

__device__ __forceinline__ double sum8_tree(const double* q, const double* x) {
    const double e0 = fma(x[0], q[0], __dmul_rn(x[1], q[1]));
    const double e1 = fma(x[2], q[2], __dmul_rn(x[3], q[3]));
    const double e2 = fma(x[4], q[4], __dmul_rn(x[5], q[5]));
    const double e3 = fma(x[6], q[6], __dmul_rn(x[7], q[7]));
    return __dadd_rn(__dadd_rn(e0, e1), __dadd_rn(e2, e3));
}

__device__ __forceinline__ double sum8_chain(const double* q, const double* x) {
    double t = __dmul_rn(q[1], x[1]);
    t = fma(q[0], x[0], t);
#pragma unroll
    for (int u = 2; u < 8; ++u) t = fma(q[u], x[u], t);
    return t;
}

// Rows 0 .. rows-1 of X (columns 0 .. n-1, n <= 90) := X T^{-1} with T the
// unit upper (UPPER) or unit lower n x n triangle.  blk is the row-block
// length that decides the vector / tail split (60, or n for one block).
template <bool UPPER>
__global__ void __launch_bounds__(INV_THREADS) inv_rows_kernel(int rows, int blk, int n, const double* __restrict__ T,
                                                              int ldt, double* __restrict__ X, int ldx) {
    extern __shared__ __align__(16) double smem[];
    double* sT = smem;       // n x n column-major
    double* sx = smem + n * n;  // [n][INV_THREADS]
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) sT[e] = T[(e % n) + (size_t)(e / n) * ldt];
    const int t = threadIdx.x, row = blockIdx.x * INV_THREADS + t;
    if (row < rows)
        for (int c = 0; c < n; ++c) sx[c * INV_THREADS + t] = X[row + (size_t)c * ldx];
    __syncthreads();
    if (row >= rows) return;
    const int i0 = (row / blk) * blk;
    const int m = min(blk, rows - i0);
    const bool tree = (row - i0) < m - m % 8;
#define XC(c) sx[(c) * INV_THREADS + t]
    if (UPPER) {
        int r = 0;
        for (; r + 8 <= n; r += 8) {
            for (int j = r; j < r + 8; ++j) {
                const double xj = XC(j);
                for (int i = j + 1; i < r + 8; ++i) XC(i) = fma(xj, -sT[j + i * n], XC(i));
            }
            double xv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) xv[u] = XC(r + u);
            for (int i = r + 8; i < n; ++i) {
                double q[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) q[u] = -sT[(r + u) + i * n];
                XC(i) = __dadd_rn(XC(i), tree ? sum8_tree(q, xv) : sum8_chain(q, xv));
            }
        }
        for (; r < n; ++r) {
            const double xr = XC(r);
            for (int i = r + 1; i < n; ++i) XC(i) = fma(xr, -sT[r + i * n], XC(i));
        }
    } else {
        int r = n - 1;
        for (; r - 7 >= 1; r -= 8) {
            for (int j = r; j > r - 7; --j) {
                const double xj = XC(j);
                for (int i = r - 7; i < j; ++i) XC(i) = fma(xj, -sT[j + i * n], XC(i));
            }
            double xv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) xv[u] = XC(r - u);
            for (int i = 0; i < r - 7; ++i) {
                double q[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) q[u] = -sT[(r - u) + i * n];
                XC(i) = __dadd_rn(XC(i), tree ? sum8_tree(q, xv) : sum8_chain(q, xv));
            }
        }
        for (; r > 0; --r) {
            const double xr = XC(r);
            for (int i = 0; i < r; ++i) XC(i) = fma(xr, -sT[r + i * n], XC(i));
        }
    }
    for (int c = 0; c < n; ++c) X[row + (size_t)c * ldx] = XC(c);
#undef XC
}

// Ainv(:, pos[i]) = X(:, i)
__global__ void inv_permute_cols_kernel(int n, const int* __restrict__ pos, const double* __restrict__ X, int ldx,
                                        double* __restrict__ Ainv, int ldinv) {
    const size_t total = (size_t)n * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % n), i = (int)(e / n);
        Ainv[r + (size_t)pos[i] * ldinv] = X[r + (size_t)i * ldx];
    }
}

template <bool UPPER>
mg_status_t launch_rows(mg_handle_t h, int rows, int blk, int n, const double* T, int ldt, double* X, int ldx) {
    if (rows <= 0 || n <= 0) return MG_OK;
    const size_t smem = ((size_t)n * n + (size_t)n * INV_THREADS) * sizeof(double);
    auto kern = inv_rows_kernel<UPPER>;
    MG_CHECK_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mg::ProfScope prof(h, "inv_rows", (double)rows * n * n, 2.0 * rows * n * sizeof(double));
    kern<<<(rows + INV_THREADS - 1) / INV_THREADS, INV_THREADS, smem, h->stream>>>(rows, blk, n, T, ldt, X, ldx);
    return mg::post_launch(h, UPPER ? "inv_rows_kernel<upper>" : "inv_rows_kernel<lower>");
}

}  // namespace

namespace mg {

// Ainv := A^{-1} from the in-place PLU factors LU (ld n, modified: U's
// columns are scaled) and pos; X is an n x n scratch (ld n).
mg_status_t dinv_from_lu(mg_handle_t h, int n, double* LU, const int* pos, double* X, double* Ainv, int ldinv) {
    MG_CHECK_CUDA(h, cudaMemsetAsync(X, 0, (size_t)n * n * sizeof(double), h->stream));
    inv_scale_kernel<<<n < h->num_sms * 8 ? n : h->num_sms * 8, 128, 0, h->stream>>>(n, LU, n, X, n);
    MG_TRY(post_launch(h, "inv_scale_kernel"));
    if (n <= INV_BS * 3 / 2) {
        MG_TRY(launch_rows<true>(h, n, n, n, LU, n, X, n));
        MG_TRY(launch_rows<false>(h, n, n, n, LU, n, X, n));
    } else {
        for (int r = 0; r < n; r += INV_BS) {
            const int l = n - r < INV_BS ? n - r : INV_BS;
            MG_TRY(launch_rows<true>(h, r + l, INV_BS, l, LU + r + (size_t)r * n, n, X + (size_t)r * n, n));
            if (r + INV_BS < n)
                MG_TRY(dgemm_launch(h, 0, 0, r + l, n - r - INV_BS, l, -1.0, X + (size_t)r * n, n,
                                    LU + r + (size_t)(r + INV_BS) * n, n, 1.0, X + (size_t)(r + INV_BS) * n, n, 0));
        }
        for (int r = ((n - 1) / INV_BS) * INV_BS; r >= 0; r -= INV_BS) {
            const int l = n - r < INV_BS ? n - r : INV_BS;
            MG_TRY(launch_rows<false>(h, n, INV_BS, l, LU + r + (size_t)r * n, n, X + (size_t)r * n, n));
            if (r > 0)
                MG_TRY(dgemm_launch(h, 0, 0, n, r, l, -1.0, X + (size_t)r * n, n, LU + r, n, 1.0, X, n, 0));
        }
    }
    const size_t total = (size_t)n * n;
    int blocks = (int)((total + 255) / 256);
    if (blocks > h->num_sms * 8) blocks = h->num_sms * 8;
    inv_permute_cols_kernel<<<blocks, 256, 0, h->stream>>>(n, pos, X, n, Ainv, ldinv);
    return post_launch(h, "inv_permute_cols_kernel");
}

}  // namespace mg

extern "C" mg_status_t mg_dinv(mg_handle_t h, int n, const double* A, int lda, double* Ainv, int ldinv, int* info) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || lda < (n > 1 ? n : 1) || ldinv < (n > 1 ? n : 1) || (n && (!A || !Ainv)))
        return mg::fail(h, MG_ERR_ARG, "mg_dinv: bad arguments");
    if (info) *info = 0;
    if (n == 0) return MG_OK;
    // Inv takes A by value (LU/__Inv.h:212): factor a copy.
    const size_t abytes = mg::align_up((size_t)n * n * sizeof(double), 256);
    const size_t pbytes = mg::align_up((size_t)n * sizeof(int), 256);
    const size_t base = mg::align_up(mg::dgetrf_ws_bytes(h->num_sms), 256);
    MG_TRY(mg::ensure_ws(h, base + 2 * abytes + pbytes));
    double* LU = (double*)((char*)h->ws + base);
    double* X = (double*)((char*)h->ws + base + abytes);
    int* pos = (int*)((char*)h->ws + base + 2 * abytes);
    MG_CHECK_CUDA(h, cudaMemcpy2DAsync(LU, (size_t)n * sizeof(double), A, (size_t)lda * sizeof(double),
                                       (size_t)n * sizeof(double), n, cudaMemcpyDeviceToDevice, h->stream));
    const mg_status_t s = mg::dgetrf_impl(h, n, n, LU, n, pos, info);
    if (s != MG_OK && s != MG_SINGULAR) return s;
    // Mat does not check for singularity: the inverse is formed regardless
    MG_TRY(mg::dinv_from_lu(h, n, LU, pos, X, Ainv, ldinv));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    return s;
}
