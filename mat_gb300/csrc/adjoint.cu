// Reverse-mode (adjoint) kernels: Cholesky, triangular solve, log-determinant,
// and the Gaussian-process loss built from them.  Mat has no derivatives;
// these are the backward calls of its LLT / Solve_direct_XLT / Det family.
//
// Cholesky backward: the blocked reverse-mode recurrence of I. Murray,
// "Differentiation of the Cholesky decomposition" (2016), in place on Abar
// (which enters holding Lbar, lower triangle):
//   for each block column j (last to first), with R = L[j, :j], D = L[j, j],
//   B = L[below, :j], C = L[below, j] and the same blocks of Abar:
//     Cbar <- Cbar D^{-1};  Bbar -= Cbar R;  Dbar -= tril(Cbar^T C);
//     Dbar <- Phi(D^{-T} (P + P^T) D^{-1}),  P = Phi(D^T Dbar);
//     Rbar -= Cbar^T B + (Dbar + Dbar^T) R
// where Phi takes the lower triangle with the diagonal halved.  The result is
// the gradient with respect to the lower triangle of A (the part a Cholesky
// reads); mg_dpotrf_backward returns its symmetric form
// (Abar + Abar^T)/2 off the diagonal.  Only L is read: no intermediate of the
// forward pass is stored, every block of L is re-read where it is needed.
#include <cmath>

#include "mg_internal.cuh"

namespace {

constexpr int ADJ_BS = 48;

// X (rows x k) := X D^{-1}, D lower (k x k, k <= 48), one thread per row:
// x_q = (c_q - sum_{p>q} x_p D(p,q)) / D(q,q) for q = k-1 .. 0.
template <typename T>
__global__ void trsm_right_lower_kernel(const T* __restrict__ D, int ldd, T* __restrict__ X, int ldx,
                                        int rows, int k) {
    __shared__ T sd[ADJ_BS * ADJ_BS];
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) sd[e] = D[(e % k) + (size_t)(e / k) * ldd];
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    T x[ADJ_BS];
#pragma unroll
    for (int j = 0; j < ADJ_BS; ++j) x[j] = j < k ? X[r + (size_t)j * ldx] : T(0);
#pragma unroll
    for (int q = ADJ_BS - 1; q >= 0; --q) {
        if (q < k) {
            T c = x[q];
#pragma unroll
            for (int p = q + 1; p < ADJ_BS; ++p)
                if (p < k) c = fma(-x[p], sd[p + q * k], c);
            x[q] = c / sd[q + q * k];
        }
    }
#pragma unroll
    for (int j = 0; j < ADJ_BS; ++j)
        if (j < k) X[r + (size_t)j * ldx] = x[j];
}

// Dbar <- Phi(D^{-T} (P + P^T) D^{-1}) with P = Phi(D^T tril(Dbar)), one CTA (k <= 48).
template <typename T>
__global__ void chol_block_rev_kernel(const T* __restrict__ D, int ldd, T* __restrict__ Db, int lddb, int k) {
    __shared__ T sd[ADJ_BS * ADJ_BS];  // D (lower)
    __shared__ T sb[ADJ_BS * ADJ_BS];  // Dbar (lower) -> P -> S
    __shared__ T st[ADJ_BS * ADJ_BS];  // scratch
    const int t = threadIdx.x;
    for (int e = t; e < k * k; e += blockDim.x) {
        const int r = e % k, c = e / k;
        sd[e] = r >= c ? D[r + (size_t)c * ldd] : T(0);
        sb[e] = r >= c ? Db[r + (size_t)c * lddb] : T(0);
    }
    __syncthreads();
    // P = Phi(D^T Dbar): P(r,c) = sum_q D(q,r) Dbar(q,c), kept for r >= c, diagonal halved
    for (int e = t; e < k * k; e += blockDim.x) {
        const int r = e % k, c = e / k;
        T v = T(0);
        if (r >= c)
            for (int q = r; q < k; ++q) v = fma(sd[q + r * k], sb[q + c * k], v);
        st[e] = r > c ? v : (r == c ? T(0.5) * v : T(0));
    }
    __syncthreads();
    // M = P + P^T (symmetric)
    for (int e = t; e < k * k; e += blockDim.x) {
        const int r = e % k, c = e / k;
        sb[e] = st[e] + st[c + r * k];
    }
    __syncthreads();
    // Y = D^{-T} M: solve D^T Y = M column by column (thread per column)
    if (t < k) {
        T* y = sb + t * k;
        for (int i = k - 1; i >= 0; --i) {
            T v = y[i];
            for (int q = i + 1; q < k; ++q) v = fma(-sd[q + i * k], y[q], v);
            y[i] = v / sd[i + i * k];
        }
    }
    __syncthreads();
    // S = Y D^{-1}: solve S D = Y row by row (thread per row)
    if (t < k) {
        for (int q = k - 1; q >= 0; --q) {
            T v = sb[t + q * k];
            for (int p = q + 1; p < k; ++p) v = fma(-sb[t + p * k], sd[p + q * k], v);
            sb[t + q * k] = v / sd[q + q * k];
        }
    }
    __syncthreads();
    // Dbar = Phi(S) (S is already the symmetric combination)
    for (int e = t; e < k * k; e += blockDim.x) {
        const int r = e % k, c = e / k;
        if (r >= c) Db[r + (size_t)c * lddb] = r == c ? T(0.5) * sb[e] : sb[e];
    }
}

// E = Dbar + Dbar^T from the lower triangle of Dbar (k x k, ld k output).
template <typename T>
__global__ void sym_from_lower_kernel(const T* __restrict__ Db, int lddb, int k, T* __restrict__ E) {
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        const int r = e % k, c = e / k;
        const T a = r >= c ? Db[r + (size_t)c * lddb] : Db[c + (size_t)r * lddb];
        E[e] = r == c ? T(2) * a : a;
    }
}

// Symmetric gradient from the lower-triangle gradient: G(i,j) = Abar(i,j)/2 (i != j), Abar(i,i).
template <typename T>
__global__ void symmetrize_grad_kernel(const T* __restrict__ Ab, int ldab, int n, T* __restrict__ G, int ldg) {
    const size_t total = (size_t)n * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e % n), c = (int)(e / n);
        const T a = r >= c ? Ab[r + (size_t)c * ldab] : Ab[c + (size_t)r * ldab];
        G[r + (size_t)c * ldg] = r == c ? a : T(0.5) * a;
    }
}

// (sum in fp64 for either element type)
template <typename T>
__global__ void logdet_kernel(const T* __restrict__ L, int ldl, int n, double* __restrict__ out) {
    __shared__ double red[256];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += (double)log(L[i + (size_t)i * ldl]);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = 2.0 * red[0];
}

template <typename T>
__global__ void logdet_backward_kernel(const T* __restrict__ L, int ldl, int n, T gbar, T* __restrict__ Lb,
                                       int ldlb) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        Lb[i + (size_t)i * ldlb] += T(2) * gbar / L[i + (size_t)i * ldl];
}

// K(i,j) = sigma2 * exp(-|x_i - x_j|^2 / (2 ell^2)) + jitter * [i == j], points X (n x 3, column-major).
template <typename T>
__global__ void rbf_kernel(const T* __restrict__ X, int n, T ell, T sigma2, T jitter, T* __restrict__ K, int ldk) {
    const size_t total = (size_t)n * n;
    const T inv = T(1) / (T(2) * ell * ell);
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        T d2 = T(0);
        for (int q = 0; q < 3; ++q) {
            const T d = X[i + (size_t)q * n] - X[j + (size_t)q * n];
            d2 = fma(d, d, d2);
        }
        K[i + (size_t)j * ldk] = sigma2 * exp(-d2 * inv) + (i == j ? jitter : T(0));
    }
}

// sum_ij G(i,j) dK(i,j)/d ell with dK/d ell = sigma2 exp(-d2/(2 ell^2)) d2 / ell^3.
// (partial sums in fp64 for either element type)
template <typename T>
__global__ void rbf_ell_grad_kernel(const T* __restrict__ X, int n, T ell, T sigma2, const T* __restrict__ G, int ldg,
                                    double* __restrict__ partial) {
    __shared__ double red[256];
    const size_t total = (size_t)n * n;
    const T inv = T(1) / (T(2) * ell * ell), inv3 = T(1) / (ell * ell * ell);
    double s = 0.0;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        T d2 = T(0);
        for (int q = 0; q < 3; ++q) {
            const T d = X[i + (size_t)q * n] - X[j + (size_t)q * n];
            d2 = fma(d, d, d2);
        }
        s += (double)(G[i + (size_t)j * ldg] * sigma2 * exp(-d2 * inv) * d2 * inv3);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

template <typename T>
__global__ void dot_partial_kernel(const T* __restrict__ a, const T* __restrict__ b, int n, double* __restrict__ partial) {
    __shared__ double red[256];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        s = fma((double)a[i], (double)b[i], s);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

int gridn(mg_handle_t h, size_t total) {
    size_t g = (total + 255) / 256;
    const size_t cap = (size_t)h->num_sms * 8;
    return (int)(g < 1 ? 1 : g > cap ? cap : g);
}

}  // namespace

namespace mg {

// In place: Ab holds Lbar (lower) on entry and the lower-triangle gradient on exit.
template <typename T>
mg_status_t potrf_backward_lower(mg_handle_t h, int n, const T* L, int ldl, T* Ab, int ldab, T* E) {
    cudaStream_t st = h->stream;
    ProfScope prof(h, "chol_backward", 2.0 * n * (double)n * n / 3.0, 4.0 * sizeof(T) * n * (double)n);
    const int last = ((n - 1) / ADJ_BS) * ADJ_BS;
    for (int j0 = last; j0 >= 0; j0 -= ADJ_BS) {
        const int j1 = j0 + ADJ_BS < n ? j0 + ADJ_BS : n;
        const int b = j1 - j0, below = n - j1;
        const T* R = L + j0;                        // b x j0
        const T* D = L + j0 + (size_t)j0 * ldl;     // b x b
        const T* Bm = L + j1;                       // below x j0
        const T* Cm = L + j1 + (size_t)j0 * ldl;    // below x b
        T* Rb = Ab + j0;
        T* Db = Ab + j0 + (size_t)j0 * ldab;
        T* Bb = Ab + j1;
        T* Cb = Ab + j1 + (size_t)j0 * ldab;
        if (below > 0) {
            trsm_right_lower_kernel<T><<<(below + 127) / 128, 128, 0, st>>>(D, ldl, Cb, ldab, below, b);
            MG_TRY(post_launch(h, "trsm_right_lower_kernel"));
            if (j0 > 0) MG_TRY(gemm_of(h, 0, 0, below, j0, b, T(-1), Cb, ldab, R, ldl, T(1), Bb, ldab, 0));
            MG_TRY(gemm_of(h, 1, 0, b, b, below, T(-1), Cb, ldab, Cm, ldl, T(1), Db, ldab, 0));
        }
        chol_block_rev_kernel<T><<<1, 256, 0, st>>>(D, ldl, Db, ldab, b);
        MG_TRY(post_launch(h, "chol_block_rev_kernel"));
        if (j0 > 0) {
            if (below > 0) MG_TRY(gemm_of(h, 1, 0, b, j0, below, T(-1), Cb, ldab, Bm, ldl, T(1), Rb, ldab, 0));
            sym_from_lower_kernel<T><<<1, 256, 0, st>>>(Db, ldab, b, E);
            MG_TRY(post_launch(h, "sym_from_lower_kernel"));
            MG_TRY(gemm_of(h, 0, 0, b, j0, b, T(-1), E, b, R, ldl, T(1), Rb, ldab, 0));
        }
    }
    return MG_OK;
}

template <typename T>
mg_status_t potrf_backward(mg_handle_t h, int n, const T* L, int ldl, const T* Lbar, int ldlbar, T* Abar,
                           int ldabar) {
    if (n == 0) return MG_OK;
    const size_t nn = (size_t)n * n;
    MG_TRY(ensure_ws(h, nn * sizeof(T) + ADJ_BS * ADJ_BS * sizeof(T) + 1024));
    T* W = (T*)h->ws;
    T* E = W + nn;
    cudaStream_t st = h->stream;
    MG_CHECK_CUDA(h, cudaMemcpy2DAsync(W, (size_t)n * sizeof(T), Lbar, (size_t)ldlbar * sizeof(T),
                                       (size_t)n * sizeof(T), n, cudaMemcpyDeviceToDevice, st));
    MG_TRY(potrf_backward_lower<T>(h, n, L, ldl, W, n, E));
    symmetrize_grad_kernel<T><<<gridn(h, nn), 256, 0, st>>>(W, n, n, Abar, ldabar);
    return post_launch(h, "symmetrize_grad_kernel");
}

// GP negative log-likelihood (up to the constant): 0.5 y^T K^{-1} y + 0.5 logdet K,
// K = RBF(X; ell, sigma2) + jitter I; gradient with respect to K (symmetric,
// optional) and ell.  Forward: Cholesky, z = L^{-1} y, logdet; backward:
// Lbar = -tril(alpha z^T) (alpha = L^{-T} z) + diag(1/L_ii), then Kbar by the
// blocked Cholesky adjoint.  All matrix work in T; the scalar sums (z.z,
// logdet, dloss/dell) in fp64.
template <typename T>
mg_status_t gp_loss_grad(mg_handle_t h, int n, const T* X, T ell, T sigma2, T jitter, const T* y, double* host_loss,
                         double* host_dell, T* Kbar, int ldkbar) {
    const size_t nn = (size_t)n * n;
    const int nparts = h->num_sms * 4;
    MG_TRY(ensure_ws(h, (3 * nn + 3 * (size_t)n + ADJ_BS * ADJ_BS) * sizeof(T) + (2 * (size_t)nparts + 64) * 8 +
                            4096));
    MG_TRY(ensure_hws(h, (size_t)(2 * nparts + 8) * 8));
    T* L = (T*)h->ws;
    T* Lb = L + nn;
    T* G = Lb + nn;
    T* z = G + nn;
    T* a = z + n;
    T* E = a + n;
    double* part = (double*)align_up((size_t)(E + ADJ_BS * ADJ_BS), 256);  // [nparts] z.z, [nparts] dloss/dell
    double* d1 = part + 2 * nparts;                                          // logdet
    cudaStream_t st = h->stream;
    rbf_kernel<T><<<gridn(h, nn), 256, 0, st>>>(X, n, ell, sigma2, jitter, L, n);
    MG_TRY(post_launch(h, "rbf_kernel"));
    int info = 0;
    mg_status_t s = potrf_impl<T>(h, n, L, n, &info);
    if (s != MG_OK) return s;
    // z = L^{-1} y, alpha = L^{-T} z
    MG_CHECK_CUDA(h, cudaMemcpyAsync(z, y, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    MG_TRY(chol_lower_solve<T>(h, n, 1, L, n, z, n));
    MG_CHECK_CUDA(h, cudaMemcpyAsync(a, z, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    MG_TRY(chol_lower_t_solve<T>(h, n, 1, L, n, a, n));
    dot_partial_kernel<T><<<nparts, 256, 0, st>>>(z, z, n, part);
    MG_TRY(post_launch(h, "dot_partial_kernel"));
    logdet_kernel<T><<<1, 256, 0, st>>>(L, n, n, d1);
    MG_TRY(post_launch(h, "logdet_kernel"));
    // Lbar = -tril(alpha z^T) + diag(1 / L_ii)   (0.5 * 2 from the logdet term)
    MG_CHECK_CUDA(h, cudaMemsetAsync(Lb, 0, nn * sizeof(T), st));
    MG_TRY(gemm_of(h, 0, 1, n, n, 1, T(-1), a, n, z, n, T(1), Lb, n, 1));
    logdet_backward_kernel<T><<<gridn(h, n), 256, 0, st>>>(L, n, n, T(0.5), Lb, n);
    MG_TRY(post_launch(h, "logdet_backward_kernel"));
    MG_TRY(potrf_backward_lower<T>(h, n, L, n, Lb, n, E));
    symmetrize_grad_kernel<T><<<gridn(h, nn), 256, 0, st>>>(Lb, n, n, G, n);
    MG_TRY(post_launch(h, "symmetrize_grad_kernel"));
    rbf_ell_grad_kernel<T><<<nparts, 256, 0, st>>>(X, n, ell, sigma2, G, n, part + nparts);
    MG_TRY(post_launch(h, "rbf_ell_grad_kernel"));
    if (Kbar)
        MG_CHECK_CUDA(h, cudaMemcpy2DAsync(Kbar, (size_t)ldkbar * sizeof(T), G, (size_t)n * sizeof(T),
                                           (size_t)n * sizeof(T), n, cudaMemcpyDeviceToDevice, st));
    double* hp = (double*)h->hws;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(hp, part, (size_t)(2 * nparts + 1) * 8, cudaMemcpyDeviceToHost, st));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
    double zz = 0.0, dl = 0.0;
    for (int i = 0; i < nparts; ++i) {
        zz += hp[i];
        dl += hp[nparts + i];
    }
    *host_loss = 0.5 * zz + 0.5 * hp[2 * nparts];
    *host_dell = dl;
    return MG_OK;
}

}  // namespace mg

extern "C" {

mg_status_t mg_dpotrf_backward(mg_handle_t h, int n, const double* L, int ldl, const double* Lbar, int ldlbar,
                               double* Abar, int ldabar) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || ldl < (n > 1 ? n : 1) || ldlbar < (n > 1 ? n : 1) || ldabar < (n > 1 ? n : 1) ||
        (n && (!L || !Lbar || !Abar)))
        return mg::fail(h, MG_ERR_ARG, "mg_dpotrf_backward: bad arguments");
    return mg::potrf_backward<double>(h, n, L, ldl, Lbar, ldlbar, Abar, ldabar);
}

mg_status_t mg_spotrf_backward(mg_handle_t h, int n, const float* L, int ldl, const float* Lbar, int ldlbar,
                               float* Abar, int ldabar) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || ldl < (n > 1 ? n : 1) || ldlbar < (n > 1 ? n : 1) || ldabar < (n > 1 ? n : 1) ||
        (n && (!L || !Lbar || !Abar)))
        return mg::fail(h, MG_ERR_ARG, "mg_spotrf_backward: bad arguments");
    return mg::potrf_backward<float>(h, n, L, ldl, Lbar, ldlbar, Abar, ldabar);
}

mg_status_t mg_dtrsm_backward(mg_handle_t h, int trans, int n, int nrhs, const double* L, int ldl, const double* X,
                              int ldx, const double* Xbar, int ldxbar, double* Bbar, int ldbbar, double* Lbar,
                              int ldlbar) {
    if (!h) return MG_ERR_ARG;
    if (n < 0 || nrhs < 0 || ldl < (n > 1 ? n : 1) || ldx < (n > 1 ? n : 1) || ldxbar < (n > 1 ? n : 1) ||
        ldbbar < (n > 1 ? n : 1) || ldlbar < (n > 1 ? n : 1) ||
        ((size_t)n * nrhs && (!L || !X || !Xbar || !Bbar || !Lbar)))
        return mg::fail(h, MG_ERR_ARG, "mg_dtrsm_backward: bad arguments");
    if ((size_t)n * nrhs == 0) return MG_OK;
    cudaStream_t st = h->stream;
    MG_CHECK_CUDA(h, cudaMemcpy2DAsync(Bbar, (size_t)ldbbar * 8, Xbar, (size_t)ldxbar * 8, (size_t)n * 8, nrhs,
                                       cudaMemcpyDeviceToDevice, st));
    if (!trans) {
        // X = L^{-1} B: Bbar = L^{-T} Xbar, Lbar -= tril(Bbar X^T)
        MG_TRY(mg::chol_lower_t_solve<double>(h, n, nrhs, L, ldl, Bbar, ldbbar));
        return mg::dgemm_launch(h, 0, 1, n, n, nrhs, -1.0, Bbar, ldbbar, X, ldx, 1.0, Lbar, ldlbar, 1);
    }
    // X = L^{-T} B: Bbar = L^{-1} Xbar, Lbar -= tril(X Bbar^T)
    MG_TRY(mg::chol_lower_solve<double>(h, n, nrhs, L, ldl, Bbar, ldbbar));
    return mg::dgemm_launch(h, 0, 1, n, n, nrhs, -1.0, X, ldx, Bbar, ldbbar, 1.0, Lbar, ldlbar, 1);
}

mg_status_t mg_dlogdet_chol(mg_handle_t h, int n, const double* L, int ldl, double* host_out) {
    if (!h || n < 0 || ldl < (n > 1 ? n : 1) || !host_out || (n && !L)) return MG_ERR_ARG;
    MG_TRY(mg::ensure_hws(h, 64));
    double* d = (double*)(h->status + 16);
    logdet_kernel<double><<<1, 256, 0, h->stream>>>(L, ldl, n, d);
    MG_TRY(mg::post_launch(h, "logdet_kernel"));
    MG_CHECK_CUDA(h, cudaMemcpyAsync(h->hws, d, 8, cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    *host_out = *(double*)h->hws;
    return MG_OK;
}

mg_status_t mg_dlogdet_chol_backward(mg_handle_t h, int n, const double* L, int ldl, double gbar, double* Lbar,
                                     int ldlbar) {
    if (!h || n < 0 || ldl < (n > 1 ? n : 1) || ldlbar < (n > 1 ? n : 1) || (n && (!L || !Lbar))) return MG_ERR_ARG;
    if (n == 0) return MG_OK;
    logdet_backward_kernel<double><<<gridn(h, n), 256, 0, h->stream>>>(L, ldl, n, gbar, Lbar, ldlbar);
    return mg::post_launch(h, "logdet_backward_kernel");
}

mg_status_t mg_gen_rbf_kernel(mg_handle_t h, int n, const double* X, double ell, double sigma2, double jitter,
                              double* K, int ldk) {
    if (!h || n < 0 || ldk < (n > 1 ? n : 1) || (n && (!X || !K)) || !(ell > 0)) return MG_ERR_ARG;
    if (n == 0) return MG_OK;
    rbf_kernel<double><<<gridn(h, (size_t)n * n), 256, 0, h->stream>>>(X, n, ell, sigma2, jitter, K, ldk);
    return mg::post_launch(h, "rbf_kernel");
}

mg_status_t mg_gp_loss_grad(mg_handle_t h, int n, const double* X, double ell, double sigma2, double jitter,
                            const double* y, double* host_loss, double* host_dell, double* Kbar, int ldkbar) {
    if (!h || n <= 0 || !X || !y || !host_loss || !host_dell || !(ell > 0) || (Kbar && ldkbar < n))
        return MG_ERR_ARG;
    return mg::gp_loss_grad<double>(h, n, X, ell, sigma2, jitter, y, host_loss, host_dell, Kbar, ldkbar);
}

mg_status_t mg_sgp_loss_grad(mg_handle_t h, int n, const float* X, float ell, float sigma2, float jitter,
                             const float* y, double* host_loss, double* host_dell, float* Kbar, int ldkbar) {
    if (!h || n <= 0 || !X || !y || !host_loss || !host_dell || !(ell > 0) || (Kbar && ldkbar < n))
        return MG_ERR_ARG;
    return mg::gp_loss_grad<float>(h, n, X, ell, sigma2, jitter, y, host_loss, host_dell, Kbar, ldkbar);
}

}  // extern "C"
