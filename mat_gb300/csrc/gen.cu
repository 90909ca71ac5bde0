// Seeded benchmark-input generators built from the library's own kernels.
//
// mg_gen_svd_matrix: A = Q1 diag(sigma) Q2 (sigma_r = sigma_min^(r/(n-1)),
// mgrng::geometric_at), each Q a product of `nrefl`
// Householder reflectors H = I - tau v v^T (tau = 2 / v^T v, v iid N(0,1)),
// applied in compact WY form Q = I - V T V^T (T upper triangular, the
// forward recurrence of the block reflector) with three FP64 GEMMs per side.
// mg_gen_spd_gram: S = G G^T / n + I.
#include <cmath>
#include <vector>

#include "mg_internal.cuh"
#include "rng.cuh"

namespace {

__global__ void diag_fill_kernel(double* A, int lda, int n, double sigma_min) {
    const size_t total = (size_t)n * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t r = e % n, c = e / n;
        A[r + c * lda] = r == c ? mgrng::geometric_at((int)r, n, sigma_min) : 0.0;
    }
}

__global__ void add_identity_kernel(double* A, int lda, int n, double v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) A[i + (size_t)i * lda] += v;
}

// T (k x k, upper) of Q = H_0 ... H_{k-1} = I - V T V^T from G = V^T V.
void build_T(int k, const std::vector<double>& G, std::vector<double>& T) {
    T.assign((size_t)k * k, 0.0);
    for (int i = 0; i < k; ++i) {
        const double tau = 2.0 / G[i + (size_t)i * k];
        // T[0:i, i] = -tau * T[0:i, 0:i] * G[0:i, i]
        for (int r = 0; r < i; ++r) {
            double s = 0.0;
            for (int c = r; c < i; ++c) s += T[r + (size_t)c * k] * G[c + (size_t)i * k];
            T[r + (size_t)i * k] = -tau * s;
        }
        T[i + (size_t)i * k] = tau;
    }
}

}  // namespace

extern "C" mg_status_t mg_gen_svd_matrix(mg_handle_t h, int n, double* A, int lda, uint64_t seed, int nrefl,
                                         double sigma_min) {
    if (!h || n < 0 || lda < (n > 1 ? n : 1) || nrefl < 0 || (n && !A) || !(sigma_min > 0.0 && sigma_min <= 1.0))
        return MG_ERR_ARG;
    if (n == 0) return MG_OK;
    const int k = nrefl;
    // workspace: V1, V2 (n x k), W, W2 (k x n), G, T (k x k)
    const size_t nk = (size_t)n * (k > 0 ? k : 1), kk = (size_t)(k > 0 ? k : 1) * (k > 0 ? k : 1);
    MG_TRY(mg::ensure_ws(h, (4 * nk + 2 * kk) * sizeof(double) + 4096));
    double* V1 = (double*)h->ws;
    double* V2 = V1 + nk;
    double* W = V2 + nk;
    double* W2 = W + nk;
    double* G = W2 + nk;
    double* T = G + kk;
    cudaStream_t st = h->stream;
    diag_fill_kernel<<<h->num_sms * 8, 256, 0, st>>>(A, lda, n, sigma_min);
    MG_TRY(mg::post_launch(h, "diag_fill_kernel"));
    if (k == 0) return MG_OK;
    MG_TRY(mg_fill_normal(h, V1, n, k, n, seed * 2 + 1, 1));
    MG_TRY(mg_fill_normal(h, V2, n, k, n, seed * 2 + 2, 1));
    std::vector<double> hG((size_t)k * k), hT;
    for (int side = 0; side < 2; ++side) {
        double* V = side == 0 ? V1 : V2;
        MG_TRY(mg::dgemm_launch(h, 1, 0, k, k, n, 1.0, V, n, V, n, 0.0, G, k, 0));
        MG_CHECK_CUDA(h, cudaMemcpyAsync(hG.data(), G, kk * sizeof(double), cudaMemcpyDeviceToHost, st));
        MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
        build_T(k, hG, hT);
        MG_CHECK_CUDA(h, cudaMemcpyAsync(T, hT.data(), kk * sizeof(double), cudaMemcpyHostToDevice, st));
        if (side == 0) {
            // A := Q1 A = A - V (T (V^T A))
            MG_TRY(mg::dgemm_launch(h, 1, 0, k, n, n, 1.0, V, n, A, lda, 0.0, W, k, 0));
            MG_TRY(mg::dgemm_launch(h, 0, 0, k, n, k, 1.0, T, k, W, k, 0.0, W2, k, 0));
            MG_TRY(mg::dgemm_launch(h, 0, 0, n, n, k, -1.0, V, n, W2, k, 1.0, A, lda, 0));
        } else {
            // A := A Q2 = A - ((A V) T) V^T
            MG_TRY(mg::dgemm_launch(h, 0, 0, n, k, n, 1.0, A, lda, V, n, 0.0, W, n, 0));
            MG_TRY(mg::dgemm_launch(h, 0, 0, n, k, k, 1.0, W, n, T, k, 0.0, W2, n, 0));
            MG_TRY(mg::dgemm_launch(h, 0, 1, n, n, k, -1.0, W2, n, V, n, 1.0, A, lda, 0));
        }
    }
    MG_CHECK_CUDA(h, cudaStreamSynchronize(st));
    return MG_OK;
}

extern "C" mg_status_t mg_gen_spd_gram(mg_handle_t h, int n, double* S, int lds, uint64_t seed) {
    if (!h || n < 0 || lds < (n > 1 ? n : 1) || (n && !S)) return MG_ERR_ARG;
    if (n == 0) return MG_OK;
    MG_TRY(mg::ensure_ws(h, (size_t)n * n * sizeof(double) + 4096));
    double* Gm = (double*)h->ws;
    MG_TRY(mg_fill_normal(h, Gm, n, n, n, seed, 1));
    MG_TRY(mg::dgemm_launch(h, 0, 1, n, n, n, 1.0 / n, Gm, n, Gm, n, 0.0, S, lds, 0));
    add_identity_kernel<<<(n + 255) / 256, 256, 0, h->stream>>>(S, lds, n, 1.0);
    MG_TRY(mg::post_launch(h, "add_identity_kernel"));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    return MG_OK;
}
