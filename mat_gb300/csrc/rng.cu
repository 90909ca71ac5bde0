// Seeded matrix generators (host and device, bit-identical).
#include "mg_internal.cuh"
#include "rng.cuh"

namespace {

__global__ void fill_kernel(double* __restrict__ A, int rows, int cols, int ld, uint64_t key,
                            double lo, double hi, int rowmajor, int normal) {
    const size_t total = (size_t)rows * cols;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t r = e % rows, c = e / rows;
        const uint64_t idx = rowmajor ? (uint64_t)r * cols + c : (uint64_t)e;
        A[r + c * (size_t)ld] = normal ? mgrng::normal_at(key, idx) : mgrng::uniform_at(key, idx, lo, hi);
    }
}

void host_fill(double* A, int rows, int cols, int ld, uint64_t key, double lo, double hi, int rowmajor,
               int normal) {
    for (int c = 0; c < cols; ++c)
        for (int r = 0; r < rows; ++r) {
            const uint64_t idx = rowmajor ? (uint64_t)r * cols + c : (uint64_t)r + (uint64_t)c * rows;
            A[r + c * (size_t)ld] = normal ? mgrng::normal_at(key, idx) : mgrng::uniform_at(key, idx, lo, hi);
        }
}

mg_status_t dev_fill(mg_handle_t h, double* A, int rows, int cols, int ld, uint64_t key, double lo, double hi,
                     int rowmajor, int normal) {
    if (!h || rows < 0 || cols < 0 || ld < (rows > 1 ? rows : 1) || (rows * (size_t)cols && !A))
        return MG_ERR_ARG;
    if ((size_t)rows * cols == 0) return MG_OK;
    const int threads = 256;
    const size_t total = (size_t)rows * cols;
    size_t blocks = (total + threads - 1) / threads;
    const size_t cap = (size_t)h->num_sms * 8;
    if (blocks > cap) blocks = cap;
    fill_kernel<<<(unsigned)blocks, threads, 0, h->stream>>>(A, rows, cols, ld, key, lo, hi, rowmajor, normal);
    return mg::post_launch(h, "fill_kernel");
}

}  // namespace

extern "C" {

void mg_host_fill_uniform(double* A, int rows, int cols, int ld, uint64_t seed, double lo, double hi,
                          int rowmajor_stream) {
    if (!A || rows <= 0 || cols <= 0) return;
    host_fill(A, rows, cols, ld, mgrng::stream_key(seed, mgrng::kSaltUniform), lo, hi, rowmajor_stream, 0);
}

void mg_host_fill_normal(double* A, int rows, int cols, int ld, uint64_t seed, int rowmajor_stream) {
    if (!A || rows <= 0 || cols <= 0) return;
    host_fill(A, rows, cols, ld, mgrng::stream_key(seed, mgrng::kSaltNormal), 0, 0, rowmajor_stream, 1);
}

mg_status_t mg_fill_uniform(mg_handle_t h, double* A, int rows, int cols, int ld, uint64_t seed, double lo,
                            double hi, int rowmajor_stream) {
    return dev_fill(h, A, rows, cols, ld, mgrng::stream_key(seed, mgrng::kSaltUniform), lo, hi, rowmajor_stream,
                    0);
}

mg_status_t mg_fill_normal(mg_handle_t h, double* A, int rows, int cols, int ld, uint64_t seed,
                           int rowmajor_stream) {
    return dev_fill(h, A, rows, cols, ld, mgrng::stream_key(seed, mgrng::kSaltNormal), 0, 0, rowmajor_stream, 1);
}

}  // extern "C"
