// FP64 peak microbenchmarks (the FP64 denominators of the roofline).
//
// The measured-peak file of the pool lists only HBM copy bandwidth and the
// BF16 tensor rate; the FP64 rates of GB300 are measured here: one kernel of
// independent FMA chains (DFMA pipe) and one of independent m16n8k4 f64 MMAs
// (DMMA pipe), both sized to fill every SM, timed with CUDA events.
#include "mg_internal.cuh"

namespace {

constexpr int PEAK_ITERS = 4096;

__global__ void __launch_bounds__(256) dfma_peak_kernel(double seed, double* out) {
    double a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = seed + threadIdx.x * 1e-3 + i;
    const double x = 1.0 + 1e-12, y = 1e-15;
    for (int it = 0; it < PEAK_ITERS; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = fma(a[i], x, y);
    }
    double s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i];
    if (s == 12345.678) out[threadIdx.x] = s;  // never true; keeps the loop alive
}

__global__ void __launch_bounds__(256) dmma_peak_kernel(double seed, double* out) {
    double c[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int r = 0; r < 4; ++r) c[i][r] = 0.0;
    const double a0 = seed + threadIdx.x * 1e-3, a1 = a0 + 1.0, b0 = 1e-3;
    for (int it = 0; it < PEAK_ITERS / 4; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i)
            asm volatile(
                "mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, "
                "{%0,%1,%2,%3};\n"
                : "+d"(c[i][0]), "+d"(c[i][1]), "+d"(c[i][2]), "+d"(c[i][3])
                : "d"(a0), "d"(a1), "d"(b0));
    }
    double s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += c[i][0] + c[i][1] + c[i][2] + c[i][3];
    if (s == 12345.678) out[threadIdx.x] = s;
}

}  // namespace

extern "C" mg_status_t mg_measure_fp64_peaks(mg_handle_t h, double* dfma_tflops, double* dmma_tflops) {
    if (!h || !dfma_tflops || !dmma_tflops) return MG_ERR_ARG;
    MG_TRY(mg::ensure_ws(h, 256 * sizeof(double)));
    double* out = (double*)h->ws;
    cudaEvent_t e0, e1;
    MG_CHECK_CUDA(h, cudaEventCreate(&e0));
    MG_CHECK_CUDA(h, cudaEventCreate(&e1));
    const int blocks = h->num_sms * 4, threads = 256;
    float best_f = 1e30f, best_m = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        float ms = 0;
        cudaEventRecord(e0, h->stream);
        dfma_peak_kernel<<<blocks, threads, 0, h->stream>>>(1.0, out);
        cudaEventRecord(e1, h->stream);
        MG_TRY(mg::post_launch(h, "dfma_peak_kernel"));
        MG_CHECK_CUDA(h, cudaEventSynchronize(e1));
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best_f) best_f = ms;
        cudaEventRecord(e0, h->stream);
        dmma_peak_kernel<<<blocks, threads, 0, h->stream>>>(1.0, out);
        cudaEventRecord(e1, h->stream);
        MG_TRY(mg::post_launch(h, "dmma_peak_kernel"));
        MG_CHECK_CUDA(h, cudaEventSynchronize(e1));
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best_m) best_m = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double threads_total = (double)blocks * threads;
    const double fma_flops = threads_total * PEAK_ITERS * 8 * 2.0;
    const double warps = threads_total / 32.0;
    const double mma_flops = warps * (PEAK_ITERS / 4) * 8 * (16.0 * 8 * 4 * 2);
    *dfma_tflops = fma_flops / (best_f * 1e-3) / 1e12;
    *dmma_tflops = mma_flops / (best_m * 1e-3) / 1e12;
    return MG_OK;
}
