// Self-test of the bounded device-side waits.
//
// Every wait inside the library's kernels (the grid barriers of the
// cooperative panels, the mbarrier waits of the tensor-core GEMM and the
// cluster panel) gives up after a poll budget, records MG_TIMEOUT in an error
// word and lets the kernel return, so that a lost CTA can never hang the GPU
// and the host reports the failure.  Mat has no counterpart (no error
// channel at all: a zero pivot is a silent break, Mat-8.3.1/LU/__PLU.h:68-71).
//
// mg_selftest_bounded_wait makes one such wait run out on purpose, through
// the same barrier code with a small poll budget: nothing is left running,
// nothing traps, and the context stays usable for the next call.
//   kind 0: grid barrier of a cooperative launch of 8 CTAs; CTA `withhold`
//           returns without arriving (withhold < 0: every CTA arrives).
//   kind 1: mbarrier wait in one CTA on a phase that nothing completes
//           (withhold < 0: the waiting thread arrives itself first).
#include "grid_sync.cuh"
#include "mg_internal.cuh"
#include "tc_common.cuh"

namespace {

constexpr int kTestCtas = 8;

__global__ void barrier_selftest_kernel(unsigned* counter, int* err, int withhold, unsigned limit) {
    if ((int)blockIdx.x == withhold) return;  // this CTA never arrives
    mg::grid_barrier(counter, gridDim.x, err, limit);
}

__global__ void mbar_selftest_kernel(int* err, int withhold, unsigned limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (withhold < 0) tc::mbar_arrive(&bar);
        if (!tc::mbar_wait(&bar, 0, limit)) atomicExch(err, 8 /* MG_TIMEOUT */);
    }
}

}  // namespace

extern "C" mg_status_t mg_selftest_bounded_wait(mg_handle_t h, int kind, int withhold, unsigned poll_limit) {
    if (!h || kind < 0 || kind > 1 || withhold >= kTestCtas || poll_limit == 0 || poll_limit > mg::kSpinLimit)
        return MG_ERR_ARG;
    MG_TRY(mg::ensure_ws(h, 256));
    unsigned* counter = (unsigned*)h->ws;
    int* err = (int*)((char*)h->ws + 128);
    MG_CHECK_CUDA(h, cudaMemsetAsync(h->ws, 0, 256, h->stream));
    if (kind == 0) {
        void* args[] = {&counter, &err, &withhold, &poll_limit};
        const cudaError_t e = cudaLaunchCooperativeKernel((const void*)barrier_selftest_kernel, dim3(kTestCtas),
                                                          dim3(128), args, 0, h->stream);
        if (e != cudaSuccess) return mg::cuda_fail(h, e, "barrier_selftest_kernel launch");
        h->launches++;
    } else {
        mbar_selftest_kernel<<<1, 32, 0, h->stream>>>(err, withhold, poll_limit);
        MG_TRY(mg::post_launch(h, "mbar_selftest_kernel"));
    }
    int herr = 0;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    if (herr) return mg::fail(h, MG_TIMEOUT, "self-test: the %s wait ran out after %u polls",
                              kind == 0 ? "grid barrier" : "mbarrier", poll_limit);
    return MG_OK;
}
