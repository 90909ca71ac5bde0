// Bounded grid-wide barrier for cooperative (co-resident) launches.
//
// The counter is zeroed by the host (cudaMemsetAsync) before each launch and
// only grows; the k-th barrier waits for k * gridDim.x arrivals.  Every wait
// is bounded: after kSpinLimit polls (~1-2 s with the back-off) the CTA
// records MG_TIMEOUT in the error word and the caller returns, so a lost CTA
// can never hang the GPU.
#pragma once
#include <cuda_runtime.h>

namespace mg {

constexpr unsigned kSpinLimit = 1u << 24;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// The arrival: a release-ordered add at GPU scope.  The CTA barrier before it
// orders the other threads' writes before this thread's, and the release
// carries them (cumulativity) to whoever acquires the counter.
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// A flag store with release semantics at GPU scope (after a CTA barrier it
// publishes the CTA's prior writes to whoever acquires the flag).
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// Returns false (in every thread of the CTA) if the wait timed out.  `limit`
// is the poll budget (the self-test lowers it to make a wait run out).
__device__ __forceinline__ bool grid_barrier(unsigned* counter, unsigned target, int* err,
                                             unsigned limit = kSpinLimit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        if (gridDim.x > 1) {
            red_release_add(counter, 1u);
            unsigned spins = 0;
            while (ld_acquire_u32(counter) < target) {
                if (++spins > limit) {
                    atomicExch(err, 8 /* MG_TIMEOUT */);
                    ok = 0;
                    break;
                }
                __nanosleep(spins < 64 ? 20 : 100);
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Split form of the barrier: arrive() publishes this CTA's prior writes and
// counts it in; wait() blocks until `target` arrivals (bounded).  Work placed
// between the two overlaps the other CTAs' arrival.
__device__ __forceinline__ void grid_arrive(unsigned* counter) {
    __syncthreads();
    if (threadIdx.x == 0 && gridDim.x > 1) red_release_add(counter, 1u);
}

__device__ __forceinline__ bool grid_wait(unsigned* counter, unsigned target, int* err) {
    __shared__ int s_ok2;
    if (threadIdx.x == 0) {
        int ok = 1;
        if (gridDim.x > 1) {
            unsigned spins = 0;
            while (ld_acquire_u32(counter) < target) {
                if (++spins > kSpinLimit) {
                    atomicExch(err, 8 /* MG_TIMEOUT */);
                    ok = 0;
                    break;
                }
                __nanosleep(spins < 64 ? 20 : 100);
            }
        }
        s_ok2 = ok;
    }
    __syncthreads();
    return s_ok2 != 0;
}

}  // namespace mg
