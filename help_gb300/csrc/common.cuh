// Device-side building blocks shared by the kernels: bounded grid barrier,
// deterministic block reductions, cache-hinted loads.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define HELP_DEVINL __device__ __forceinline__

namespace help {

constexpr int kWarp = 32;

// Wall-clock nanoseconds from the GPU global timer.
HELP_DEVINL uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Read-only (for the whole kernel) data: non-coherent path, evict-first in L2
// so the streamed matrix does not push the reused vectors out of L2.
template <class T>
HELP_DEVINL T ld_stream(const T* p) {
    return __ldcs(p);
}
template <class T>
HELP_DEVINL T ld_ro(const T* p) {
    return __ldg(p);
}

// Status codes a kernel can leave in its status word (mirror HELP_E_*).
constexpr int kStatusOk = 0;
constexpr int kStatusTimeout = -5;
constexpr int kStatusNumeric = -4;

// Grid-wide barrier for cooperative launches (all blocks co-resident).
// Generation-counting: the last block to arrive resets the counter and bumps
// the generation; the others spin on the generation with a wall-clock limit.
// On timeout, or when another block already gave up, the barrier returns
// false and the caller must return from the kernel.  The limit bounds every
// wait, so a faulty phase ends the kernel with an error status instead of a
// hang.
struct GridBarrier {
    unsigned int* count;
    unsigned int* gen;
    int* status;  // 0 ok, < 0 error (set once)
};

constexpr uint64_t kBarrierTimeoutNs = 2000000000ull;  // 2 s

HELP_DEVINL bool grid_sync(const GridBarrier& b) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* vgen = b.gen;
        volatile int* vstat = b.status;
        const unsigned int g = *vgen;
        __threadfence();
        const unsigned int arrived = atomicAdd(b.count, 1u) + 1u;
        int ok = 1;
        if (arrived == gridDim.x) {
            atomicExch(b.count, 0u);
            __threadfence();
            atomicAdd(b.gen, 1u);
        } else {
            const uint64_t t0 = globaltimer_ns();
            while (*vgen == g) {
                if (*vstat != 0) {
                    ok = 0;
                    break;
                }
                if (globaltimer_ns() - t0 > kBarrierTimeoutNs) {
                    atomicCAS(b.status, 0, kStatusTimeout);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        if (*vstat != 0) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Deterministic block-wide sum (fixed tree for a fixed blockDim).  `red` must
// hold blockDim.x / 32 doubles.  Result valid in every thread.
HELP_DEVINL double block_sum(double v, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[w];
    __syncthreads();
    return s;
}

template <class T>
HELP_DEVINL T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

HELP_DEVINL double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }
HELP_DEVINL float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }

}  // namespace help
