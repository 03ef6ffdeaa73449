// Device-side building blocks shared by the kernels: deterministic block
// reductions, cache-hinted loads.
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

// Streamed once per kernel (a matrix's indices and values): non-coherent
// path without allocating in L1, so L1 keeps the gathered vector's lines.
HELP_DEVINL int2 ld_stream_na(const int2* p) {
    int2 v;
    asm("ld.global.nc.L1::no_allocate.v2.s32 {%0,%1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}
HELP_DEVINL double2 ld_stream_na(const double2* p) {
    double2 v;
    asm("ld.global.nc.L1::no_allocate.v2.f64 {%0,%1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
    return v;
}
HELP_DEVINL float2 ld_stream_na(const float2* p) {
    float2 v;
    asm("ld.global.nc.L1::no_allocate.v2.f32 {%0,%1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
    return v;
}
template <class V>
struct Vec2;
template <>
struct Vec2<double> {
    using T = double2;
};
template <>
struct Vec2<float> {
    using T = float2;
};

// Status codes a kernel can leave in its status word (mirror HELP_E_*).
constexpr int kStatusOk = 0;
constexpr int kStatusTimeout = -5;
constexpr int kStatusNumeric = -4;

// Deterministic block-wide sum with few FP64 instructions (GB300 issues FP64
// at ~2 lanes/clk/SM, so a reduction where every thread adds every warp's
// partial costs microseconds): a shared-memory tree halving the active
// threads, then one warp's shuffles.  blockDim.x must be a power of two
// <= 1024; `red` holds blockDim.x doubles.  Result valid in every thread.
HELP_DEVINL double block_sum(double v, double* red) {
    const int tid = threadIdx.x;
    __syncthreads();
    red[tid] = v;
    __syncthreads();
    for (int s = blockDim.x >> 1; s >= 32; s >>= 1) {
        if (tid < s) red[tid] += red[tid + s];
        __syncthreads();
    }
    if (tid < 32) {
        double w = red[tid];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
        if (tid == 0) red[0] = w;
    }
    __syncthreads();
    return red[0];
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
