// Standalone SpMV launches (the two passes of one A D^-1 A^T v, the
// right-hand side A D^-1 b_1 - b_2 and the back-substitution
// D^-1 (b_1 - A^T x_2) of UsePCG_CPU.cpp:103-177, the FP64 residual of the
// refinement loop) and small vector kernels.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "spmv.cuh"

namespace help {

namespace {

template <class V, int EPI>
__global__ void __launch_bounds__(256) k_spmv(const SpmvView<V> M, const V* __restrict__ x, V* __restrict__ y,
                                              const V* __restrict__ aux, const V* __restrict__ aux2,
                                              const double* __restrict__ s2, double delta) {
    __shared__ double red[256];
    spmv_rows<V, 4>(
        M, [&](int c) { return ld_ro(x + c); },
        [&](int row, V s) {
            if (EPI == kEpiStore) {
                y[row] = s;
            } else if (EPI == kEpiRhs) {
                y[row] = s - aux[row];
            } else if (EPI == kEpiBacksub) {
                y[row] = (V)(s2[row] * ((double)aux[row] - (double)s));
            } else if (EPI == kEpiResid) {
                y[row] = aux[row] - fma_t((V)delta, aux2[row], s);
            } else if (EPI == kEpiAcc) {
                y[row] = fma_t((V)delta, s, aux[row]);
            } else {
                y[row] = fma_t((V)delta, aux[row], s);
            }
        },
        red);
}

// B's values into a sliced layout: dst[q] = src[map[q]], 0 on padding
template <class V>
__global__ void k_sell_gather(const int* __restrict__ map, const V* __restrict__ src, V* __restrict__ dst, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = map[i];
        dst[i] = c >= 0 ? ld_ro(src + c) : V(0);
    }
}

__global__ void k_mul(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = a[i] * b[i];
}
__global__ void k_to_f32(const double* __restrict__ a, float* __restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)a[i];
}
__global__ void k_add_f32(double* __restrict__ x, const float* __restrict__ e, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] += (double)e[i];
}
__global__ void k_to_f32_scaled(const double* __restrict__ a, double scale, float* __restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)(a[i] * scale);
}
__global__ void k_add_f32_scaled(double* __restrict__ x, const float* __restrict__ e, double scale, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = fma((double)e[i], scale, x[i]);
}
__global__ void k_fill(double* __restrict__ x, double v, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = v;
}
__global__ void k_fill_f32(float* __restrict__ x, float v, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = v;
}
__global__ void k_sumsq_part(const double* __restrict__ x, int64_t n, double* __restrict__ part) {
    __shared__ double red[1024];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(x[i], x[i], s);
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void k_dot_part(const double* __restrict__ x, const double* __restrict__ y, int64_t n,
                           double* __restrict__ part) {
    __shared__ double red[1024];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(x[i], y[i], s);
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void k_scale(double* __restrict__ x, double a, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= a;
}
__global__ void k_sum_parts(const double* __restrict__ part, int np, double* __restrict__ out) {
    __shared__ double red[1024];
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) *out = s;
}

inline int grid_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 4096) b = 4096;
    return (int)b;
}

}  // namespace

int spmv_blocks_per_sm() {
    static const int per_sm = [] {
        int lo = 0;
        auto take = [&](const void* f) {
            int b = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f, 256, 0) == cudaSuccess && b > 0)
                lo = lo ? std::min(lo, b) : b;
        };
        take((const void*)k_spmv<double, kEpiStore>);
        take((const void*)k_spmv<double, kEpiRhs>);
        take((const void*)k_spmv<double, kEpiBacksub>);
        take((const void*)k_spmv<double, kEpiResid>);
        take((const void*)k_spmv<double, kEpiAddDelta>);
        take((const void*)k_spmv<double, kEpiAcc>);
        take((const void*)k_spmv<float, kEpiStore>);
        take((const void*)k_spmv<float, kEpiAddDelta>);
        cudaGetLastError();
        return lo > 0 ? lo : 8;
    }();
    return per_sm;
}

template <class V, int E>
cudaError_t spmv_launch_one(const SpmvView<V>& M, const V* x, V* y, const V* aux, const V* aux2, const double* s2,
                            double delta, int blocks, int threads, cudaStream_t stream) {
    k_spmv<V, E><<<blocks, threads, 0, stream>>>(M, x, y, aux, aux2, s2, delta);
    return cudaGetLastError();
}

template <class V>
cudaError_t spmv_launch(int epi, const SpmvView<V>& M, const V* x, V* y, const V* aux, const V* aux2,
                        const double* s2, double delta, int blocks, int threads, cudaStream_t stream) {
    if (M.rows <= 0) return cudaSuccess;
    if (blocks <= 0) blocks = 1;
    switch (epi) {
        case kEpiStore: return spmv_launch_one<V, kEpiStore>(M, x, y, aux, aux2, s2, delta, blocks, threads, stream);
        case kEpiRhs: return spmv_launch_one<V, kEpiRhs>(M, x, y, aux, aux2, s2, delta, blocks, threads, stream);
        case kEpiBacksub: return spmv_launch_one<V, kEpiBacksub>(M, x, y, aux, aux2, s2, delta, blocks, threads, stream);
        case kEpiResid: return spmv_launch_one<V, kEpiResid>(M, x, y, aux, aux2, s2, delta, blocks, threads, stream);
        case kEpiAddDelta:
            return spmv_launch_one<V, kEpiAddDelta>(M, x, y, aux, aux2, s2, delta, blocks, threads, stream);
        case kEpiAcc: return spmv_launch_one<V, kEpiAcc>(M, x, y, aux, aux2, s2, delta, blocks, threads, stream);
        default:
            return cudaErrorInvalidValue;
    }
}

template cudaError_t spmv_launch<double>(int, const SpmvView<double>&, const double*, double*, const double*,
                                         const double*, const double*, double, int, int, cudaStream_t);
template cudaError_t spmv_launch<float>(int, const SpmvView<float>&, const float*, float*, const float*, const float*,
                                        const double*, double, int, int, cudaStream_t);

cudaError_t vec_scale_mul(const double* a, const double* b, double* out, int64_t n, cudaStream_t st) {
    k_mul<<<grid_for(n, 256), 256, 0, st>>>(a, b, out, n);
    return cudaGetLastError();
}
cudaError_t vec_to_f32(const double* a, float* out, int64_t n, cudaStream_t st) {
    k_to_f32<<<grid_for(n, 256), 256, 0, st>>>(a, out, n);
    return cudaGetLastError();
}
cudaError_t vec_add_f32(double* x, const float* e, int64_t n, cudaStream_t st) {
    k_add_f32<<<grid_for(n, 256), 256, 0, st>>>(x, e, n);
    return cudaGetLastError();
}
cudaError_t vec_to_f32_scaled(const double* a, double scale, float* out, int64_t n, cudaStream_t st) {
    k_to_f32_scaled<<<grid_for(n, 256), 256, 0, st>>>(a, scale, out, n);
    return cudaGetLastError();
}
cudaError_t vec_add_f32_scaled(double* x, const float* e, double scale, int64_t n, cudaStream_t st) {
    k_add_f32_scaled<<<grid_for(n, 256), 256, 0, st>>>(x, e, scale, n);
    return cudaGetLastError();
}
namespace {
__global__ void k_copy16(const double2* __restrict__ src, double2* __restrict__ dst, int64_t n2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}
__global__ void k_copy8(const double* __restrict__ src, double* __restrict__ dst, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}
}  // namespace

cudaError_t vec_copy(const double* src, double* dst, int64_t n, int num_sms, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int blocks = num_sms > 0 ? num_sms * 4 : 256;
    if ((((uintptr_t)src | (uintptr_t)dst) & 15) == 0) {
        const int64_t n2 = n / 2;
        if (n2 > 0) k_copy16<<<blocks, 256, 0, st>>>(reinterpret_cast<const double2*>(src), reinterpret_cast<double2*>(dst), n2);
        if (n & 1) k_copy8<<<1, 32, 0, st>>>(src + 2 * n2, dst + 2 * n2, 1);
    } else {
        k_copy8<<<blocks, 256, 0, st>>>(src, dst, n);
    }
    return cudaGetLastError();
}

cudaError_t vec_fill(double* x, double v, int64_t n, cudaStream_t st) {
    k_fill<<<grid_for(n, 256), 256, 0, st>>>(x, v, n);
    return cudaGetLastError();
}
cudaError_t vec_fill_f32(float* x, float v, int64_t n, cudaStream_t st) {
    k_fill_f32<<<grid_for(n, 256), 256, 0, st>>>(x, v, n);
    return cudaGetLastError();
}
cudaError_t vec_dot(const double* x, const double* y, int64_t n, double* part, double* out, cudaStream_t st) {
    const int nb = 1024;
    k_dot_part<<<nb, 256, 0, st>>>(x, y, n, part);
    k_sum_parts<<<1, 1024, 0, st>>>(part, nb, out);
    return cudaGetLastError();
}
cudaError_t vec_scale(double* x, double a, int64_t n, cudaStream_t st) {
    k_scale<<<grid_for(n, 256), 256, 0, st>>>(x, a, n);
    return cudaGetLastError();
}
cudaError_t vec_sumsq(const double* x, int64_t n, double* part, double* out, cudaStream_t st) {
    const int nb = 1024;
    k_sumsq_part<<<nb, 256, 0, st>>>(x, n, part);
    k_sum_parts<<<1, 1024, 0, st>>>(part, nb, out);
    return cudaGetLastError();
}

template <class V>
cudaError_t sell_gather(const int* map, const V* src, V* dst, int64_t n, int num_sms, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int64_t want = (n + 255) / 256;
    const int blocks = (int)std::min<int64_t>(want, (int64_t)num_sms * 8);
    k_sell_gather<V><<<blocks, 256, 0, st>>>(map, src, dst, n);
    return cudaGetLastError();
}
template cudaError_t sell_gather<double>(const int*, const double*, double*, int64_t, int, cudaStream_t);
template cudaError_t sell_gather<float>(const int*, const float*, float*, int64_t, int, cudaStream_t);

}  // namespace help
