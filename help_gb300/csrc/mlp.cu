// Learned part of the preconditioner: a 16 -> 64 -> 64 -> 2 MLP (ReLU) over
// per-row features of the normal equations, in BF16 with FP32 accumulation
// on the tensor cores: the inference forward on tcgen05 with TMEM
// accumulators (k_mlp_fwd_tc, below), the training forward and backward on
// mma.sync m16n8k16.
//
//   out[i, 0]  log-factor of a correction of the Schur diagonal D_S,i
//   out[i, 1]  per-row scale of the warm start (previous solution of the
//              same solve slot)
//
// Training: each warp takes tiles of 16 rows.  Forward: the accumulator fragment of
// one layer is exactly the A-operand fragment of the next (after ReLU and
// rounding to BF16), so activations never leave registers; in training mode
// they are also stored (BF16) for the backward pass.  Backward: per group of
// 64 rows each warp back-propagates its 16-row tile (dH = dZ W on the tensor
// cores, ReLU masks from the stored activations), stages the tiles in shared
// memory, and then each warp accumulates one 16-row slice of every weight
// gradient over the group (K = rows); blocks write per-block partials that a
// second kernel adds in block order, so gradients are deterministic.
//
// The matrices are 64 wide: one launch over 500k rows is ~16 GFLOP forward,
// microseconds of tensor work; the kernels are bound by reading the
// features and activations.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/help_gpu.h"
#include "common.cuh"
#include "kernels.h"
#include "mlp.h"

namespace help {
namespace {

constexpr int kMlpThreads = 128;  // 4 warps
constexpr int kF = HELP_MLP_IN, kH = HELP_MLP_HIDDEN;

HELP_DEVINL uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}
HELP_DEVINL uint32_t pack_raw(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}
HELP_DEVINL float bf(__nv_bfloat16 v) { return __bfloat162float(v); }
HELP_DEVINL uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// D = A B + C, A 16x16 (row), B 16x8 (col), BF16 in, FP32 accumulate.
HELP_DEVINL void mma16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                          uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

struct MlpSmemW {
    __nv_bfloat16 w1[kH * kF];
    __nv_bfloat16 w2[kH * kH];
    __nv_bfloat16 w3[16 * kH];  // rows >= HELP_MLP_OUT are zero
    float b1[kH], b2[kH], b3[8];
};

HELP_DEVINL void load_weights(const MlpDevWeights* w, MlpSmemW& s) {
    for (int i = threadIdx.x; i < kH * kF; i += blockDim.x) s.w1[i] = w->w1[i];
    for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) s.w2[i] = w->w2[i];
    for (int i = threadIdx.x; i < 16 * kH; i += blockDim.x) s.w3[i] = i < 8 * kH ? w->w3[i] : __float2bfloat16(0.f);
    for (int i = threadIdx.x; i < kH; i += blockDim.x) {
        s.b1[i] = w->b1[i];
        s.b2[i] = w->b2[i];
    }
    if (threadIdx.x < 8) s.b3[threadIdx.x] = w->b3[threadIdx.x];
    __syncthreads();
}

// ---- forward over rows; SAVE: keep H1, H2 (BF16, rows x 64) for backward
template <bool SAVE>
__global__ void __launch_bounds__(kMlpThreads) k_mlp_fwd(const __nv_bfloat16* __restrict__ X, long long rows,
                                                         const MlpDevWeights* __restrict__ w, float* __restrict__ out,
                                                         __nv_bfloat16* __restrict__ H1, __nv_bfloat16* __restrict__ H2) {
    __shared__ MlpSmemW s;
    load_weights(w, s);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const long long ntiles = (rows + 15) / 16;
    for (long long tile = (long long)blockIdx.x * 4 + warp; tile < ntiles; tile += (long long)gridDim.x * 4) {
        const long long ra = tile * 16 + g, rb = ra + 8;
        const bool va = ra < rows, vb = rb < rows;
        const uint32_t x0 = va ? ld32(X + ra * kF + 2 * t) : 0u;
        const uint32_t x1 = vb ? ld32(X + rb * kF + 2 * t) : 0u;
        const uint32_t x2 = va ? ld32(X + ra * kF + 2 * t + 8) : 0u;
        const uint32_t x3 = vb ? ld32(X + rb * kF + 2 * t + 8) : 0u;
        // layer 1
        uint32_t h1[8][2];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = 8 * j + g;
            float z[4] = {s.b1[8 * j + 2 * t], s.b1[8 * j + 2 * t + 1], s.b1[8 * j + 2 * t], s.b1[8 * j + 2 * t + 1]};
            mma16816(z, x0, x1, x2, x3, ld32(s.w1 + n * kF + 2 * t), ld32(s.w1 + n * kF + 2 * t + 8));
            h1[j][0] = pack_bf16(fmaxf(z[0], 0.f), fmaxf(z[1], 0.f));
            h1[j][1] = pack_bf16(fmaxf(z[2], 0.f), fmaxf(z[3], 0.f));
            if (SAVE) {
                if (va) *reinterpret_cast<uint32_t*>(H1 + ra * kH + 8 * j + 2 * t) = h1[j][0];
                if (vb) *reinterpret_cast<uint32_t*>(H1 + rb * kH + 8 * j + 2 * t) = h1[j][1];
            }
        }
        // layer 2
        uint32_t h2[8][2];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = 8 * j + g;
            float z[4] = {s.b2[8 * j + 2 * t], s.b2[8 * j + 2 * t + 1], s.b2[8 * j + 2 * t], s.b2[8 * j + 2 * t + 1]};
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                mma16816(z, h1[2 * kk][0], h1[2 * kk][1], h1[2 * kk + 1][0], h1[2 * kk + 1][1],
                         ld32(s.w2 + n * kH + 16 * kk + 2 * t), ld32(s.w2 + n * kH + 16 * kk + 2 * t + 8));
            h2[j][0] = pack_bf16(fmaxf(z[0], 0.f), fmaxf(z[1], 0.f));
            h2[j][1] = pack_bf16(fmaxf(z[2], 0.f), fmaxf(z[3], 0.f));
            if (SAVE) {
                if (va) *reinterpret_cast<uint32_t*>(H2 + ra * kH + 8 * j + 2 * t) = h2[j][0];
                if (vb) *reinterpret_cast<uint32_t*>(H2 + rb * kH + 8 * j + 2 * t) = h2[j][1];
            }
        }
        // layer 3 (outputs padded to one 8-wide tile)
        float z[4] = {s.b3[2 * t], s.b3[2 * t + 1], s.b3[2 * t], s.b3[2 * t + 1]};
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
            mma16816(z, h2[2 * kk][0], h2[2 * kk][1], h2[2 * kk + 1][0], h2[2 * kk + 1][1],
                     ld32(s.w3 + g * kH + 16 * kk + 2 * t), ld32(s.w3 + g * kH + 16 * kk + 2 * t + 8));
        if (t == 0) {
            if (va) {
                out[ra * 2] = z[0];
                out[ra * 2 + 1] = z[1];
            }
            if (vb) {
                out[rb * 2] = z[2];
                out[rb * 2 + 1] = z[3];
            }
        }
    }
}

// ---- inference forward on the 5th-generation tensor cores (tcgen05 + TMEM)
//
// One CTA of 4 warps takes tiles of 128 rows: the tile's features and the
// weights sit in shared memory in the canonical K-major layout without
// swizzle (core matrices of 8 rows x 16 bytes; LBO = 128 bytes between core
// matrices along K, SBO = (K / 8) x 128 bytes between 8-row groups), one
// thread issues the layer's tcgen05.mma (M = 128, K = 16 per instruction)
// into a 64-column TMEM accumulator and commits it to an mbarrier; each warp
// then reads its 32 rows back with tcgen05.ld, adds the bias, applies ReLU,
// rounds to BF16 (as the mma.sync kernel does) and writes the next layer's
// A operand.  Every mbarrier wait is bounded: past the bound the tile's
// outputs are NaN, the CTA waits once more for the MMA in flight and frees
// its TMEM before returning.
constexpr int kTcRows = 128;
constexpr int kTcThreads = 128;
constexpr int kTcCols = 64;  // TMEM columns per CTA (FP32 accumulators of N = 64)
constexpr long kTcWaitPolls = 1L << 20;

struct TcSmem {
    __nv_bfloat16 x[kTcRows * kF];  // layer-1 A: 16 groups x 2 chunks (SBO 256)
    __nv_bfloat16 h[kTcRows * kH];  // layer-2/3 A: 16 groups x 8 chunks (SBO 1024)
    __nv_bfloat16 w1[kH * kF];      // layer-1 B: 8 groups x 2 chunks
    __nv_bfloat16 w2[kH * kH];      // layer-2 B: 8 groups x 8 chunks
    __nv_bfloat16 w3[16 * kH];      // layer-3 B: 2 groups x 8 chunks, rows >= HELP_MLP_OUT zero
    float b1[kH], b2[kH], b3[16];
    unsigned long long mbar;
    uint32_t tmem;
};

// byte offset of element (r, k) of an operand with K columns in the canonical layout
HELP_DEVINL uint32_t canon(int r, int k, int K) {
    return (uint32_t)((r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

HELP_DEVINL uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start >> 4, LBO >> 4, SBO >> 4, version 1, no swizzle
HELP_DEVINL uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major, N, M = 128
HELP_DEVINL uint32_t tc_idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);
}

HELP_DEVINL void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

HELP_DEVINL void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

HELP_DEVINL bool mbar_wait(uint32_t mbar, uint32_t phase) {
    for (long i = 0; i < kTcWaitPolls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

HELP_DEVINL void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
HELP_DEVINL void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
HELP_DEVINL void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes
HELP_DEVINL void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// bias, ReLU, BF16, into row `row` of the next layer's A operand (64 columns)
HELP_DEVINL void tc_hidden_out(uint32_t taddr, const float* bias, unsigned char* h, int row) {
#pragma unroll
    for (int q = 0; q < kH / 16; ++q) {
        float v[16];
        tc_ld16(taddr + 16 * q, v);
        uint32_t p[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
            p[j] = pack_bf16(fmaxf(v[2 * j] + bias[16 * q + 2 * j], 0.f),
                             fmaxf(v[2 * j + 1] + bias[16 * q + 2 * j + 1], 0.f));
        *reinterpret_cast<uint4*>(h + canon(row, 16 * q, kH)) = make_uint4(p[0], p[1], p[2], p[3]);
        *reinterpret_cast<uint4*>(h + canon(row, 16 * q + 8, kH)) = make_uint4(p[4], p[5], p[6], p[7]);
    }
}

__global__ void __launch_bounds__(kTcThreads) k_mlp_fwd_tc(const __nv_bfloat16* __restrict__ X, long long rows,
                                                            const MlpDevWeights* __restrict__ w,
                                                            float* __restrict__ out, bool x16) {
    extern __shared__ __align__(1024) unsigned char tc_raw[];
    TcSmem& s = *reinterpret_cast<TcSmem*>(tc_raw);
    unsigned char* sx = reinterpret_cast<unsigned char*>(s.x);
    unsigned char* sh = reinterpret_cast<unsigned char*>(s.h);
    unsigned char* sw1 = reinterpret_cast<unsigned char*>(s.w1);
    unsigned char* sw2 = reinterpret_cast<unsigned char*>(s.w2);
    unsigned char* sw3 = reinterpret_cast<unsigned char*>(s.w3);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < kH * kF; i += kTcThreads)
        *reinterpret_cast<__nv_bfloat16*>(sw1 + canon(i / kF, i % kF, kF)) = w->w1[i];
    for (int i = tid; i < kH * kH; i += kTcThreads)
        *reinterpret_cast<__nv_bfloat16*>(sw2 + canon(i / kH, i % kH, kH)) = w->w2[i];
    for (int i = tid; i < 16 * kH; i += kTcThreads)
        *reinterpret_cast<__nv_bfloat16*>(sw3 + canon(i / kH, i % kH, kH)) =
            i < 8 * kH ? w->w3[i] : __float2bfloat16(0.f);
    for (int i = tid; i < kH; i += kTcThreads) {
        s.b1[i] = w->b1[i];
        s.b2[i] = w->b2[i];
    }
    if (tid < 16) s.b3[tid] = tid < 8 ? w->b3[tid] : 0.f;
    const uint32_t mbar = smem_u32(&s.mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s.tmem)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    proxy_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s.tmem;
    const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's 32 lanes
    const uint32_t ax = smem_u32(sx), ah = smem_u32(sh);
    const uint32_t b1a = smem_u32(sw1), b2a = smem_u32(sw2), b3a = smem_u32(sw3);
    uint32_t phase = 0;
    bool ok = true;
    const long long ntiles = (rows + kTcRows - 1) / kTcRows;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long r = tile * kTcRows + tid;
        // features of row r (BF16 pairs: 4-byte aligned) into the layer-1 A operand
        uint4 f0 = make_uint4(0u, 0u, 0u, 0u), f1 = f0;
        if (ok && r < rows) {
            if (x16) {  // a row is 32 bytes: two 16-byte loads
                const uint4* xr = reinterpret_cast<const uint4*>(X + r * kF);
                f0 = __ldg(xr);
                f1 = __ldg(xr + 1);
            } else {
                const __nv_bfloat16* xr = X + r * kF;
                f0 = make_uint4(ld32(xr), ld32(xr + 2), ld32(xr + 4), ld32(xr + 6));
                f1 = make_uint4(ld32(xr + 8), ld32(xr + 10), ld32(xr + 12), ld32(xr + 14));
            }
        }
        *reinterpret_cast<uint4*>(sx + canon(tid, 0, kF)) = f0;
        *reinterpret_cast<uint4*>(sx + canon(tid, 8, kF)) = f1;
        proxy_fence();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        // layer 1: K = 16, one instruction
        if (ok && tid == 0) {
            tc_mma(tmem, tc_desc(ax, 128, 256), tc_desc(b1a, 128, 256), tc_idesc(kH), 0u);
            tc_commit(mbar);
        }
        if (ok) ok = mbar_wait(mbar, phase);
        phase ^= 1u;
        ok = __syncthreads_and(ok);  // tcgen05.ld is warp-collective: one outcome for the whole CTA
        if (!ok) break;              // phase ^ 1 stays the pending phase for the wait below
        tc_fence_after();
        if (ok) tc_hidden_out(trow, s.b1, sh, tid);
        proxy_fence();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        ok = __syncthreads_and(ok);
        // layer 2: K = 64, four instructions of K = 16 (two core matrices each)
        if (ok && tid == 0) {
#pragma unroll
            for (int ks = 0; ks < kH / 16; ++ks)
                tc_mma(tmem, tc_desc(ah + 256 * ks, 128, 1024), tc_desc(b2a + 256 * ks, 128, 1024), tc_idesc(kH),
                       ks > 0 ? 1u : 0u);
            tc_commit(mbar);
        }
        if (ok) ok = mbar_wait(mbar, phase);
        phase ^= 1u;
        ok = __syncthreads_and(ok);  // tcgen05.ld is warp-collective: one outcome for the whole CTA
        if (!ok) break;              // phase ^ 1 stays the pending phase for the wait below
        tc_fence_after();
        if (ok) tc_hidden_out(trow, s.b2, sh, tid);
        proxy_fence();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        ok = __syncthreads_and(ok);
        // layer 3: N = 16 (two outputs used), K = 64
        if (ok && tid == 0) {
#pragma unroll
            for (int ks = 0; ks < kH / 16; ++ks)
                tc_mma(tmem, tc_desc(ah + 256 * ks, 128, 1024), tc_desc(b3a + 256 * ks, 128, 1024), tc_idesc(16),
                       ks > 0 ? 1u : 0u);
            tc_commit(mbar);
        }
        if (ok) ok = mbar_wait(mbar, phase);
        phase ^= 1u;
        ok = __syncthreads_and(ok);  // tcgen05.ld is warp-collective: one outcome for the whole CTA
        if (!ok) break;              // phase ^ 1 stays the pending phase for the wait below
        tc_fence_after();
        float v[16];
        if (ok) tc_ld16(trow, v);
        if (r < rows) {
            out[r * 2] = ok ? v[0] + s.b3[0] : __int_as_float(0x7fc00000);
            out[r * 2 + 1] = ok ? v[1] + s.b3[1] : __int_as_float(0x7fc00000);
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        ok = __syncthreads_and(ok);
    }
    if (!ok) {
        // an MMA never signalled: give it one more bounded wait before the
        // accumulator is freed, and mark all of the CTA's rows
        if (tid == 0) mbar_wait(mbar, phase ^ 1u);
        for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const long long r = tile * kTcRows + tid;
            if (r < rows) out[r * 2] = out[r * 2 + 1] = __int_as_float(0x7fc00000);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
}

// ---- weighted squared error: loss partials, G3 = dL/dout
__global__ void __launch_bounds__(256) k_mlp_wsum(const float* __restrict__ wt, long long n, double* part) {
    __shared__ double red[256];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += (double)wt[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void __launch_bounds__(256) k_mlp_loss(const float* __restrict__ out, const float* __restrict__ tg,
                                                  const float* __restrict__ wt, long long n, const double* wpart,
                                                  int nwpart, float* __restrict__ G3, double* part) {
    __shared__ double red[256];
    __shared__ float s_inv;
    if (threadIdx.x == 0) {
        double ws = 0.0;
        for (int b = 0; b < nwpart; ++b) ws += wpart[b];
        s_inv = ws > 0.0 ? (float)(1.0 / ws) : 0.f;
    }
    __syncthreads();
    const float inv = s_inv;
    double l = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float e = out[i] - tg[i];
        G3[i] = 2.f * wt[i] * e * inv;
        l += (double)(wt[i] * e * e * inv);
    }
    l = block_sum(l, red);
    if (threadIdx.x == 0) part[blockIdx.x] = l;
}

// ---- backward: per-block partial gradients (layout of the trainable params)
struct BwdSmem {
    MlpSmemW w;
    __nv_bfloat16 xs[64 * kF];
    __nv_bfloat16 h1[64 * kH];
    __nv_bfloat16 h2[64 * kH];
    __nv_bfloat16 dz1[64 * kH];
    __nv_bfloat16 dz2[64 * kH];
    __nv_bfloat16 g3[64 * 16];  // columns >= HELP_MLP_OUT are zero
};

__global__ void __launch_bounds__(kMlpThreads) k_mlp_bwd(const __nv_bfloat16* __restrict__ X, long long rows,
                                                         const MlpDevWeights* __restrict__ w,
                                                         const float* __restrict__ G3,
                                                         const __nv_bfloat16* __restrict__ H1,
                                                         const __nv_bfloat16* __restrict__ H2,
                                                         float* __restrict__ part) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BwdSmem& s = *reinterpret_cast<BwdSmem*>(smem_raw);
    load_weights(w, s.w);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    float acc2[8][4], acc1[2][4], acc3[2][4];
#pragma unroll
    for (int j = 0; j < 8; ++j)
        for (int c = 0; c < 4; ++c) acc2[j][c] = 0.f;
#pragma unroll
    for (int j = 0; j < 2; ++j)
        for (int c = 0; c < 4; ++c) acc1[j][c] = acc3[j][c] = 0.f;
    float bsum0 = 0.f, bsum1 = 0.f;  // bias gradients: warp 0 db2, warp 1 db1, warp 2 db3 (lanes 0, 1)
    const long long ngroups = (rows + 63) / 64;
    for (long long grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        // ---- step 1: this warp's tile (rows 16 warp .. 16 warp + 15 of the group)
        const int lr = 16 * warp;  // local row base in the group tiles
        const long long r0 = grp * 64 + lr;
        for (int i = lane; i < 16 * kF; i += 32) {
            const long long r = r0 + i / kF;
            s.xs[lr * kF + i] = r < rows ? X[r * kF + i % kF] : zero;
        }
        for (int i = lane; i < 16 * kH; i += 32) {
            const long long r = r0 + i / kH;
            s.h1[lr * kH + i] = r < rows ? H1[r * kH + i % kH] : zero;
            s.h2[lr * kH + i] = r < rows ? H2[r * kH + i % kH] : zero;
        }
        for (int i = lane; i < 16 * 16; i += 32) {
            const long long r = r0 + i / 16;
            const int o = i % 16;
            s.g3[lr * 16 + i] = (r < rows && o < HELP_MLP_OUT) ? __float2bfloat16(G3[r * HELP_MLP_OUT + o]) : zero;
        }
        __syncwarp();
        const __nv_bfloat16* g3t = s.g3 + lr * 16;
        const __nv_bfloat16* h1t = s.h1 + lr * kH;
        const __nv_bfloat16* h2t = s.h2 + lr * kH;
        // dH2 = G3 W3 (K = outputs, padded to 16)
        const uint32_t ga0 = ld32(g3t + g * 16 + 2 * t), ga1 = ld32(g3t + (g + 8) * 16 + 2 * t);
        const uint32_t ga2 = ld32(g3t + g * 16 + 2 * t + 8), ga3 = ld32(g3t + (g + 8) * 16 + 2 * t + 8);
        uint32_t dz2[8][2];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = 8 * j + g;
            float d[4] = {0.f, 0.f, 0.f, 0.f};
            mma16816(d, ga0, ga1, ga2, ga3, pack_raw(s.w.w3[(2 * t) * kH + n], s.w.w3[(2 * t + 1) * kH + n]),
                     pack_raw(s.w.w3[(2 * t + 8) * kH + n], s.w.w3[(2 * t + 9) * kH + n]));
            const int c = 8 * j + 2 * t;
            d[0] = bf(h2t[g * kH + c]) > 0.f ? d[0] : 0.f;
            d[1] = bf(h2t[g * kH + c + 1]) > 0.f ? d[1] : 0.f;
            d[2] = bf(h2t[(g + 8) * kH + c]) > 0.f ? d[2] : 0.f;
            d[3] = bf(h2t[(g + 8) * kH + c + 1]) > 0.f ? d[3] : 0.f;
            dz2[j][0] = pack_bf16(d[0], d[1]);
            dz2[j][1] = pack_bf16(d[2], d[3]);
            *reinterpret_cast<uint32_t*>(s.dz2 + (lr + g) * kH + c) = dz2[j][0];
            *reinterpret_cast<uint32_t*>(s.dz2 + (lr + g + 8) * kH + c) = dz2[j][1];
        }
        // dH1 = dZ2 W2 (K = 64)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = 8 * j + g;
            float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const int k0 = 16 * kk + 2 * t;
                mma16816(d, dz2[2 * kk][0], dz2[2 * kk][1], dz2[2 * kk + 1][0], dz2[2 * kk + 1][1],
                         pack_raw(s.w.w2[k0 * kH + n], s.w.w2[(k0 + 1) * kH + n]),
                         pack_raw(s.w.w2[(k0 + 8) * kH + n], s.w.w2[(k0 + 9) * kH + n]));
            }
            const int c = 8 * j + 2 * t;
            d[0] = bf(h1t[g * kH + c]) > 0.f ? d[0] : 0.f;
            d[1] = bf(h1t[g * kH + c + 1]) > 0.f ? d[1] : 0.f;
            d[2] = bf(h1t[(g + 8) * kH + c]) > 0.f ? d[2] : 0.f;
            d[3] = bf(h1t[(g + 8) * kH + c + 1]) > 0.f ? d[3] : 0.f;
            *reinterpret_cast<uint32_t*>(s.dz1 + (lr + g) * kH + c) = pack_bf16(d[0], d[1]);
            *reinterpret_cast<uint32_t*>(s.dz1 + (lr + g + 8) * kH + c) = pack_bf16(d[2], d[3]);
        }
        __syncthreads();
        // ---- step 2: weight gradients over the group's 64 rows (K = rows, 4 steps of 16)
        const int m0 = 16 * warp;  // this warp's 16-row slice of dW2 / dW1, 16-column slice of dW3
#pragma unroll
        for (int kb = 0; kb < 64; kb += 16) {
            const int ka = kb + 2 * t;
            // A = dZ2^T slice: A[m][k] = dz2[k][m0 + m]
            const uint32_t a0 = pack_raw(s.dz2[ka * kH + m0 + g], s.dz2[(ka + 1) * kH + m0 + g]);
            const uint32_t a1 = pack_raw(s.dz2[ka * kH + m0 + g + 8], s.dz2[(ka + 1) * kH + m0 + g + 8]);
            const uint32_t a2 = pack_raw(s.dz2[(ka + 8) * kH + m0 + g], s.dz2[(ka + 9) * kH + m0 + g]);
            const uint32_t a3 = pack_raw(s.dz2[(ka + 8) * kH + m0 + g + 8], s.dz2[(ka + 9) * kH + m0 + g + 8]);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int n = 8 * j + g;
                mma16816(acc2[j], a0, a1, a2, a3, pack_raw(s.h1[ka * kH + n], s.h1[(ka + 1) * kH + n]),
                         pack_raw(s.h1[(ka + 8) * kH + n], s.h1[(ka + 9) * kH + n]));
            }
            // A = dZ1^T slice, B = X
            const uint32_t e0 = pack_raw(s.dz1[ka * kH + m0 + g], s.dz1[(ka + 1) * kH + m0 + g]);
            const uint32_t e1 = pack_raw(s.dz1[ka * kH + m0 + g + 8], s.dz1[(ka + 1) * kH + m0 + g + 8]);
            const uint32_t e2 = pack_raw(s.dz1[(ka + 8) * kH + m0 + g], s.dz1[(ka + 9) * kH + m0 + g]);
            const uint32_t e3 = pack_raw(s.dz1[(ka + 8) * kH + m0 + g + 8], s.dz1[(ka + 9) * kH + m0 + g + 8]);
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int n = 8 * j + g;
                mma16816(acc1[j], e0, e1, e2, e3, pack_raw(s.xs[ka * kF + n], s.xs[(ka + 1) * kF + n]),
                         pack_raw(s.xs[(ka + 8) * kF + n], s.xs[(ka + 9) * kF + n]));
            }
            // A = G3^T (outputs padded to 16), B = H2 columns m0 .. m0 + 15
            const uint32_t f0 = pack_raw(s.g3[ka * 16 + g], s.g3[(ka + 1) * 16 + g]);
            const uint32_t f1 = pack_raw(s.g3[ka * 16 + g + 8], s.g3[(ka + 1) * 16 + g + 8]);
            const uint32_t f2 = pack_raw(s.g3[(ka + 8) * 16 + g], s.g3[(ka + 9) * 16 + g]);
            const uint32_t f3 = pack_raw(s.g3[(ka + 8) * 16 + g + 8], s.g3[(ka + 9) * 16 + g + 8]);
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int n = m0 + 8 * j + g;
                mma16816(acc3[j], f0, f1, f2, f3, pack_raw(s.h2[ka * kH + n], s.h2[(ka + 1) * kH + n]),
                         pack_raw(s.h2[(ka + 8) * kH + n], s.h2[(ka + 9) * kH + n]));
            }
        }
        // bias gradients, rows in order
        if (warp == 0) {
            for (int r = 0; r < 64; ++r) {
                bsum0 += bf(s.dz2[r * kH + lane]);
                bsum1 += bf(s.dz2[r * kH + lane + 32]);
            }
        } else if (warp == 1) {
            for (int r = 0; r < 64; ++r) {
                bsum0 += bf(s.dz1[r * kH + lane]);
                bsum1 += bf(s.dz1[r * kH + lane + 32]);
            }
        } else if (warp == 2 && lane < HELP_MLP_OUT) {
            for (int r = 0; r < 64; ++r) bsum0 += bf(s.g3[r * 16 + lane]);
        }
        __syncthreads();
    }
    // ---- this block's partial, in the parameter order of help_gpu.h
    float* p = part + (size_t)blockIdx.x * kMlpGradParams;
    const int m0 = 16 * warp;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int c = 8 * j + 2 * t;
        p[HELP_MLP_OFF_W2 + (m0 + g) * kH + c] = acc2[j][0];
        p[HELP_MLP_OFF_W2 + (m0 + g) * kH + c + 1] = acc2[j][1];
        p[HELP_MLP_OFF_W2 + (m0 + g + 8) * kH + c] = acc2[j][2];
        p[HELP_MLP_OFF_W2 + (m0 + g + 8) * kH + c + 1] = acc2[j][3];
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int c = 8 * j + 2 * t;
        p[HELP_MLP_OFF_W1 + (m0 + g) * kF + c] = acc1[j][0];
        p[HELP_MLP_OFF_W1 + (m0 + g) * kF + c + 1] = acc1[j][1];
        p[HELP_MLP_OFF_W1 + (m0 + g + 8) * kF + c] = acc1[j][2];
        p[HELP_MLP_OFF_W1 + (m0 + g + 8) * kF + c + 1] = acc1[j][3];
        // dW3 rows are the outputs (only g < HELP_MLP_OUT exist), columns m0 + 8 j + 2 t
        if (g < HELP_MLP_OUT) {
            p[HELP_MLP_OFF_W3 + g * kH + m0 + c] = acc3[j][0];
            p[HELP_MLP_OFF_W3 + g * kH + m0 + c + 1] = acc3[j][1];
        }
    }
    if (warp == 0) {
        p[HELP_MLP_OFF_B2 + lane] = bsum0;
        p[HELP_MLP_OFF_B2 + lane + 32] = bsum1;
    } else if (warp == 1) {
        p[HELP_MLP_OFF_B1 + lane] = bsum0;
        p[HELP_MLP_OFF_B1 + lane + 32] = bsum1;
    } else if (warp == 2 && lane < HELP_MLP_OUT) {
        p[HELP_MLP_OFF_B3 + lane] = bsum0;
    }
}

// grad[j] = sum over blocks (in order) of part[b][j]
__global__ void k_mlp_grad_reduce(const float* __restrict__ part, int nblk, float* __restrict__ grad) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < kMlpGradParams; j += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nblk; ++b) s += part[(size_t)b * kMlpGradParams + j];
        grad[j] = s;
    }
}

// Adam on the trainable parameters; refreshes the BF16 / FP32 device weights.
__global__ void k_mlp_adam(float* __restrict__ prm, float* __restrict__ m1, float* __restrict__ m2,
                           const float* __restrict__ grad, float lr, float bc1, float bc2, MlpDevWeights* w) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < kMlpGradParams; j += gridDim.x * blockDim.x) {
        const float gj = grad[j];
        const float a = 0.9f * m1[j] + 0.1f * gj;
        const float b = 0.999f * m2[j] + 0.001f * gj * gj;
        m1[j] = a;
        m2[j] = b;
        const float v = prm[j] - lr * (a / bc1) / (sqrtf(b / bc2) + 1e-8f);
        prm[j] = v;
        mlp_store_param(w, j, v);
    }
}

__global__ void k_mlp_upload(const float* __restrict__ prm, MlpDevWeights* w) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < kMlpGradParams; j += gridDim.x * blockDim.x)
        mlp_store_param(w, j, prm[j]);
    if (blockIdx.x == 0 && threadIdx.x < 16) {
        w->mean[threadIdx.x] = prm[HELP_MLP_OFF_MEAN + threadIdx.x];
        w->scale[threadIdx.x] = prm[HELP_MLP_OFF_SCALE + threadIdx.x];
    }
}

}  // namespace

// ---- launchers (mlp.h)
int mlp_blocks(long long rows, int num_sms) {
    const long long tiles = (rows + 63) / 64;
    long long b = tiles < 1 ? 1 : tiles;
    if (b > 4LL * num_sms) b = 4LL * num_sms;
    return (int)b;
}

cudaError_t mlp_forward(const __nv_bfloat16* X, long long rows, const MlpDevWeights* w, float* out,
                        __nv_bfloat16* H1, __nv_bfloat16* H2, int num_sms, cudaStream_t st) {
    if (rows <= 0) return cudaSuccess;
    const int nb = mlp_blocks(rows, num_sms);
    if (H1) {
        k_mlp_fwd<true><<<nb, kMlpThreads, 0, st>>>(X, rows, w, out, H1, H2);
    } else {
        // inference: the tcgen05 kernel, 128-row tiles, 6 CTAs per SM (the
        // most its shared memory allows; 6 x 64 TMEM columns of the SM's 512,
        // so an allocation never waits)
        const long long tiles = (rows + kTcRows - 1) / kTcRows;
        const int tb = (int)std::min<long long>(tiles, 6LL * num_sms);
        const bool x16 = (reinterpret_cast<uintptr_t>(X) & 15u) == 0;
        k_mlp_fwd_tc<<<tb, kTcThreads, sizeof(TcSmem), st>>>(X, rows, w, out, x16);
    }
    return cudaGetLastError();
}

cudaError_t mlp_configure() {
    return raise_smem_limit((const void*)k_mlp_bwd, (int)sizeof(BwdSmem));
}

cudaError_t mlp_loss_grad(const __nv_bfloat16* X, long long rows, const MlpDevWeights* w, const float* out,
                          const float* tg, const float* wt, float* G3, const __nv_bfloat16* H1,
                          const __nv_bfloat16* H2, double* lpart, float* gpart, float* grad, int num_sms,
                          cudaStream_t st) {
    const long long n = rows * HELP_MLP_OUT;
    k_mlp_wsum<<<kMlpLossBlocks, 256, 0, st>>>(wt, n, lpart + kMlpLossBlocks);
    k_mlp_loss<<<kMlpLossBlocks, 256, 0, st>>>(out, tg, wt, n, lpart + kMlpLossBlocks, kMlpLossBlocks, G3, lpart);
    const int nb = mlp_blocks(rows, num_sms);
    k_mlp_bwd<<<nb, kMlpThreads, sizeof(BwdSmem), st>>>(X, rows, w, G3, H1, H2, gpart);
    k_mlp_grad_reduce<<<(kMlpGradParams + 255) / 256, 256, 0, st>>>(gpart, nb, grad);
    return cudaGetLastError();
}

cudaError_t mlp_adam(float* prm, float* m1, float* m2, const float* grad, float lr, int step, MlpDevWeights* w,
                     cudaStream_t st) {
    const float bc1 = 1.f - powf(0.9f, (float)step), bc2 = 1.f - powf(0.999f, (float)step);
    k_mlp_adam<<<(kMlpGradParams + 255) / 256, 256, 0, st>>>(prm, m1, m2, grad, lr, bc1, bc2, w);
    return cudaGetLastError();
}

cudaError_t mlp_upload(const float* prm, MlpDevWeights* w, cudaStream_t st) {
    k_mlp_upload<<<(kMlpGradParams + 255) / 256, 256, 0, st>>>(prm, w);
    return cudaGetLastError();
}

}  // namespace help
