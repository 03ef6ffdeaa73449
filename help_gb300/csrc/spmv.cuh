// CSR sparse matrix-vector products over planned work items.
//
// The reference's CSRMV_N / CSRMV_T (Helper.cpp:57-81) are serial loops; the
// transpose product is a scatter.  Here both A x and A^T x are row gathers:
// A^T lives in HBM as its own CSR (= CSC of A), so every product is
// "for each row: sum_e val[e] * x[idx[e]]".
//
// Work items (planned once per matrix on the host, see items.cpp) are either
//   * a block of consecutive rows holding at most `cap` nonzeros: all threads
//     of the CTA stream the block's values and indices with coalesced loads
//     and gather the matching x entries (every load independent, so many are
//     in flight per thread), storing value and x side by side in shared
//     memory; then each thread accumulates one row from shared memory with
//     one fused multiply-add per nonzero (rows longer than kThreadRowMax
//     inside the block are taken warp-per-row), or
//   * one row longer than `cap`, which the whole CTA reduces.
// One FMA per nonzero and no shuffle reductions for short rows matter on
// GB300, whose FP64 rate (~2 DFMA/clk/SM) is close to the HBM rate for SpMV.
#pragma once

#include "common.cuh"

namespace help {

constexpr int kItemHasLongRows = 1 << 30;  // flag in item.y: some row > kThreadRowMax
constexpr int kItemRowMask = (1 << 30) - 1;
constexpr int kThreadRowMax = 48;

// Shared-memory bytes spmv_items needs for a given cap.
template <class V>
constexpr size_t spmv_smem_bytes(int cap) {
    return (size_t)cap * 2 * sizeof(V);
}

// Process items first, first + stride, ... of the list.
//   xf(col)       -> V      value of the dense operand at index `col`
//   ep(row, sum)             epilogue for one finished row (called by one thread)
// s_val / s_x: shared staging of `cap` entries each; red: blockDim/32 doubles.
template <class V, class XF, class EP>
HELP_DEVINL void spmv_items(const int4* __restrict__ items, int n_items, int first, int stride,
                            const int* __restrict__ ptr, const int* __restrict__ idx,
                            const V* __restrict__ val, int cap, const XF& xf, const EP& ep, V* s_val,
                            V* s_x, double* red) {
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
    for (int it = first; it < n_items; it += stride) {
        const int4 w = ld_ro(items + it);
        const int row0 = w.x, row1 = w.y & kItemRowMask;
        const int e0 = w.z, e1 = w.w;
        if (e1 - e0 > cap) {
            // one long row: strided FMA per thread, deterministic block reduction
            V acc = V(0);
            int e = e0 + tid;
            for (; e + 3 * nthr < e1; e += 4 * nthr) {
                const int c0 = ld_stream(idx + e), c1 = ld_stream(idx + e + nthr);
                const int c2 = ld_stream(idx + e + 2 * nthr), c3 = ld_stream(idx + e + 3 * nthr);
                const V v0 = ld_stream(val + e), v1 = ld_stream(val + e + nthr);
                const V v2 = ld_stream(val + e + 2 * nthr), v3 = ld_stream(val + e + 3 * nthr);
                const V x0 = xf(c0), x1 = xf(c1), x2 = xf(c2), x3 = xf(c3);
                acc = fma_t(v0, x0, acc);
                acc = fma_t(v1, x1, acc);
                acc = fma_t(v2, x2, acc);
                acc = fma_t(v3, x3, acc);
            }
            for (; e < e1; e += nthr) acc = fma_t(ld_stream(val + e), xf(ld_stream(idx + e)), acc);
            const double s = block_sum((double)acc, red);
            if (tid == 0) ep(row0, (V)s);
            continue;
        }
        const int ne = e1 - e0;
        {
            int e = tid;
            for (; e + 3 * nthr < ne; e += 4 * nthr) {
                const int c0 = ld_stream(idx + e0 + e), c1 = ld_stream(idx + e0 + e + nthr);
                const int c2 = ld_stream(idx + e0 + e + 2 * nthr), c3 = ld_stream(idx + e0 + e + 3 * nthr);
                const V v0 = ld_stream(val + e0 + e), v1 = ld_stream(val + e0 + e + nthr);
                const V v2 = ld_stream(val + e0 + e + 2 * nthr), v3 = ld_stream(val + e0 + e + 3 * nthr);
                const V x0 = xf(c0), x1 = xf(c1), x2 = xf(c2), x3 = xf(c3);
                s_val[e] = v0, s_val[e + nthr] = v1, s_val[e + 2 * nthr] = v2, s_val[e + 3 * nthr] = v3;
                s_x[e] = x0, s_x[e + nthr] = x1, s_x[e + 2 * nthr] = x2, s_x[e + 3 * nthr] = x3;
            }
            for (; e < ne; e += nthr) {
                const int c = ld_stream(idx + e0 + e);
                s_val[e] = ld_stream(val + e0 + e);
                s_x[e] = xf(c);
            }
        }
        __syncthreads();
        const int nr = row1 - row0;
        for (int r = tid; r < nr; r += nthr) {
            const int b = ld_ro(ptr + row0 + r) - e0, e = ld_ro(ptr + row0 + r + 1) - e0;
            if (e - b <= kThreadRowMax) {
                V acc = V(0);
                for (int q = b; q < e; ++q) acc = fma_t(s_val[q], s_x[q], acc);
                ep(row0 + r, acc);
            }
        }
        if (w.y & kItemHasLongRows) {
            for (int r = warp; r < nr; r += nwarps) {
                const int b = ld_ro(ptr + row0 + r) - e0, e = ld_ro(ptr + row0 + r + 1) - e0;
                if (e - b > kThreadRowMax) {
                    V acc = V(0);
                    for (int q = b + lane; q < e; q += 32) acc = fma_t(s_val[q], s_x[q], acc);
                    acc = warp_sum(acc);
                    if (lane == 0) ep(row0 + r, acc);
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace help
