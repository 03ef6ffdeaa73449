// CSR sparse matrix-vector products: y_r = sum_e val[e] * x[idx[e]] per row.
//
// The reference's CSRMV_N / CSRMV_T (Helper.cpp:57-81) are serial loops and
// the transpose product is a scatter.  Here A^T lives in HBM as its own CSR
// (= CSC of A), so both A x and A^T x are row gathers with this one routine.
//
// Rows are split by length when the matrix is planned (host, once per matrix
// and precision; see items.cpp):
//   * short rows (len <= short_max = 32 G): a group of G lanes per row, G a
//     power of two (at least 2) chosen so each lane handles <= 7 (FP64) or 4
//     (FP32) nonzeros of an average row.  A warp covers 32 / G rows -- in
//     index order, so its loads sweep one contiguous span of the value and
//     index arrays, or, for matrices whose row lengths vary a lot, by
//     decreasing length within windows of consecutive rows (short_order) so a
//     warp's rows finish together; each lane keeps one FMA accumulator and
//     the group combines with log2(G) shuffles;
//   * medium rows (short_max < len <= kLongRowMin): one warp per row;
//   * long rows (len > kLongRowMin): cut into segments of kSegLen nonzeros,
//     one CTA per segment.  Each CTA writes its segment's sum to a partial
//     slot and takes a ticket on the row; the CTA that takes the last ticket
//     adds the row's partials in segment order (deterministic), resets the
//     ticket and runs the epilogue.  No CTA waits for another.
// Short rows go through the sliced layout where the matrix has one (B = A
// D^-1/2 of A and A^T), else through L1 (read-only path) so the neighbouring
// elements a group reads next reuse the sectors already fetched; medium and
// long rows are read in aligned pairs (range_dot).  All loops are grid-stride
// over every warp / block of the launch, so the same routine serves the
// standalone kernels, the CG graph kernels and the single-cluster CG kernel.  One FMA per
// nonzero and few shuffle adds matter on GB300, whose FP64 rate (~2
// DFMA/clk/SM) is close to the HBM rate for SpMV.
#pragma once

#include "common.cuh"
#include "items.h"

namespace help {

// Device view of one planned CSR matrix.
template <class V>
struct SpmvView {
    int rows;
    int G;          // lanes per short row (power of two, 1..32)
    int short_max;  // rows longer than this are in med_rows or long_rows
    int n_med, n_long;
    const int* ptr;
    const int* idx;
    const V* val;
    const int* med_rows;   // warp-per-row
    const int* long_rows;  // rows longer than kLongRowMin, ascending
    // segments of the long rows (items.h): {row, begin, end, long-row index}
    int n_seg = 0;
    const int4* segs = nullptr;
    const int* long_nseg = nullptr;
    const int* long_base = nullptr;
    unsigned int* tickets = nullptr;  // one per long row, zero between launches
    double* parts = nullptr;          // partial sums of the segments
    // short rows in processing order (null: index order, non-short rows skipped)
    const int* short_order = nullptr;
    int n_short = 0;
    // short rows in the sliced layout (items.h, SellHost); n_sell = 0: the
    // CSR short-row loop instead
    int n_sell = 0;
    int sell_W = 1;
    const int* sell_ptr = nullptr;
    const int* sell_perm = nullptr;
    const int* sell_idx = nullptr;
    const V* sell_val = nullptr;
};

// Short rows in the sliced layout: one lane per row, a slice of 32 rows per
// group of W warps of the CTA (warp `sub` of the group takes step blocks
// sub, sub + W, ...; each step block is kSellStep entries read with one
// vector load of indices and one of values); the W partial sums of a row
// are added in warp order through shared memory (red: the CTA's blockDim
// doubles) by the group's first warp, which runs the epilogue.  One FMA per
// entry and no shuffle reductions: GB300's FP64 pipe (~2 lanes / clk / SM)
// is close to the HBM rate of these passes.  Every thread of the CTA must
// call it (it synchronises the CTA).  kDepth (2 or 4): step blocks a lane
// has in flight (4 or 8 gathers); the sum runs over the lane's blocks in the
// same order either way, so the results are bitwise the same.  4 pays in
// the standalone pass (32 -> 40 registers, occupancy unchanged: config 1's
// B pass 23.9 -> 22.5 us), 2 in the CG kernels (their 40 registers would
// grow to 48 and cost a CTA per SM: config 1's iteration 83 -> 90 us).
template <class V, int kDepth, class XF, class EP>
HELP_DEVINL void spmv_sell(const SpmvView<V>& M, const XF& xf, const EP& ep, double* red) {
    static_assert(kDepth == 2 || kDepth == 4, "step blocks in flight: 2 or 4");
    using V2 = typename Vec2<V>::T;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int W = M.sell_W <= nw ? M.sell_W : nw;
    const int groups = nw / W, grp = warp / W, sub = warp - grp * W;
    const int* __restrict__ sidx = M.sell_idx;
    const V* __restrict__ sval = M.sell_val;
    constexpr int BS = 32 * kSellStep;  // entries per step block of a slice
    for (int base = blockIdx.x * groups; base < M.n_sell; base += gridDim.x * groups) {
        const int s = base + grp;
        V acc = V(0);
        if (grp < groups && s < M.n_sell) {
            const int b = ld_ro(M.sell_ptr + s), e = ld_ro(M.sell_ptr + s + 1);
            int q = b + sub * BS + lane * kSellStep;
            if constexpr (kDepth == 4) {
                for (; q + 3 * W * BS < e; q += 4 * W * BS) {
                    const int2 c0 = ld_stream_na(reinterpret_cast<const int2*>(sidx + q));
                    const int2 c1 = ld_stream_na(reinterpret_cast<const int2*>(sidx + q + W * BS));
                    const int2 c2 = ld_stream_na(reinterpret_cast<const int2*>(sidx + q + 2 * W * BS));
                    const int2 c3 = ld_stream_na(reinterpret_cast<const int2*>(sidx + q + 3 * W * BS));
                    const V x0 = xf(c0.x), x1 = xf(c0.y), x2 = xf(c1.x), x3 = xf(c1.y);
                    const V x4 = xf(c2.x), x5 = xf(c2.y), x6 = xf(c3.x), x7 = xf(c3.y);
                    const V2 v0 = ld_stream_na(reinterpret_cast<const V2*>(sval + q));
                    const V2 v1 = ld_stream_na(reinterpret_cast<const V2*>(sval + q + W * BS));
                    const V2 v2 = ld_stream_na(reinterpret_cast<const V2*>(sval + q + 2 * W * BS));
                    const V2 v3 = ld_stream_na(reinterpret_cast<const V2*>(sval + q + 3 * W * BS));
                    acc = fma_t(v0.x, x0, acc);
                    acc = fma_t(v0.y, x1, acc);
                    acc = fma_t(v1.x, x2, acc);
                    acc = fma_t(v1.y, x3, acc);
                    acc = fma_t(v2.x, x4, acc);
                    acc = fma_t(v2.y, x5, acc);
                    acc = fma_t(v3.x, x6, acc);
                    acc = fma_t(v3.y, x7, acc);
                }
            }
            for (; q + W * BS < e; q += 2 * W * BS) {  // after the loop above: at most once
                const int2 c0 = ld_stream_na(reinterpret_cast<const int2*>(sidx + q));
                const int2 c1 = ld_stream_na(reinterpret_cast<const int2*>(sidx + q + W * BS));
                const V2 v0 = ld_stream_na(reinterpret_cast<const V2*>(sval + q));
                const V2 v1 = ld_stream_na(reinterpret_cast<const V2*>(sval + q + W * BS));
                const V x0 = xf(c0.x), x1 = xf(c0.y), x2 = xf(c1.x), x3 = xf(c1.y);
                acc = fma_t(v0.x, x0, acc);
                acc = fma_t(v0.y, x1, acc);
                acc = fma_t(v1.x, x2, acc);
                acc = fma_t(v1.y, x3, acc);
            }
            if (q < e) {
                const int2 c0 = ld_stream_na(reinterpret_cast<const int2*>(sidx + q));
                const V2 v0 = ld_stream_na(reinterpret_cast<const V2*>(sval + q));
                const V x0 = xf(c0.x), x1 = xf(c0.y);
                acc = fma_t(v0.x, x0, acc);
                acc = fma_t(v0.y, x1, acc);
            }
        }
        if (W == 1) {
            if (s < M.n_sell) {
                const int r = ld_ro(M.sell_perm + 32 * s + lane);
                if (r >= 0) ep(r, acc);
            }
            continue;
        }
        __syncthreads();  // red is free (previous slice's sums read)
        red[threadIdx.x] = (double)acc;
        __syncthreads();
        if (sub == 0 && grp < groups && s < M.n_sell) {
            double t = red[threadIdx.x];
            for (int u = 1; u < W; ++u) t += red[threadIdx.x + 32 * u];
            const int r = ld_ro(M.sell_perm + 32 * s + lane);
            if (r >= 0) ep(r, (V)t);
        }
    }
}

// Sum over one contiguous range [b, e) of a CSR row by a team of T threads
// (t = the thread's place in it): entries in aligned pairs, one vector load
// of indices and one of values per pair, two pairs in flight per thread; the
// unpaired first and last entries by thread 0.
template <class V, class XF>
HELP_DEVINL V range_dot(const int* __restrict__ idx, const V* __restrict__ val, int b, int e, int t, int T,
                        const XF& xf) {
    using V2 = typename Vec2<V>::T;
    V acc = V(0);
    int q0 = b;
    if ((q0 & 1) && q0 < e) {
        if (t == 0) acc = fma_t(ld_ro(val + q0), xf(ld_ro(idx + q0)), acc);
        ++q0;
    }
    const int np = (e - q0) >> 1;
    const int2* __restrict__ ip = reinterpret_cast<const int2*>(idx + q0);
    const V2* __restrict__ vp = reinterpret_cast<const V2*>(val + q0);
    int p = t;
    for (; p + T < np; p += 2 * T) {
        const int2 c0 = ld_stream_na(ip + p), c1 = ld_stream_na(ip + p + T);
        const V2 v0 = ld_stream_na(vp + p), v1 = ld_stream_na(vp + p + T);
        const V x0 = xf(c0.x), x1 = xf(c0.y), x2 = xf(c1.x), x3 = xf(c1.y);
        acc = fma_t(v0.x, x0, acc);
        acc = fma_t(v0.y, x1, acc);
        acc = fma_t(v1.x, x2, acc);
        acc = fma_t(v1.y, x3, acc);
    }
    if (p < np) {
        const int2 c0 = ld_stream_na(ip + p);
        const V2 v0 = ld_stream_na(vp + p);
        const V x0 = xf(c0.x), x1 = xf(c0.y);
        acc = fma_t(v0.x, x0, acc);
        acc = fma_t(v0.y, x1, acc);
    }
    if (((e - q0) & 1) && t == 0) acc = fma_t(ld_ro(val + e - 1), xf(ld_ro(idx + e - 1)), acc);
    return acc;
}

//   xf(col)  -> V     value of the dense operand at index `col`
//   ep(row, sum)      epilogue for one finished row (called by one thread)
//   epl(row, sum)     the same for long rows; it runs in whichever CTA
//                     finishes the row last, so a kernel whose epilogue also
//                     accumulates a reduction passes an epl that only stores
//                     and adds the long rows' terms in a fixed order itself
// red: blockDim doubles of shared memory (CTA reductions of long rows).
template <class V, int kDepth = 2, class XF, class EP, class EPL>
HELP_DEVINL void spmv_rows(const SpmvView<V>& M, const XF& xf, const EP& ep, const EPL& epl, double* red) {
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nw = nthr >> 5;
    const int gw = blockIdx.x * nw + warp, tw = gridDim.x * nw;
    const int* __restrict__ ptr = M.ptr;
    const int* __restrict__ idx = M.idx;
    const V* __restrict__ val = M.val;
    __shared__ int s_last;

    // long rows: one CTA per segment
    for (int sg = blockIdx.x; sg < M.n_seg; sg += gridDim.x) {
        const int4 S = ld_ro(M.segs + sg);
        const int r = S.x, b = S.y, e = S.z, j = S.w;
        const V acc = range_dot<V>(idx, val, b, e, tid, nthr, xf);
        const double sum = block_sum((double)acc, red);
        const int nseg = ld_ro(M.long_nseg + j);
        if (nseg == 1) {
            if (tid == 0) epl(r, (V)sum);
            continue;
        }
        const int base = ld_ro(M.long_base + j);
        if (tid == 0) {
            M.parts[base + (b - ld_ro(ptr + r)) / kSegLen] = sum;
            __threadfence();
            const unsigned int t = atomicAdd(M.tickets + j, 1u);
            s_last = (t == (unsigned int)nseg - 1u);
        }
        __syncthreads();
        if (s_last && tid == 0) {
            __threadfence();
            double tot = 0.0;
            for (int k = 0; k < nseg; ++k) tot += __ldcg(M.parts + base + k);
            M.tickets[j] = 0u;
            epl(r, (V)tot);
        }
        __syncthreads();
    }

    // medium rows: one warp each
    for (int i = gw; i < M.n_med; i += tw) {
        const int r = ld_ro(M.med_rows + i);
        const int b = ld_ro(ptr + r), e = ld_ro(ptr + r + 1);
        V acc = range_dot<V>(idx, val, b, e, lane, 32, xf);
        acc = warp_sum(acc);
        if (lane == 0) ep(r, acc);
    }

    if (M.n_sell > 0) {
        spmv_sell<V, kDepth>(M, xf, ep, red);
        return;
    }
    // short rows: G lanes per row, 32 / G rows per warp step
    const int G = M.G, lg = __ffs(G) - 1;
    const int sub = lane & (G - 1), rpw = 32 >> lg;
    const bool ordered = M.short_order != nullptr;
    const int slots = ordered ? M.n_short : M.rows;
    for (int base = gw * rpw; base < slots; base += tw * rpw) {
        const int slot = base + (lane >> lg);
        const int r = (ordered && slot < slots) ? ld_ro(M.short_order + slot) : slot;
        int b = 0, e = 0;
        if (slot < slots) {
            b = ld_ro(ptr + r);
            e = ld_ro(ptr + r + 1);
        }
        const bool mine = (slot < slots) && (e - b <= M.short_max);
        if (!mine) e = b;
        V acc = V(0);
        int q = b + sub;
        for (; q + 3 * G < e; q += 4 * G) {
            const int c0 = ld_ro(idx + q), c1 = ld_ro(idx + q + G);
            const int c2 = ld_ro(idx + q + 2 * G), c3 = ld_ro(idx + q + 3 * G);
            const V v0 = ld_ro(val + q), v1 = ld_ro(val + q + G);
            const V v2 = ld_ro(val + q + 2 * G), v3 = ld_ro(val + q + 3 * G);
            const V x0 = xf(c0), x1 = xf(c1), x2 = xf(c2), x3 = xf(c3);
            acc = fma_t(v0, x0, acc);
            acc = fma_t(v1, x1, acc);
            acc = fma_t(v2, x2, acc);
            acc = fma_t(v3, x3, acc);
        }
        for (; q < e; q += G) acc = fma_t(ld_ro(val + q), xf(ld_ro(idx + q)), acc);
        for (int o = G >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (mine && sub == 0) ep(r, acc);
    }
}

template <class V, int kDepth = 2, class XF, class EP>
HELP_DEVINL void spmv_rows(const SpmvView<V>& M, const XF& xf, const EP& ep, double* red) {
    spmv_rows<V, kDepth>(M, xf, ep, ep, red);
}

}  // namespace help
