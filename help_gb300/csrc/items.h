#pragma once
#include <stdint.h>

#include <vector>

namespace help {

// Host-side split of the rows of one CSR matrix for spmv_rows (spmv.cuh).
struct RowPlanHost {
    int32_t G = 1;          // lanes per short row
    int32_t short_max = 32; // longer rows are medium or long
    std::vector<int32_t> med, lng;
    // long rows cut into segments of at most kSegLen nonzeros, one CTA each:
    // seg = {row, begin, end, long-row index j}; row j's partial sums go to
    // slots long_base[j] .. long_base[j] + long_nseg[j] - 1
    std::vector<int32_t> seg;  // 4 ints per segment
    std::vector<int32_t> long_nseg, long_base;
    int32_t n_parts = 0;
    // short rows in processing order when their lengths are uneven (empty:
    // all rows in index order, non-short ones skipped)
    std::vector<int32_t> short_order;
    double warp_waste = 1.0;  // lane-steps of the chosen order over the useful ones
};

constexpr int32_t kLongRowMin = 4096;  // rows above this length are long
constexpr int32_t kSegLen = 16384;     // nonzeros per segment of a long row (one CTA)
constexpr int32_t kOrderWindow = 4096; // short rows are reordered only within windows of this many rows
constexpr double kOrderWaste = 1.5;    // reorder when index order wastes this factor of lane steps
// C = G[N, P] is rebuilt at every renew and its pass is bound by the FP64
// pipe, which a warp's idle lanes still occupy: reorder at a smaller waste
// (config 4's C: rows of ~85 entries, ~1.14 in index order)
constexpr double kOrderWasteC = 1.05;

// g_min: smallest group; per_lane: target nonzeros per lane of an average row;
// short rows are reordered when index order wastes more than order_waste.
RowPlanHost plan_rows(const int32_t* ptr, int32_t rows, int32_t g_min, int32_t per_lane,
                      double order_waste = kOrderWaste);

// Sliced layout of the short rows (length <= short_max) of one CSR matrix:
// rows taken by decreasing length within windows of kOrderWindow rows, 32
// per slice (one lane each), every slice padded to its longest row (rounded
// up to kSellStep); entry j of the row in lane r of slice s sits at
//   ptr[s] + (j / kSellStep) * 32 * kSellStep + r * kSellStep + j % kSellStep,
// so a lane reads kSellStep consecutive entries with one vector load and a
// warp's loads are contiguous.  perm[32 s + r] is the row (-1: no row); map
// holds each entry's CSR position (-1: padding, value 0, index repeating the
// row's last column).  W warps share a slice (each takes every W-th step
// block) when slices are long: W = largest power of two <= mean slice
// length / 8, at most 8.
struct SellHost {
    int32_t nslices = 0, W = 1;
    std::vector<int32_t> ptr, perm, idx, map;
};
constexpr int32_t kSellStep = 2;
// Empty result (nslices = 0) when there are no short rows or the layout
// would pass 2^31 entries.
SellHost plan_sell(const int32_t* ptr, const int32_t* idx, int32_t rows, int32_t short_max);

}  // namespace help
