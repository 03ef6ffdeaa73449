// Host-side planning of one CSR matrix for spmv_rows (spmv.cuh).
//
// G, the number of lanes that share a short row, is the smallest power of two
// (at least g_min, at most 32) giving each lane at most `per_lane` nonzeros of
// an average row.  Rows up to 32 G nonzeros are short; rows up to kLongRowMin
// are taken one warp each; longer rows are cut into segments of kSegLen
// nonzeros, one CTA per segment, so one row of 250k nonzeros (a pivot column
// of a Zipf matrix's Schur block) does not hold a whole launch behind one CTA.
// Medium rows, long rows and segments are listed explicitly.
//
// A warp walks 32 / G short rows together until the longest is done, and on
// GB300 an FP64 instruction costs its issue slots whatever lanes are active,
// so rows of very uneven length next to each other waste the FP64 pipe (the
// Schur block of a Zipf matrix: median row 7, some 900).  When index order
// wastes more than kOrderWaste of the lane steps, short rows are processed by
// decreasing length within windows of kOrderWindow consecutive rows, which
// keeps a warp's rows' vector entries close together.
#include "items.h"

#include <algorithm>

namespace help {

// Appends the rows r in [w0, w1) with length <= max_len by decreasing length,
// rows of equal length in index order (a stable counting sort: O(rows +
// max_len) per window, against O(rows log rows) for a comparison sort --
// 1.92M rows of C per renew in ~10 ms instead of ~140 ms).
static void append_by_length(const int32_t* ptr, int32_t w0, int32_t w1, int32_t max_len, std::vector<int32_t>& cnt,
                             std::vector<int32_t>& out) {
    cnt.assign((size_t)max_len + 2, 0);
    for (int32_t r = w0; r < w1; ++r) {
        const int32_t len = ptr[r + 1] - ptr[r];
        if (len <= max_len) ++cnt[(size_t)(max_len - len) + 1];  // bucket 0: the longest
    }
    for (size_t b = 1; b < cnt.size(); ++b) cnt[b] += cnt[b - 1];
    const size_t base = out.size();
    out.resize(base + (size_t)cnt.back());
    for (int32_t r = w0; r < w1; ++r) {
        const int32_t len = ptr[r + 1] - ptr[r];
        if (len <= max_len) out[base + (size_t)cnt[(size_t)(max_len - len)]++] = r;
    }
}

RowPlanHost plan_rows(const int32_t* ptr, int32_t rows, int32_t g_min, int32_t per_lane, double order_waste) {
    RowPlanHost p;
    int64_t tot = 0, cnt = 0;
    for (int32_t i = 0; i < rows; ++i) {
        const int32_t len = ptr[i + 1] - ptr[i];
        if (len <= kLongRowMin) {
            tot += len;
            ++cnt;
        }
    }
    const double avg = cnt ? (double)tot / (double)cnt : 0.0;
    int32_t G = 1;
    while (G < g_min) G *= 2;
    while (G < 32 && G * per_lane < avg) G *= 2;
    p.G = G;
    p.short_max = 32 * G;
    for (int32_t i = 0; i < rows; ++i) {
        const int32_t len = ptr[i + 1] - ptr[i];
        if (len > kLongRowMin) {
            const int32_t j = (int32_t)p.lng.size();
            const int32_t nseg = (len + kSegLen - 1) / kSegLen;
            p.lng.push_back(i);
            p.long_nseg.push_back(nseg);
            p.long_base.push_back(p.n_parts);
            p.n_parts += nseg;
            for (int32_t s = 0; s < nseg; ++s) {
                const int32_t b = ptr[i] + s * kSegLen;
                const int32_t e = (s + 1 == nseg) ? ptr[i + 1] : b + kSegLen;
                p.seg.insert(p.seg.end(), {i, b, e, j});
            }
        } else if (len > p.short_max) {
            p.med.push_back(i);
        }
    }
    // lane steps of a warp group = rows per warp x steps of its longest row
    const int32_t rpw = 32 / G;
    auto steps = [&](int32_t r) -> int64_t {
        const int32_t len = ptr[r + 1] - ptr[r];
        return len <= p.short_max ? (len + G - 1) / G : 0;
    };
    int64_t useful = 0, index_cost = 0;
    for (int32_t b = 0; b < rows; b += rpw) {
        int64_t mx = 0;
        for (int32_t r = b; r < std::min(rows, b + rpw); ++r) {
            const int64_t st = steps(r);
            useful += st;
            mx = std::max(mx, st);
        }
        index_cost += mx * rpw;
    }
    if (useful > 0 && (double)index_cost > order_waste * (double)useful) {
        std::vector<int32_t> cnt;
        for (int32_t w0 = 0; w0 < rows; w0 += kOrderWindow)
            append_by_length(ptr, w0, std::min(rows, w0 + kOrderWindow), p.short_max, cnt, p.short_order);
        int64_t cost = 0;
        for (size_t b = 0; b < p.short_order.size(); b += rpw) {
            int64_t mx = 0;
            for (size_t q = b; q < std::min(p.short_order.size(), b + rpw); ++q) mx = std::max(mx, steps(p.short_order[q]));
            cost += mx * rpw;
        }
        p.warp_waste = (double)cost / (double)useful;
    } else if (useful > 0) {
        p.warp_waste = (double)index_cost / (double)useful;
    }
    return p;
}

SellHost plan_sell(const int32_t* ptr, const int32_t* idx, int32_t rows, int32_t short_max) {
    SellHost h;
    std::vector<int32_t> order, cnt;
    order.reserve((size_t)rows);
    for (int32_t w0 = 0; w0 < rows; w0 += kOrderWindow)
        append_by_length(ptr, w0, std::min(rows, w0 + kOrderWindow), short_max, cnt, order);
    if (order.empty()) return h;
    const int64_t ns = ((int64_t)order.size() + 31) / 32;
    std::vector<int32_t> sp((size_t)ns + 1);
    int64_t tot = 0, len_sum = 0;
    for (int64_t s = 0; s < ns; ++s) {
        int32_t mx = 0;
        for (int64_t q = 32 * s; q < std::min<int64_t>((int64_t)order.size(), 32 * s + 32); ++q)
            mx = std::max(mx, ptr[order[q] + 1] - ptr[order[q]]);
        mx = (mx + kSellStep - 1) / kSellStep * kSellStep;
        if (tot > (int64_t)0x7fffffff - 32 * (int64_t)mx) return SellHost();
        sp[(size_t)s] = (int32_t)tot;
        tot += 32 * (int64_t)mx;
        len_sum += mx;
    }
    sp[(size_t)ns] = (int32_t)tot;
    h.nslices = (int32_t)ns;
    const double mean = (double)len_sum / (double)ns;
    while (h.W < 8 && 8.0 * (h.W * 2) <= mean) h.W *= 2;
    h.ptr = std::move(sp);
    h.perm.assign((size_t)ns * 32, -1);
    h.idx.assign((size_t)tot, 0);
    h.map.assign((size_t)tot, -1);
    for (int64_t s = 0; s < ns; ++s) {
        const int64_t base = h.ptr[(size_t)s], len = (h.ptr[(size_t)s + 1] - base) / 32;
        for (int32_t r = 0; r < 32; ++r) {
            const int64_t q = 32 * s + r;
            if (q >= (int64_t)order.size()) break;
            const int32_t row = order[(size_t)q], b = ptr[row], n = ptr[row + 1] - b;
            h.perm[(size_t)q] = row;
            const int32_t pad_col = n > 0 ? idx[b + n - 1] : 0;
            for (int64_t j = 0; j < len; ++j) {
                const int64_t at = base + (j / kSellStep) * 32 * kSellStep + r * kSellStep + j % kSellStep;
                if (j < n) {
                    h.idx[(size_t)at] = idx[b + j];
                    h.map[(size_t)at] = b + (int32_t)j;
                } else {
                    h.idx[(size_t)at] = pad_col;
                }
            }
        }
    }
    return h;
}

}  // namespace help
