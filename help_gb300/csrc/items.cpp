// Host-side planning of SpMV work items for one CSR matrix (see spmv.cuh).
//
// Rows longer than `cap` become single-row items (processed CTA-wide) and are
// listed first so they start early; the other rows are packed in order into
// blocks of consecutive rows with at most `cap` nonzeros and at most
// `max_rows` rows each.  Items are int4 {row0, row1 | flags, e0, e1}.
#include "items.h"

#include <algorithm>

namespace help {

std::vector<Int4> plan_items(const int32_t* ptr, int32_t rows, int32_t cap, int32_t max_rows,
                             int32_t thread_row_max) {
    std::vector<Int4> longs, shorts;
    int32_t start = -1;
    bool has_long = false;
    auto close = [&](int32_t end_row) {
        if (start >= 0) {
            shorts.push_back({start, end_row | (has_long ? kItemHasLongRowsHost : 0), ptr[start], ptr[end_row]});
            start = -1;
            has_long = false;
        }
    };
    for (int32_t i = 0; i < rows; ++i) {
        const int32_t len = ptr[i + 1] - ptr[i];
        if (len > cap) {
            close(i);
            longs.push_back({i, i + 1, ptr[i], ptr[i + 1]});
            continue;
        }
        if (start >= 0 && (ptr[i + 1] - ptr[start] > cap || i - start >= max_rows)) close(i);
        if (start < 0) start = i;
        if (len > thread_row_max) has_long = true;
    }
    close(rows);
    longs.insert(longs.end(), shorts.begin(), shorts.end());
    return longs;
}

}  // namespace help
