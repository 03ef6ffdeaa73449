#pragma once
#include <stdint.h>

#include <vector>

namespace help {

struct Int4 {
    int32_t x, y, z, w;
};
static_assert(sizeof(Int4) == 16, "Int4 must match the device int4 layout");

constexpr int32_t kItemHasLongRowsHost = 1 << 30;  // must equal kItemHasLongRows (spmv.cuh)

std::vector<Int4> plan_items(const int32_t* ptr, int32_t rows, int32_t cap, int32_t max_rows,
                             int32_t thread_row_max);

}  // namespace help
