// Host-side planning of one CSR matrix for spmv_rows (spmv.cuh).
//
// G, the number of lanes that share a short row, is the smallest power of two
// (at least g_min, at most 32) giving each lane at most `per_lane` nonzeros of
// an average row.  Rows up to 32 G nonzeros are short; rows up to kLongRowMin
// are taken one warp each; longer rows one CTA each.  Medium and long rows are
// listed explicitly.
#include "items.h"

namespace help {

RowPlanHost plan_rows(const int32_t* ptr, int32_t rows, int32_t g_min, int32_t per_lane) {
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
        if (len > kLongRowMin) p.lng.push_back(i);
        else if (len > p.short_max) p.med.push_back(i);
    }
    return p;
}

}  // namespace help
