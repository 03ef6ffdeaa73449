// Host-side planning of one CSR matrix for spmv_rows (spmv.cuh).
//
// G, the number of lanes that share a short row, is the smallest power of two
// (at least g_min, at most 32) giving each lane at most `per_lane` nonzeros of
// an average row.  Rows up to 32 G nonzeros are short; rows up to kLongRowMin
// are taken one warp each; longer rows are cut into segments of kSegLen
// nonzeros, one CTA per segment, so one row of 250k nonzeros (a pivot column
// of a Zipf matrix's Schur block) does not hold a whole launch behind one CTA.
// Medium rows, long rows and segments are listed explicitly.
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
    return p;
}

}  // namespace help
