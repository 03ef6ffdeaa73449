// Explicit upper triangle of A diag(w) A^T -- ADAt_Allocate + ADAt_Calc
// (Helper.cpp:215-377), the assembly the reference's direct backends time.
//
// Row i of the triangle collects, for every entry (i, j) of A and every entry
// (k, j) of column j with k >= i, the product A_ij w_j A_kj.  The reference
// accumulates these into a dense per-thread array in exactly that order
// (row entries by increasing j, each column downward).  Here one warp owns
// one row: it gathers the row's contributions into shared memory tagged with
// (k, generation index), bitonic-sorts them and sums each run of equal k in
// generation order, with the multiply and add rounded separately as the
// reference's loops do; columns come out sorted inside each row.
//
// Rows with more than kAdatCap contributions (the Zipf rows of a skewed
// matrix, the dense linking rows of a block-angular one) take a second
// kernel: one warp per heavy row walks the row's entries in order and, for
// each, the column's entries k >= i, adding A_ij w_j A_kj into a dense
// accumulator over the row's column range [i, kmax] -- the reference's own
// dense per-thread accumulator (Helper.cpp:210-211, :350-377), in the same
// order (one column at a time; inside a column every k is distinct, so the
// lanes never add to the same entry) -- and marks k in a bitmap; the bitmap,
// read word by word, gives the columns in increasing order.  Each warp has
// its own accumulator slot in global memory (acc[R] doubles, stamp[R] ints
// marking which row last wrote an entry, so nothing is cleared between rows,
// and R/32 bitmap words cleared as they are read), R the widest heavy row's
// range.
#include "common.cuh"
#include "kernels.h"

namespace help {

namespace {

constexpr int kAdatCap = 2048;
constexpr int kAdatWarps = 4;

__device__ __forceinline__ int next_pow2(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

// Gather (key, value) contributions of row i; returns the count (may exceed cap).
template <bool VALUES>
__device__ int adat_gather(int i, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ av,
                           const int* __restrict__ cp, const int* __restrict__ ri, const double* __restrict__ avT,
                           const double* __restrict__ wv, unsigned long long* keys, double* vals) {
    const int lane = threadIdx.x & 31;
    int count = 0;
    for (int e = rp[i]; e < rp[i + 1]; ++e) {
        const int j = ci[e];
        const int qb = cp[j], qe = cp[j + 1];
        // first position in column j with row >= i (rows sorted): binary search
        int lo = qb, hi = qe;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (ri[mid] < i) lo = mid + 1;
            else hi = mid;
        }
        double vd = 0.0;
        if (VALUES) vd = __dmul_rn(av[e], wv[j]);
        for (int q = lo + lane; q < qe; q += 32) {
            const int o = count + (q - lo);
            if (o < kAdatCap) {
                keys[o] = ((unsigned long long)(unsigned)ri[q] << 32) | (unsigned)o;
                if (VALUES) vals[o] = __dmul_rn(vd, avT[q]);
            }
        }
        count += qe - lo;
    }
    __syncwarp();
    return count;
}

__device__ void warp_bitonic(unsigned long long* keys, double* vals, int n, bool with_vals) {
    const int lane = threadIdx.x & 31;
    for (int size = 2; size <= n; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = lane; t < n / 2; t += 32) {
                const int a = 2 * t - (t & (stride - 1));
                const int b = a + stride;
                const bool up = ((a & size) == 0);
                const unsigned long long ka = keys[a], kb = keys[b];
                if ((ka > kb) == up) {
                    keys[a] = kb;
                    keys[b] = ka;
                    if (with_vals) {
                        const double va = vals[a];
                        vals[a] = vals[b];
                        vals[b] = va;
                    }
                }
            }
            __syncwarp();
        }
    }
}

template <bool FILL>
__global__ void k_adat(const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ av,
                       const int* __restrict__ cp, const int* __restrict__ ri, const double* __restrict__ avT,
                       const double* __restrict__ wv, int m, int* __restrict__ cnt, const int* __restrict__ out_rp,
                       int* __restrict__ out_ci, double* __restrict__ out_v) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const size_t per = (size_t)kAdatCap * (8 + (FILL ? 8 : 0));
    unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem + per * warp);
    double* vals = reinterpret_cast<double*>(keys + kAdatCap);
    for (int64_t i = (int64_t)blockIdx.x * nw + warp; i < m; i += (int64_t)gridDim.x * nw) {
        const int n = adat_gather<FILL>((int)i, rp, ci, av, cp, ri, avT, wv, keys, vals);
        if (n > kAdatCap) {
            if (!FILL && lane == 0) cnt[i] = -1;
            continue;
        }
        const int np = next_pow2(n);
        for (int t = n + lane; t < np; t += 32) keys[t] = ~0ull;
        __syncwarp();
        warp_bitonic(keys, vals, np, FILL);
        // runs of equal column: lane-parallel head flags, sequential sums per run
        int pos = FILL ? out_rp[i] : 0;
        for (int base = 0; base < n; base += 32) {
            const int t = base + lane;
            const bool head = (t < n) && (t == 0 || (keys[t] >> 32) != (keys[t - 1] >> 32));
            const unsigned ball = __ballot_sync(0xffffffffu, head);
            if (FILL && head) {
                const unsigned kcol = (unsigned)(keys[t] >> 32);
                double s = 0.0;
                for (int u = t; u < n && (unsigned)(keys[u] >> 32) == kcol; ++u) s = __dadd_rn(s, vals[u]);
                const int o = pos + __popc(ball & ((1u << lane) - 1u));
                out_ci[o] = (int)kcol;
                out_v[o] = s;
            }
            pos += __popc(ball);
        }
        if (!FILL && lane == 0) cnt[i] = pos;
        __syncwarp();
    }
}

// kmax of each heavy row: the last row of every column it touches (rows are
// sorted inside columns), so its output columns lie in [i, kmax].
__global__ void k_adat_heavy_range(const int* __restrict__ heavy, int nh, const int* __restrict__ rp,
                                   const int* __restrict__ ci, const int* __restrict__ cp, const int* __restrict__ ri,
                                   int* __restrict__ range) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int h = blockIdx.x * nw + warp; h < nh; h += gridDim.x * nw) {
        const int i = heavy[h];
        int mx = i;
        for (int e = rp[i] + lane; e < rp[i + 1]; e += 32) {
            const int j = ci[e];
            if (cp[j + 1] > cp[j]) mx = max(mx, ri[cp[j + 1] - 1]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) range[h] = mx - i + 1;
    }
}

// One warp per heavy row, slot = the warp's index in the grid (the grid has
// at most `slots` warps).  Count pass: the number of distinct k (lanes take
// row entries; setting bits is order-free).  Fill pass: the sums, in the
// reference's order (row entries one after another, lanes over a column's
// entries), and the sorted columns.
template <bool FILL>
__global__ void k_adat_heavy(const int* __restrict__ heavy, int nh, const int* __restrict__ rp,
                             const int* __restrict__ ci, const double* __restrict__ av, const int* __restrict__ cp,
                             const int* __restrict__ ri, const double* __restrict__ avT, const double* __restrict__ wv,
                             double* acc_all, int* stamp_all, unsigned* bits_all, size_t R, int* __restrict__ hcnt,
                             const int* __restrict__ out_rp, int* __restrict__ out_ci, double* __restrict__ out_v) {
    const int lane = threadIdx.x & 31;
    const int slot = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nslots = (gridDim.x * blockDim.x) >> 5;
    const size_t words = (R + 31) / 32;
    double* acc = acc_all + (size_t)slot * R;
    int* stamp = stamp_all + (size_t)slot * R;
    unsigned* bits = bits_all + (size_t)slot * words;
    for (int h = slot; h < nh; h += nslots) {
        const int i = heavy[h];
        unsigned top = 0;  // highest offset touched + 1
        if (!FILL) {
            // the pattern does not depend on order: lanes take row entries
            for (int e = rp[i] + lane; e < rp[i + 1]; e += 32) {
                const int j = ci[e];
                const int qb = cp[j], qe = cp[j + 1];
                int lo = qb, hi = qe;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (ri[mid] < i) lo = mid + 1;
                    else hi = mid;
                }
                for (int q = lo; q < qe; ++q) {
                    const unsigned o = (unsigned)(ri[q] - i);
                    atomicOr(bits + (o >> 5), 1u << (o & 31));
                    top = max(top, o + 1);
                }
            }
        }
        // fill: row entries strictly in order; the column searches and the
        // scaled values of 32 entries are found at once, one per lane, and
        // broadcast entry by entry
        for (int e0 = rp[i]; FILL && e0 < rp[i + 1]; e0 += 32) {
            const int e = e0 + lane;
            int lo = 0, qe = 0;
            double vd = 0.0;
            if (e < rp[i + 1]) {
                const int j = ci[e];
                int hi = cp[j + 1];
                lo = cp[j];
                qe = hi;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (ri[mid] < i) lo = mid + 1;
                    else hi = mid;
                }
                vd = __dmul_rn(av[e], wv[j]);
            }
            const int cnt = min(32, rp[i + 1] - e0);
            for (int t = 0; t < cnt; ++t) {
                const int lo_t = __shfl_sync(0xffffffffu, lo, t);
                const int qe_t = __shfl_sync(0xffffffffu, qe, t);
                const double vd_t = __shfl_sync(0xffffffffu, vd, t);
                for (int q = lo_t + lane; q < qe_t; q += 32) {
                    const unsigned o = (unsigned)(ri[q] - i);
                    atomicOr(bits + (o >> 5), 1u << (o & 31));
                    top = max(top, o + 1);
                    double a = 0.0;  // the reference's accumulator starts at zero (Helper.cpp:355-356)
                    if (__ldcg(stamp + o) == i) a = __ldcg(acc + o);
                    __stcg(acc + o, __dadd_rn(a, __dmul_rn(vd_t, avT[q])));
                    __stcg(stamp + o, i);
                }
                __syncwarp();
            }
        }
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) top = max(top, __shfl_xor_sync(0xffffffffu, top, s));
        __syncwarp();
        const int nwords = (int)((top + 31) / 32);
        int pos = FILL ? out_rp[i] : 0;
        for (int w0 = 0; w0 < nwords; w0 += 32) {
            const int wi = w0 + lane;
            unsigned word = 0;
            if (wi < nwords) {
                word = __ldcg(bits + wi);
                __stcg(bits + wi, 0u);
            }
            const int c = __popc(word);
            int incl = c;
#pragma unroll
            for (int s = 1; s < 32; s <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, s);
                if (lane >= s) incl += t;
            }
            if (FILL) {
                int o = pos + incl - c;
                while (word) {
                    const int b = __ffs(word) - 1;
                    word &= word - 1;
                    const int off = wi * 32 + b;
                    out_ci[o] = i + off;
                    out_v[o] = __ldcg(acc + off);
                    ++o;
                }
            }
            pos += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (!FILL && lane == 0) hcnt[h] = pos;
        __syncwarp();
    }
}

}  // namespace

cudaError_t adat_heavy_range(const int* heavy, int nh, const int* rp, const int* ci, const int* cp, const int* ri,
                             int* range, cudaStream_t st) {
    const int blocks = (nh + 3) / 4 < 1024 ? (nh + 3) / 4 : 1024;
    k_adat_heavy_range<<<blocks > 0 ? blocks : 1, 128, 0, st>>>(heavy, nh, rp, ci, cp, ri, range);
    return cudaGetLastError();
}

cudaError_t adat_heavy(const int* heavy, int nh, const int* rp, const int* ci, const double* av, const int* cp,
                       const int* ri, const double* avT, const double* wv, double* acc, int* stamp, unsigned* bits,
                       size_t R, int slots, int* hcnt, const int* out_rp, int* out_ci, double* out_v, cudaStream_t st) {
    // slots is a multiple of 4: 4 warps per block, every warp owns one slot
    const int blocks = slots / 4;
    if (out_ci)
        k_adat_heavy<true><<<blocks, 128, 0, st>>>(heavy, nh, rp, ci, av, cp, ri, avT, wv, acc, stamp, bits, R, hcnt,
                                                   out_rp, out_ci, out_v);
    else
        k_adat_heavy<false><<<blocks, 128, 0, st>>>(heavy, nh, rp, ci, av, cp, ri, avT, wv, acc, stamp, bits, R, hcnt,
                                                    out_rp, out_ci, out_v);
    return cudaGetLastError();
}

cudaError_t adat_count(const int* rp, const int* ci, const int* cp, const int* ri, int m, int* cnt, cudaStream_t st) {
    const size_t smem = (size_t)kAdatCap * 8 * kAdatWarps;
    cudaError_t e = raise_smem_limit((const void*)k_adat<false>, (int)smem);
    if (e != cudaSuccess) return e;
    const int blocks = (m + kAdatWarps - 1) / kAdatWarps < 4096 ? (m + kAdatWarps - 1) / kAdatWarps : 4096;
    k_adat<false><<<blocks > 0 ? blocks : 1, 32 * kAdatWarps, smem, st>>>(rp, ci, nullptr, cp, ri, nullptr, nullptr, m,
                                                                         cnt, nullptr, nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t adat_fill(const int* rp, const int* ci, const double* av, const int* cp, const int* ri, const double* avT,
                      const double* wv, int m, const int* out_rp, int* out_ci, double* out_v, cudaStream_t st) {
    const size_t smem = (size_t)kAdatCap * 16 * kAdatWarps;
    cudaError_t e = raise_smem_limit((const void*)k_adat<true>, (int)smem);
    if (e != cudaSuccess) return e;
    const int blocks = (m + kAdatWarps - 1) / kAdatWarps < 4096 ? (m + kAdatWarps - 1) / kAdatWarps : 4096;
    k_adat<true><<<blocks > 0 ? blocks : 1, 32 * kAdatWarps, smem, st>>>(rp, ci, av, cp, ri, avT, wv, m, nullptr,
                                                                        out_rp, out_ci, out_v);
    return cudaGetLastError();
}

}  // namespace help
