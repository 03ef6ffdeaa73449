// Once-per-interior-point-iteration work: RenewPartialCholesky (PCG.cpp:38-177)
// re-designed for the GPU.
//
//   1. B = A D^-1/2 in both layouts and diag(G) = rowsum(B .* B) + delta
//      (PCG.cpp:41-46 computes the same diagonal).
//   2. Pivots: the k largest diagonals by a radix select over the IEEE bit
//      patterns (8 passes of 8-bit digits), ties to the lower row index, pivots
//      returned in increasing row order.  The reference instead picks greedily
//      from the Schur-updated diagonal (PCG.cpp:54-59); the preconditioner for
//      a given pivot set is the same operator either way.
//   3. Per column j of A, the list of pivot entries (c, B[P_c, j]).
//   4. G[i, P] for every row i, accumulated in column order into a warp-private
//      dense k-vector in shared memory (sums in the same order for G[i,c] and
//      G[c,i], so G11 comes out exactly symmetric): non-pivot rows give the
//      sparse block C = G[N, P] (CSR), pivot rows give the dense G11.
//   5. C^T by a deterministic counting transpose.
//   6. The Schur diagonal D_S = diag(G_NN) - diag(C G11^-1 C^T) (PCG.cpp:100-102
//      keeps the same quantity by rank-1 downdates).
#include "common.cuh"
#include "context.h"
#include "kernels.h"

namespace help {

namespace {

inline int grid_for(int64_t n, int threads, int cap_blocks = 65535 * 8) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > cap_blocks) b = cap_blocks;
    return (int)b;
}

__global__ void k_inv_sqrt(const double* __restrict__ d, double* __restrict__ s, int n, int* status) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double dj = d[j];
        if (!(dj > 0.0) || !(dj < 1.0e300)) {
            atomicCAS(status, 0, kStatusNumeric);
            s[j] = 0.0;
        } else {
            s[j] = 1.0 / sqrt(dj);
        }
    }
}

// bv[e] = av[e] * s[ci[e]] (element-parallel, coalesced)
__global__ void k_scale_elems(const int* __restrict__ ci, const double* __restrict__ av, const double* __restrict__ s,
                              double* __restrict__ bv, float* __restrict__ bv32, int64_t nnz) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
        const double b = av[e] * s[ci[e]];
        bv[e] = b;
        if (bv32) bv32[e] = (float)b;
    }
}

// CSC values: bvT[e] = avT[e] * s[j] for the entries of column j (thread per column)
__global__ void k_scale_cols(const int* __restrict__ cp, const double* __restrict__ avT, const double* __restrict__ s,
                             double* __restrict__ bvT, float* __restrict__ bvT32, int n) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double sj = s[j];
        for (int e = cp[j]; e < cp[j + 1]; ++e) {
            const double b = avT[e] * sj;
            bvT[e] = b;
            if (bvT32) bvT32[e] = (float)b;
        }
    }
}

// diag[i] = sum_e bv[e]^2 + delta (thread per row, FMA in column order)
// diag(G) = rowsum(B .* B) + delta; status <- numeric error where a diagonal
// is not positive (a row of A without nonzeros and delta = 0: G is singular)
__global__ void k_row_sumsq(const int* __restrict__ rp, const double* __restrict__ bv, double* __restrict__ diag,
                            double delta, int m, int* __restrict__ status) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int e = rp[i]; e < rp[i + 1]; ++e) acc = fma(bv[e], bv[e], acc);
        const double g = acc + delta;
        diag[i] = g;
        if (!(g > 0.0)) atomicExch(status, kStatusNumeric);
    }
}

// ---------------------------------------------------------------- scan

constexpr int kScanThreads = 1024;

__global__ void k_scan_block(const int* __restrict__ in, int* __restrict__ out, int64_t n, int* __restrict__ sums) {
    __shared__ int warp_tot[32];
    const int64_t i = (int64_t)blockIdx.x * kScanThreads + threadIdx.x;
    const int v = (i < n) ? in[i] : 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;  // inclusive
    }
    __syncthreads();
    const int base = (warp > 0) ? warp_tot[warp - 1] : 0;
    if (i < n) out[i] = base + x - v;
    if (threadIdx.x == kScanThreads - 1 && sums) sums[blockIdx.x] = base + x;
}

__global__ void k_scan_add(int* __restrict__ out, int64_t n, const int* __restrict__ offs) {
    const int64_t i = (int64_t)blockIdx.x * kScanThreads + threadIdx.x;
    if (i < n) out[i] += offs[blockIdx.x];
}

__global__ void k_scan_total(const int* __restrict__ in, const int* __restrict__ out, int64_t n, int* total) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *total = (n > 0) ? out[n - 1] + in[n - 1] : 0;
}

cudaError_t scan_rec(const int* in, int* out, int64_t n, int* tmp, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int64_t nb = (n + kScanThreads - 1) / kScanThreads;
    if (nb == 1) {
        k_scan_block<<<1, kScanThreads, 0, st>>>(in, out, n, nullptr);
        return cudaGetLastError();
    }
    int* sums = tmp;
    int* sums_scanned = tmp + nb;
    k_scan_block<<<(unsigned)nb, kScanThreads, 0, st>>>(in, out, n, sums);
    cudaError_t e = scan_rec(sums, sums_scanned, nb, tmp + 2 * nb, st);
    if (e != cudaSuccess) return e;
    k_scan_add<<<(unsigned)nb, kScanThreads, 0, st>>>(out, n, sums_scanned);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- top-k

__global__ void k_topk_init(TopkStateDev* st, int k, unsigned int* hist) {
    if (threadIdx.x == 0) {
        st->prefix = 0ull;
        st->mask = 0ull;
        st->remaining = k;
        st->n_greater = 0;
    }
    hist[threadIdx.x] = 0u;
}

__global__ void k_topk_keys(const double* __restrict__ diag, unsigned long long* __restrict__ keys, int m,
                            int* status) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = diag[i];
        if (!(v >= 0.0) || !(v < 1.0e308)) {
            atomicCAS(status, 0, kStatusNumeric);
            keys[i] = 0ull;
        } else {
            keys[i] = (unsigned long long)__double_as_longlong(v);  // monotone for v >= 0
        }
    }
}

__global__ void k_topk_hist(const unsigned long long* __restrict__ keys, int m, int shift,
                            const TopkStateDev* __restrict__ st, unsigned int* __restrict__ hist) {
    __shared__ unsigned int h[kTopkBins];
    for (int b = threadIdx.x; b < kTopkBins; b += blockDim.x) h[b] = 0u;
    __syncthreads();
    const unsigned long long mask = st->mask, prefix = st->prefix;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long key = keys[i];
        if ((key & mask) == prefix) atomicAdd(&h[(key >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kTopkBins; b += blockDim.x)
        if (h[b]) atomicAdd(&hist[b], h[b]);
}

__global__ void k_topk_pick(unsigned int* hist, int shift, TopkStateDev* st) {
    __shared__ int s_digit, s_cum;
    if (threadIdx.x == 0) {
        const int rem = st->remaining;
        long long cum = 0;
        int d = 255;
        for (; d > 0; --d) {
            if (cum + (long long)hist[d] >= rem) break;
            cum += hist[d];
        }
        s_digit = d;
        s_cum = (int)cum;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        st->remaining -= s_cum;
        st->n_greater += s_cum;
        st->prefix |= (unsigned long long)s_digit << shift;
        st->mask |= 255ull << shift;
    }
    hist[threadIdx.x] = 0u;
}

__global__ void k_topk_eq(const unsigned long long* __restrict__ keys, int m, const TopkStateDev* __restrict__ st,
                          int* __restrict__ eq) {
    const unsigned long long thr = st->prefix;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        eq[i] = (keys[i] == thr) ? 1 : 0;
}

__global__ void k_topk_sel(const unsigned long long* __restrict__ keys, const int* __restrict__ eqrank, int m,
                           const TopkStateDev* __restrict__ st, int* __restrict__ sel) {
    const unsigned long long thr = st->prefix;
    const int rem = st->remaining;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long key = keys[i];
        sel[i] = (key > thr || (key == thr && eqrank[i] < rem)) ? 1 : 0;
    }
}

__global__ void k_topk_scatter(const unsigned long long* __restrict__ keys, const int* __restrict__ eqrank,
                               const int* __restrict__ pos, int m, const TopkStateDev* __restrict__ st,
                               int* __restrict__ piv, int* __restrict__ pivpos) {
    const unsigned long long thr = st->prefix;
    const int rem = st->remaining;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long key = keys[i];
        const bool s = key > thr || (key == thr && eqrank[i] < rem);
        if (s) {
            piv[pos[i]] = (int)i;
            pivpos[i] = pos[i];
        } else {
            pivpos[i] = -1;
        }
    }
}

__global__ void k_iota_pivots(int* piv, int* pivpos, int m, int all) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        if (all) {
            piv[i] = (int)i;
            pivpos[i] = (int)i;
        } else {
            pivpos[i] = -1;
        }
    }
}

// ---------------------------------------------------------------- pivot lists per column

__global__ void k_bp_count(const int* __restrict__ cp, const int* __restrict__ ri, const int* __restrict__ pivpos,
                           int n, int* __restrict__ cnt) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        int c = 0;
        for (int e = cp[j]; e < cp[j + 1]; ++e) c += (pivpos[ri[e]] >= 0);
        cnt[j] = c;
    }
}

__global__ void k_bp_fill(const int* __restrict__ cp, const int* __restrict__ ri, const double* __restrict__ bvT,
                          const int* __restrict__ pivpos, int n, const int* __restrict__ bp_ptr, int* __restrict__ bp_c,
                          double* __restrict__ bp_v) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        int o = bp_ptr[j];
        for (int e = cp[j]; e < cp[j + 1]; ++e) {
            const int c = pivpos[ri[e]];
            if (c >= 0) {
                bp_c[o] = c;
                bp_v[o] = bvT[e];
                ++o;
            }
        }
    }
}

// ---------------------------------------------------------------- G[i, P]

__host__ __device__ inline size_t gcols_warp_bytes(int k) {
    return (((size_t)k * 9 + 15) / 16) * 16;  // k doubles + k flag bytes
}

template <int PASS>
__global__ void k_gcols_rows(const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ bv,
                             const int* __restrict__ bp_ptr, const int* __restrict__ bp_c,
                             const double* __restrict__ bp_v, const int* __restrict__ pivpos, int m, int k,
                             double delta, int* __restrict__ cnt, const int* __restrict__ c_rp, int* __restrict__ c_ci,
                             double* __restrict__ c_v, double* __restrict__ g11) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double* acc = reinterpret_cast<double*>(smem + gcols_warp_bytes(k) * warp);
    unsigned char* flag = reinterpret_cast<unsigned char*>(acc + k);
    for (int c = lane; c < k; c += 32) {
        acc[c] = 0.0;
        flag[c] = 0;
    }
    __syncwarp();
    const int64_t gw = (int64_t)blockIdx.x * nw + warp, tw = (int64_t)gridDim.x * nw;
    for (int64_t i = gw; i < m; i += tw) {
        const int b = rp[i], e = rp[i + 1];
        for (int base = b; base < e; base += 32) {
            const int ei = base + lane;
            int qb = 0, qe = 0;
            double bij = 0.0;
            if (ei < e) {
                const int j = ci[ei];
                bij = bv[ei];
                qb = bp_ptr[j];
                qe = bp_ptr[j + 1];
            }
            unsigned has = __ballot_sync(0xffffffffu, qe > qb);
            while (has) {
                const int src = __ffs(has) - 1;
                has &= has - 1;
                const int sqb = __shfl_sync(0xffffffffu, qb, src), sqe = __shfl_sync(0xffffffffu, qe, src);
                const double sb = __shfl_sync(0xffffffffu, bij, src);
                for (int q = sqb + lane; q < sqe; q += 32) {
                    const int c = bp_c[q];
                    acc[c] = fma(sb, bp_v[q], acc[c]);
                    flag[c] = 1;
                }
                __syncwarp();
            }
        }
        __syncwarp();
        const int pr = pivpos[i];
        int pos = (PASS == 1 && pr < 0) ? c_rp[i] : 0;
        for (int cb = 0; cb < k; cb += 32) {
            const int c = cb + lane;
            const bool t = (c < k) && flag[c];
            const unsigned ball = __ballot_sync(0xffffffffu, t);
            if (t) {
                if (PASS == 1) {
                    const double v = acc[c];
                    if (pr >= 0) {
                        g11[(size_t)pr * k + c] = (c == pr) ? v + delta : v;
                    } else {
                        const int o = pos + __popc(ball & ((1u << lane) - 1u));
                        c_ci[o] = c;
                        c_v[o] = v;
                    }
                }
                acc[c] = 0.0;
                flag[c] = 0;
            }
            pos += __popc(ball);
        }
        if (PASS == 0 && lane == 0) cnt[i] = (pr >= 0) ? 0 : pos;
        __syncwarp();
    }
}

// ---------------------------------------------------------------- C^T

constexpr int kCtRows = 1024;  // rows per counting block

__global__ void k_ct_count(const int* __restrict__ c_rp, const int* __restrict__ c_ci, int m, int k, int nblk,
                           int* __restrict__ blk_cnt) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int* cnt = reinterpret_cast<int*>(smem) + (size_t)warp * k;
    for (int64_t b = (int64_t)blockIdx.x * nw + warp; b < nblk; b += (int64_t)gridDim.x * nw) {
        for (int c = lane; c < k; c += 32) cnt[c] = 0;
        __syncwarp();
        const int i0 = (int)(b * kCtRows), i1 = min(m, i0 + kCtRows);
        for (int i = i0; i < i1; ++i) {
            for (int q = c_rp[i] + lane; q < c_rp[i + 1]; q += 32) cnt[c_ci[q]] += 1;
            __syncwarp();
        }
        for (int c = lane; c < k; c += 32) blk_cnt[(size_t)c * nblk + b] = cnt[c];
        __syncwarp();
    }
}

__global__ void k_ct_fill(const int* __restrict__ c_rp, const int* __restrict__ c_ci, const double* __restrict__ c_v,
                          int m, int k, int nblk, const int* __restrict__ blk_off, int* __restrict__ ct_ci,
                          double* __restrict__ ct_v) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int* cnt = reinterpret_cast<int*>(smem) + (size_t)warp * k;
    for (int64_t b = (int64_t)blockIdx.x * nw + warp; b < nblk; b += (int64_t)gridDim.x * nw) {
        for (int c = lane; c < k; c += 32) cnt[c] = blk_off[(size_t)c * nblk + b];
        __syncwarp();
        const int i0 = (int)(b * kCtRows), i1 = min(m, i0 + kCtRows);
        for (int i = i0; i < i1; ++i) {
            for (int q = c_rp[i] + lane; q < c_rp[i + 1]; q += 32) {
                const int c = c_ci[q];
                const int o = cnt[c];
                cnt[c] = o + 1;
                ct_ci[o] = i;
                ct_v[o] = c_v[q];
            }
            __syncwarp();
        }
    }
}

__global__ void k_ct_rp(const int* __restrict__ blk_off, int k, int nblk, const int* __restrict__ total,
                        int* __restrict__ ct_rp) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c <= k; c += gridDim.x * blockDim.x)
        ct_rp[c] = (c < k) ? blk_off[(size_t)c * nblk] : *total;
}

__global__ void k_vals_f32(const double* __restrict__ a, float* __restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)a[i];
}

// ---------------------------------------------------------------- Schur diagonal

__global__ void k_schur_diag(const int* __restrict__ c_rp, const int* __restrict__ c_ci, const double* __restrict__ c_v,
                             const double* __restrict__ W, const double* __restrict__ diag,
                             const int* __restrict__ pivpos, int m, int k, double floor_rel,
                             double* __restrict__ dsinv, float* __restrict__ dsinv32) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t i = (int64_t)blockIdx.x * nw + warp; i < m; i += (int64_t)gridDim.x * nw) {
        if (pivpos[i] >= 0) {
            if (lane == 0) {
                dsinv[i] = 0.0;
                if (dsinv32) dsinv32[i] = 0.0f;
            }
            continue;
        }
        const int b = c_rp[i], e = c_rp[i + 1];
        // c^T W c with W symmetric: sum over entries a of
        // c_a (W_aa c_a + 2 sum_{b > a} W_ab c_b), half the W reads; a lane
        // takes entry p and its mirror len-1-p, so every lane walks len - 1
        // entries of the triangle
        const int len = e - b, half = (len + 1) >> 1;
        double qf = 0.0;
        auto term = [&](int ea) {
            const int a = c_ci[ea];
            const double ca = c_v[ea];
            const double* Wr = W + (size_t)a * k;
            double acc = 0.0;
            for (int eb = ea + 1; eb < e; ++eb) acc = fma(__ldg(Wr + c_ci[eb]), c_v[eb], acc);
            return ca * fma(__ldg(Wr + a), ca, 2.0 * acc);
        };
        for (int p = lane; p < half; p += 32) {
            qf += term(b + p);
            const int q = len - 1 - p;
            if (q > p) qf += term(b + q);
        }
        qf = warp_sum(qf);
        if (lane == 0) {
            const double g = diag[i];
            double ds = g - qf;
            double fl = floor_rel * g;
            if (!(fl > 0.0)) fl = 1.0e-300;
            if (!(ds > fl)) ds = fl;
            dsinv[i] = 1.0 / ds;
            if (dsinv32) dsinv32[i] = (float)(1.0 / ds);
        }
    }
}

}  // namespace

// ================================================================ launchers

cudaError_t renew_inv_sqrt(const double* d, double* s, int n, int* status, cudaStream_t st) {
    k_inv_sqrt<<<grid_for(n, 256), 256, 0, st>>>(d, s, n, status);
    return cudaGetLastError();
}

cudaError_t renew_scale_values(const double* s, const int* rp, const int* ci, const double* av, double* bv,
                               float* bv32, const int* cp, const double* avT, double* bvT, float* bvT32,
                               double* diag, double delta, int m, int n, int64_t nnz, int* status, cudaStream_t st) {
    k_scale_elems<<<grid_for(nnz, 256), 256, 0, st>>>(ci, av, s, bv, bv32, nnz);
    k_scale_cols<<<grid_for(n, 128), 128, 0, st>>>(cp, avT, s, bvT, bvT32, n);
    k_row_sumsq<<<grid_for(m, 128), 128, 0, st>>>(rp, bv, diag, delta, m, status);
    return cudaGetLastError();
}

size_t scan_tmp_elems(int64_t n) {
    size_t t = 64;
    int64_t nb = (n + kScanThreads - 1) / kScanThreads;
    while (nb > 1) {
        t += 2 * (size_t)nb;
        nb = (nb + kScanThreads - 1) / kScanThreads;
    }
    return t + 64;
}

cudaError_t exclusive_scan(const int* in, int* out, int64_t n, int* tmp, int* total_dev, cudaStream_t st) {
    if (n > 0) {
        cudaError_t e = scan_rec(in, out, n, tmp, st);
        if (e != cudaSuccess) return e;
    }
    if (total_dev) {
        if (n > 0) {
            k_scan_total<<<1, 32, 0, st>>>(in, out, n, total_dev);
        } else {
            return cudaMemsetAsync(total_dev, 0, sizeof(int), st);
        }
    }
    return cudaGetLastError();
}

cudaError_t topk_select(const double* diag, int m, int k, unsigned long long* keys, unsigned int* hist, int* flags,
                        int* scan_tmp, TopkStateDev* tst, int* status, int* piv, int* pivpos, cudaStream_t st) {
    if (k <= 0 || k >= m) {
        k_iota_pivots<<<grid_for(m, 256), 256, 0, st>>>(piv, pivpos, m, k >= m ? 1 : 0);
        return cudaGetLastError();
    }
    k_topk_init<<<1, kTopkBins, 0, st>>>(tst, k, hist);
    k_topk_keys<<<grid_for(m, 256), 256, 0, st>>>(diag, keys, m, status);
    const int hb = grid_for(m, 256, 1024);
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = 56 - 8 * pass;
        k_topk_hist<<<hb, 256, 0, st>>>(keys, m, shift, tst, hist);
        k_topk_pick<<<1, kTopkBins, 0, st>>>(hist, shift, tst);
    }
    int* eq = flags;
    int* eqrank = flags + m;
    int* sel = flags + 2 * (size_t)m;
    k_topk_eq<<<grid_for(m, 256), 256, 0, st>>>(keys, m, tst, eq);
    cudaError_t e = exclusive_scan(eq, eqrank, m, scan_tmp, nullptr, st);
    if (e != cudaSuccess) return e;
    k_topk_sel<<<grid_for(m, 256), 256, 0, st>>>(keys, eqrank, m, tst, sel);
    int* pos = eq;  // eq no longer needed
    e = exclusive_scan(sel, pos, m, scan_tmp, nullptr, st);
    if (e != cudaSuccess) return e;
    k_topk_scatter<<<grid_for(m, 256), 256, 0, st>>>(keys, eqrank, pos, m, tst, piv, pivpos);
    return cudaGetLastError();
}

cudaError_t pivot_lists_count(const int* cp, const int* ri, const int* pivpos, int n, int* cnt, cudaStream_t st) {
    k_bp_count<<<grid_for(n, 128), 128, 0, st>>>(cp, ri, pivpos, n, cnt);
    return cudaGetLastError();
}

cudaError_t pivot_lists_fill(const int* cp, const int* ri, const double* bvT, const int* pivpos, int n,
                             const int* bp_ptr, int* bp_c, double* bp_v, cudaStream_t st) {
    k_bp_fill<<<grid_for(n, 128), 128, 0, st>>>(cp, ri, bvT, pivpos, n, bp_ptr, bp_c, bp_v);
    return cudaGetLastError();
}

int gcols_warps(int k) {
    const size_t per = gcols_warp_bytes(k > 0 ? k : 1);
    int w = (int)((96 * 1024) / per);
    if (w > 8) w = 8;
    if (w < 1) w = 1;
    return w;
}
size_t gcols_smem_bytes(int k) { return gcols_warp_bytes(k > 0 ? k : 1) * (size_t)gcols_warps(k); }

cudaError_t gcols_rows(int pass, const int* rp, const int* ci, const double* bv, const int* bp_ptr, const int* bp_c,
                       const double* bp_v, const int* pivpos, int m, int k, double delta, int* cnt, const int* c_rp,
                       int* c_ci, double* c_v, double* g11, int num_sms, cudaStream_t st) {
    const int warps = gcols_warps(k);
    const size_t smem = gcols_smem_bytes(k);
    const int threads = warps * 32;
    int blocks = num_sms * 2;
    if (blocks < 1) blocks = 1;
    cudaError_t e;
    if (pass == 0) {
        e = raise_smem_limit((const void*)k_gcols_rows<0>, (int)smem);
        if (e != cudaSuccess) return e;
        k_gcols_rows<0><<<blocks, threads, smem, st>>>(rp, ci, bv, bp_ptr, bp_c, bp_v, pivpos, m, k, delta, cnt, c_rp,
                                                       c_ci, c_v, g11);
    } else {
        e = raise_smem_limit((const void*)k_gcols_rows<1>, (int)smem);
        if (e != cudaSuccess) return e;
        k_gcols_rows<1><<<blocks, threads, smem, st>>>(rp, ci, bv, bp_ptr, bp_c, bp_v, pivpos, m, k, delta, cnt, c_rp,
                                                       c_ci, c_v, g11);
    }
    return cudaGetLastError();
}

int ct_rows_per_block() { return kCtRows; }

static int ct_warps(int k) {
    int w = (int)((64 * 1024) / ((size_t)(k > 0 ? k : 1) * 4));
    if (w > 8) w = 8;
    if (w < 1) w = 1;
    return w;
}

cudaError_t ct_count(const int* c_rp, const int* c_ci, int m, int k, int* blk_cnt, cudaStream_t st) {
    const int nblk = (m + kCtRows - 1) / kCtRows;
    const int warps = ct_warps(k);
    const size_t smem = (size_t)warps * k * sizeof(int);
    cudaError_t e = raise_smem_limit((const void*)k_ct_count, (int)smem);
    if (e != cudaSuccess) return e;
    const int blocks = (nblk + warps - 1) / warps;
    k_ct_count<<<blocks, warps * 32, smem, st>>>(c_rp, c_ci, m, k, nblk, blk_cnt);
    return cudaGetLastError();
}

cudaError_t ct_fill(const int* c_rp, const int* c_ci, const double* c_v, int m, int k, const int* blk_off, int* ct_ci,
                    double* ct_v, cudaStream_t st) {
    const int nblk = (m + kCtRows - 1) / kCtRows;
    const int warps = ct_warps(k);
    const size_t smem = (size_t)warps * k * sizeof(int);
    cudaError_t e = raise_smem_limit((const void*)k_ct_fill, (int)smem);
    if (e != cudaSuccess) return e;
    const int blocks = (nblk + warps - 1) / warps;
    k_ct_fill<<<blocks, warps * 32, smem, st>>>(c_rp, c_ci, c_v, m, k, nblk, blk_off, ct_ci, ct_v);
    return cudaGetLastError();
}

cudaError_t ct_row_ptr(const int* blk_off, int k, int nblk, const int* total_dev, int* ct_rp, cudaStream_t st) {
    k_ct_rp<<<grid_for(k + 1, 256), 256, 0, st>>>(blk_off, k, nblk, total_dev, ct_rp);
    return cudaGetLastError();
}

cudaError_t vals_to_f32(const double* a, float* out, int64_t n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_vals_f32<<<grid_for(n, 256), 256, 0, st>>>(a, out, n);
    return cudaGetLastError();
}

cudaError_t schur_diag(const int* c_rp, const int* c_ci, const double* c_v, const double* W, const double* diag,
                       const int* pivpos, int m, int k, double floor_rel, double* dsinv, float* dsinv32,
                       cudaStream_t st) {
    const int threads = 256;
    k_schur_diag<<<grid_for((int64_t)m * 32, threads), threads, 0, st>>>(c_rp, c_ci, c_v, W, diag, pivpos, m, k,
                                                                         floor_rel, dsinv, dsinv32);
    return cudaGetLastError();
}

}  // namespace help
