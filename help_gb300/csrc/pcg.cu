// Persistent preconditioned conjugate gradient on G x = b, G = B B^T + delta I,
// B = A D^-1/2 -- the loop of ConjugateGradient (PCG.cpp:296-395) with the
// partial-Cholesky preconditioner of PCG.cpp:183-196 applied in block form.
//
// One cooperative launch runs the whole solve: every block stays resident,
// phases are separated by a bounded grid barrier, and every scalar (alpha,
// beta, the stopping test) is formed by every block from the same per-block
// partial sums in the same order, so all blocks take identical decisions and
// the run is bitwise reproducible.
//
// Preconditioner M = [L11 0; L21 I] diag(D1, D_S) [L11 0; L21 I]^T restricted
// to the pivot rows P (k of them) is applied without the dense L21 the
// reference materialises (PCG.cpp:143-155).  With C = G[N, P] (N = non-pivot
// rows) and W = G11^-1:
//     a   = W r_P
//     z_N = D_S^-1 (r_N - C a)
//     w   = r_P - C^T z_N
//     z_P = W w
// and r_P . z_P = a . w (W symmetric), so beta is known in the same phase that
// forms the new search direction.  Per iteration:
//   P2: z_N, r_N.z_N          | P3: w          | P4: beta, z_P, p_new
//   A : t = B^T p_new         | B : q = B t + delta p_new, p.q
//   C : alpha, x += alpha p, r -= alpha q, r.r, a = W r_P
// Vectors are V (double, or float for the inner solves of mixed precision);
// dot products, alpha/beta and the pivot-block work stay in double.
#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.h"
#include "spmv.cuh"

namespace help {

template <class V>
__global__ void __launch_bounds__(512) pcg_persistent(const __grid_constant__ PcgArgs<V> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V* s_val = reinterpret_cast<V*>(smem_raw);
    V* s_x = s_val + A.cap;
    double* s_vec = reinterpret_cast<double*>(smem_raw);
    __shared__ double red[32];

    const int G = gridDim.x, bid = blockIdx.x, tid = threadIdx.x, T = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nw = T >> 5;
    const long long gtid = (long long)bid * T + tid, gthr = (long long)G * T;
    double* part_rr = A.part;
    double* part_rz = A.part + G;
    double* part_pq = A.part + 2 * G;

    auto sum_parts = [&](const double* p) {
        double s = 0.0;
        for (int b = tid; b < G; b += T) s += p[b];
        return block_sum(s, red);
    };
    // out(c, (W y)_c) for the rows c of W owned by this block's warps.
    auto gemv = [&](auto yf, auto out) {
        const bool active = (long long)bid * nw < A.k;
        if (active)
            for (int c = tid; c < A.k; c += T) s_vec[c] = yf(c);
        __syncthreads();
        if (active) {
            for (int c = bid * nw + warp; c < A.k; c += G * nw) {
                const double* Wr = A.W + (size_t)c * A.k;
                double acc = 0.0;
                for (int c2 = lane; c2 < A.k; c2 += 32) acc = fma(ld_ro(Wr + c2), s_vec[c2], acc);
                acc = warp_sum(acc);
                if (lane == 0) out(c, acc);
            }
        }
        __syncthreads();
    };

    // ---- I0: r.r of the initial residual, a = W r_P
    {
        const V* r = A.r0;
        double rr = 0.0;
        for (long long i = gtid; i < A.m; i += gthr) {
            const double v = (double)r[i];
            rr = fma(v, v, rr);
        }
        rr = block_sum(rr, red);
        if (tid == 0) part_rr[bid] = rr;
        gemv([&](int c) { return (double)r[A.piv[c]]; }, [&](int c, double s) { A.a[c] = s; });
        if (!grid_sync(A.bar)) return;
    }
    const double rr0 = sum_parts(part_rr);
    const double term2 = rr0 * A.tol2;
    double rr = rr0, rz_old = 0.0;
    long long it = 0;
    int cur = 0, converged = 0, status = 0;

    for (;;) {
        if (it > 0) rr = sum_parts(part_rr);
        if (!(rr == rr)) {
            status = kStatusNumeric;
            break;
        }
        if (rr < term2 || rr == 0.0) {
            converged = 1;
            break;
        }
        if (it >= A.max_iter) break;
        V* r = cur ? A.r1 : A.r0;
        V* rn = cur ? A.r0 : A.r1;
        V* p = cur ? A.p1 : A.p0;
        V* pn = cur ? A.p0 : A.p1;

        // ---- P2: z_N = D_S^-1 (r_N - C a), partial r_N . z_N
        {
            double rz = 0.0;
            spmv_items<V>(
                A.c_items, A.n_c, bid, G, A.c_rp, A.c_ci, A.c_v, A.cap, [&](int c) { return (V)A.a[c]; },
                [&](int i, V s) {
                    if (A.pivpos[i] < 0) {
                        const V ri = r[i];
                        const V zi = A.dsinv[i] * (ri - s);
                        A.z[i] = zi;
                        rz = fma((double)ri, (double)zi, rz);
                    }
                },
                s_val, s_x, red);
            rz = block_sum(rz, red);
            if (tid == 0) part_rz[bid] = rz;
            if (!grid_sync(A.bar)) return;
        }
        // ---- P3: w = r_P - C^T z_N
        spmv_items<V>(
            A.ct_items, A.n_ct, bid, G, A.ct_rp, A.ct_ci, A.ct_v, A.cap, [&](int i) { return A.z[i]; },
            [&](int c, V s) { A.w[c] = (double)r[A.piv[c]] - (double)s; }, s_val, s_x, red);
        if (!grid_sync(A.bar)) return;

        // ---- P4: rz = r_N.z_N + a.w, beta, z_P = W w, p_new = z + beta p
        double rz;
        {
            double aw = 0.0;
            for (int c = tid; c < A.k; c += T) aw = fma(A.a[c], A.w[c], aw);
            aw = block_sum(aw, red);
            rz = sum_parts(part_rz) + aw;
        }
        if (!(rz > 0.0)) {  // M^-1 not positive on r, or NaN
            status = kStatusNumeric;
            break;
        }
        const double beta = (it == 0) ? 0.0 : rz / rz_old;
        const V vb = (V)beta;
        const bool first = (it == 0);
        gemv([&](int c) { return A.w[c]; },
             [&](int c, double s) {
                 const int i = A.piv[c];
                 const V zc = (V)s;
                 pn[i] = first ? zc : fma_t(vb, p[i], zc);
             });
        for (long long i = gtid; i < A.m; i += gthr) {
            if (A.pivpos[i] < 0) {
                const V zi = A.z[i];
                pn[i] = first ? zi : fma_t(vb, p[i], zi);
            }
        }
        if (!grid_sync(A.bar)) return;
        if (A.precond_only) break;

        // ---- A: t = B^T p_new
        spmv_items<V>(
            A.csc_items, A.n_csc, bid, G, A.cp, A.ri, A.bvT, A.cap, [&](int i) { return pn[i]; },
            [&](int j, V s) { A.t[j] = s; }, s_val, s_x, red);
        if (!grid_sync(A.bar)) return;

        // ---- B: q = B t + delta p_new, partial p.q
        {
            double pq = 0.0;
            const V vd = (V)A.delta;
            const bool has_delta = (A.delta != 0.0);
            spmv_items<V>(
                A.csr_items, A.n_csr, bid, G, A.rp, A.ci, A.bv, A.cap, [&](int j) { return A.t[j]; },
                [&](int i, V s) {
                    const V pi = pn[i];
                    const V qi = has_delta ? fma_t(vd, pi, s) : s;
                    A.q[i] = qi;
                    pq = fma((double)pi, (double)qi, pq);
                },
                s_val, s_x, red);
            pq = block_sum(pq, red);
            if (tid == 0) part_pq[bid] = pq;
            if (!grid_sync(A.bar)) return;
        }

        // ---- C: alpha, x += alpha p, r -= alpha q, r.r, a = W r_P
        {
            const double pq = sum_parts(part_pq);
            if (!(pq > 0.0)) {  // G not positive on p (breakdown) or NaN
                status = kStatusNumeric;
                break;
            }
            const double alpha = rz / pq;
            const V va = (V)alpha;
            double rrl = 0.0;
            for (long long i = gtid; i < A.m; i += gthr) {
                const V pi = pn[i], qi = A.q[i];
                A.x[i] = fma_t(va, pi, A.x[i]);
                const V ri = fma_t(-va, qi, r[i]);
                rn[i] = ri;
                rrl = fma((double)ri, (double)ri, rrl);
            }
            rrl = block_sum(rrl, red);
            if (tid == 0) part_rr[bid] = rrl;
            gemv([&](int c) {
                     const int i = A.piv[c];
                     return (double)fma_t(-va, A.q[i], r[i]);
                 },
                 [&](int c, double s) { A.a[c] = s; });
            if (!grid_sync(A.bar)) return;
        }
        rz_old = rz;
        cur ^= 1;
        ++it;
    }
    if (bid == 0 && tid == 0) {
        A.out->iterations = it;
        A.out->rr0 = rr0;
        A.out->rr = rr;
        A.out->converged = converged;
        A.out->status = status;
        A.out->final_buf = cur;
    }
}

template <class V>
cudaError_t pcg_configure(int threads, size_t smem, int* blocks_per_sm) {
    cudaError_t e = cudaFuncSetAttribute(pcg_persistent<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pcg_persistent<V>, threads, smem);
}

template <class V>
cudaError_t pcg_launch(const PcgArgs<V>& args, int blocks, int threads, size_t smem, cudaStream_t stream) {
    void* params[] = {(void*)&args};
    return cudaLaunchCooperativeKernel((const void*)pcg_persistent<V>, dim3(blocks), dim3(threads), params, smem,
                                       stream);
}

template cudaError_t pcg_configure<double>(int, size_t, int*);
template cudaError_t pcg_configure<float>(int, size_t, int*);
template cudaError_t pcg_launch<double>(const PcgArgs<double>&, int, int, size_t, cudaStream_t);
template cudaError_t pcg_launch<float>(const PcgArgs<float>&, int, int, size_t, cudaStream_t);

}  // namespace help
