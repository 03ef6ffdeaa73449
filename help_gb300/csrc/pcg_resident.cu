// Single-cluster CG with the vectors and the matrix resident in shared
// memory -- the loop of ConjugateGradient (PCG.cpp:296-395) and the
// block-form preconditioner of PCG.cpp:183-196 for systems that fit on one
// cluster's SMs.
//
// A cluster of 16 (or 8) CTAs, one per SM, owns the solve.  CTA c owns a
// contiguous slice of the rows of G (m) and of the columns of A (n).  Every
// CTA keeps in its shared memory
//   * a full copy of p (m), gathered by the B^T product, and in FP32 also a
//     full copy of t = B^T p (n);
//   * its own slices of x, r, z, q;
//   * the pivot-row values r_P, q_P, a = W r_P and w (k each), replicated;
//   * its slices of the matrix (its rows of B, C and D_S^-1, its columns of
//     B -- rows of B^T --, its entries of C^T, and W), copied from HBM once
//     per launch: the acquire side of every cluster barrier invalidates L1,
//     so a matrix read through L1 would come back from L2 after each barrier.
// Each iteration is four steps separated by hardware cluster barriers
// (barrier.cluster arrive.release / wait.acquire); a CTA hands its results to
// the others by plain stores into their shared memory (DSMEM) before the
// barrier -- except t in FP64, which goes through L2 (see step iii):
//   (i)   z_N = D_S^-1 (r_N - C a) on own rows; r_N.z_N, the previous step's
//         r.r and the k-vector C^T z_N over own rows -> every CTA
//         -- barrier --  stop test on r.r
//   (ii)  w = r_P - sum C^T z_N, rz = r_N.z_N + a.w, beta, z_P = W w on own
//         pivot rows, p = z + beta p on own rows -> every CTA's p
//         -- barrier --
//   (iii) t = B^T p on own columns -> L2 (FP64) / every CTA's t (FP32)
//         -- barrier --
//   (iv)  q = B t + delta p on own rows; p.q and q_P -> every CTA
//         -- barrier --  alpha; x += alpha p, r -= alpha q on own rows;
//         r_P -= alpha q_P and a = W r_P in every CTA
// Every CTA adds the CTAs' partials in the same order, so all of them form
// bit-identical alpha, beta and stopping decisions and leave the loop
// together.  GB300 issues FP64 at ~2 lanes per clock per SM, and an FP64
// warp instruction holds its sub-partition's pipe for ~64 cycles however few
// lanes are active, so the scalar work is written as short trees over many
// warps rather than serial chains, and rows take several nonzeros per lane.
#include <cooperative_groups.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"
#include "kernels.h"
#include "spmv.cuh"

namespace cg = cooperative_groups;

namespace help {

namespace {

constexpr int kResThreads = 256;
constexpr int kResWarps = kResThreads / 32;

// A slice of rows of a CSR matrix: rows 0..rows-1 are rows row0 + r of the
// whole matrix, column indices are the whole matrix's.  In shared memory
// (load_rows: ptr rebased to 0) or read in place from HBM (global_rows: ptr
// points at the whole matrix's row pointers from row0 on).
template <class V>
struct LocalCsr {
    const int* ptr;
    const int* idx;
    const V* val;
    int rows, row0, G;
};

// ep(row0 + r, sum) once per row by the group's first lane; G lanes per row.
template <class V, bool kGatherL2 = false, class XF, class EP>
HELP_DEVINL void rows_local(const LocalCsr<V>& M, const XF& xf, const EP& ep) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int G = M.G, lg = __ffs(G) - 1;
    const int sub = lane & (G - 1), rpw = 32 >> lg;
    for (int base = warp * rpw; base < M.rows; base += kResWarps * rpw) {
        const int row = base + (lane >> lg);
        int b = 0, e = 0;
        if (row < M.rows) {
            b = M.ptr[row];
            e = M.ptr[row + 1];
        }
        V acc = V(0);
        int q = b + sub;
        if constexpr (kGatherL2) {
            // gathers from L2: up to 8 entries per lane per round, every load
            // issued before the first FMA (one L2 round trip for rows of up
            // to 8 G nonzeros); FMAs in entry order
            for (; q < e; q += 8 * G) {
                V xv[8], vv[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int qq = q + u * G;
                    const bool in = qq < e;
                    vv[u] = in ? M.val[qq] : V(0);
                    xv[u] = in ? xf(M.idx[qq]) : V(0);
                }
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (q + u * G < e) acc = fma_t(vv[u], xv[u], acc);
            }
        } else {
            for (; q + 3 * G < e; q += 4 * G) {
                const int c0 = M.idx[q], c1 = M.idx[q + G];
                const int c2 = M.idx[q + 2 * G], c3 = M.idx[q + 3 * G];
                const V v0 = M.val[q], v1 = M.val[q + G];
                const V v2 = M.val[q + 2 * G], v3 = M.val[q + 3 * G];
                const V x0 = xf(c0), x1 = xf(c1), x2 = xf(c2), x3 = xf(c3);
                acc = fma_t(v0, x0, acc);
                acc = fma_t(v1, x1, acc);
                acc = fma_t(v2, x2, acc);
                acc = fma_t(v3, x3, acc);
            }
            for (; q < e; q += G) acc = fma_t(M.val[q], xf(M.idx[q]), acc);
        }
        for (int o = G >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (row < M.rows && sub == 0) ep(M.row0 + row, acc);
    }
}

// Rows [lo, hi) of a CSR matrix in HBM, read in place.
template <class V>
HELP_DEVINL LocalCsr<V> global_rows(const SpmvView<V>& M, int lo, int hi, int G) {
    LocalCsr<V> L;
    L.ptr = M.ptr + lo;  // absolute offsets into idx / val
    L.idx = M.idx;
    L.val = M.val;
    L.rows = hi - lo;
    L.row0 = lo;
    L.G = G;
    return L;
}

// Copies rows [lo, hi) of a CSR matrix in HBM into shared memory (pointers
// rebased to 0); returns the slice.
template <class V>
HELP_DEVINL LocalCsr<V> load_rows(const SpmvView<V>& M, int lo, int hi, int G, int* sp, int* si, V* sv) {
    const int b = ld_ro(M.ptr + lo);
    for (int r = threadIdx.x; r <= hi - lo; r += kResThreads) sp[r] = ld_ro(M.ptr + lo + r) - b;
    const int e = ld_ro(M.ptr + hi);
    for (int q = threadIdx.x; q < e - b; q += kResThreads) {
        si[q] = ld_ro(M.idx + b + q);
        sv[q] = ld_ro(M.val + b + q);
    }
    LocalCsr<V> L;
    L.ptr = sp;
    L.idx = si;
    L.val = sv;
    L.rows = hi - lo;
    L.row0 = lo;
    L.G = G;
    return L;
}

// Copies buf[lo, hi) of this CTA into the same range of every other CTA's
// buf.  lo * sizeof(V) and buf are 16-byte aligned (slices start at multiples
// of 4 elements), so the body moves 16-byte words.  All (destination, word)
// pairs in one pass over the whole CTA: a DSMEM store round costs ~250 cycles
// whatever its width, so a short slice pushed destination by destination
// would leave most threads idle.
template <class V>
HELP_DEVINL void push_slice(cg::cluster_group& cl, V* buf, int lo, int hi, int rank, int cs) {
    if (hi <= lo) return;
    constexpr int kPer16 = 16 / (int)sizeof(V);
    const int n16 = (hi - lo) / kPer16;
    const int per = n16 + (hi - lo - n16 * kPer16);  // 16-byte words, then single elements
    const int total = (cs - 1) * per;
    const uint4* src = reinterpret_cast<const uint4*>(buf + lo);
    for (int x = threadIdx.x; x < total; x += kResThreads) {
        const int d = x / per, e = x - d * per;
        V* dbuf = cl.map_shared_rank(buf, (rank + 1 + d) % cs);
        if (e < n16) {
            reinterpret_cast<uint4*>(dbuf + lo)[e] = src[e];
        } else {
            const int i = lo + n16 * kPer16 + (e - n16);
            dbuf[i] = buf[i];
        }
    }
}

// Deterministic block-wide sums of two values at once (the tree of
// block_sum); results valid in every thread.
HELP_DEVINL void block_sum2(double& u, double& v, double2* red2) {
    const int tid = threadIdx.x;
    __syncthreads();
    red2[tid] = make_double2(u, v);
    __syncthreads();
    for (int s = blockDim.x >> 1; s >= 32; s >>= 1) {
        if (tid < s) {
            const double2 a = red2[tid], b = red2[tid + s];
            red2[tid] = make_double2(a.x + b.x, a.y + b.y);
        }
        __syncthreads();
    }
    if (tid < 32) {
        double2 w = red2[tid];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            w.x += __shfl_xor_sync(0xffffffffu, w.x, o);
            w.y += __shfl_xor_sync(0xffffffffu, w.y, o);
        }
        if (tid == 0) red2[0] = w;
    }
    __syncthreads();
    u = red2[0].x;
    v = red2[0].y;
}

// Sum over the 16 lanes of a half warp (xor butterfly: identical in every
// lane of the half, and in every CTA for the same inputs).
HELP_DEVINL double half_sum(double v) {
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// First position in a[b, e) (ascending) whose value is >= v.
HELP_DEVINL int lower_bound_i(const int* a, int b, int e, int v) {
    while (b < e) {
        const int mid = b + ((e - b) >> 1);
        if (ld_ro(a + mid) < v) b = mid + 1;
        else e = mid;
    }
    return b;
}

template <class V, bool kMatSmem, bool kTsmem>
__global__ void __launch_bounds__(kResThreads, 1) k_cg_resident(const CgArgs<V> A, const ResLayout L, int iters) {
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ double2 red2[kResThreads];
    double* red = reinterpret_cast<double*>(red2);
    __shared__ int s_plo, s_phi;
    __shared__ double s_sc[5];  // rr, rz, beta, p.q, alpha formed by warp 0
    __shared__ double s_inv_rz;  // 1 / rz of the previous iteration
    double* a = reinterpret_cast<double*>(sm + L.a);
    double* w = reinterpret_cast<double*>(sm + L.w);
    double* awp = reinterpret_cast<double*>(sm + L.awp);  // a_l w_l
    double* kpart = reinterpret_cast<double*>(sm + L.kpart);  // [cs][k] C^T z_N partials
    double* s_rz = reinterpret_cast<double*>(sm + L.s_rz);    // [cs] partials
    double* s_rr = reinterpret_cast<double*>(sm + L.s_rr);
    double* s_pq = reinterpret_cast<double*>(sm + L.s_pq);
    double* Wm = reinterpret_cast<double*>(sm + L.W);  // k x k, symmetric
    V* pf = reinterpret_cast<V*>(sm + L.pf);
    constexpr bool kTinL2 = !kTsmem;                  // where t = B^T p is exchanged (see step iii)
    V* tf = reinterpret_cast<V*>(sm + L.tf);          // full copy of t when kTsmem
    V* xl = reinterpret_cast<V*>(sm + L.xl);
    V* rl = reinterpret_cast<V*>(sm + L.rl);
    V* zl = reinterpret_cast<V*>(sm + L.zl);
    V* ql = reinterpret_cast<V*>(sm + L.ql);
    V* dl = reinterpret_cast<V*>(sm + L.dl);  // D_S^-1 on own rows
    V* rP = reinterpret_cast<V*>(sm + L.rp);
    V* qP = reinterpret_cast<V*>(sm + L.qp);
    int* pvl = reinterpret_cast<int*>(sm + L.pvl);  // pivot position of own rows (-1: not a pivot)
    int* pv = reinterpret_cast<int*>(sm + L.piv);   // pivot rows, ascending
    int* ctp = reinterpret_cast<int*>(sm + L.ct_p); // own entries of C^T: row l in [ctp[l], ctp[l+1])
    int* cti = reinterpret_cast<int*>(sm + L.ct_i); //   local row index
    int* ctb = reinterpret_cast<int*>(sm + L.ct_b); // first own entry of C^T row l in HBM
    V* ctv = reinterpret_cast<V*>(sm + L.ct_v);

    CgScalars* sc = A.sc;
    if (*(volatile const int*)&sc->done != 0) return;  // same value in every CTA (written before this launch)
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int rank = (int)cl.block_rank(), cs = (int)cl.num_blocks();
    const int k = A.k;
    const int lo = min(A.m, rank * L.lr), hi = min(A.m, lo + L.lr);
    const int clo = min(A.n, rank * L.lc), chi = min(A.n, clo + L.lc);
    long long it = sc->it;
    double rz_old = sc->rz_old, rz = sc->rz, rr = sc->rr, alpha = sc->alpha, beta = sc->beta;
    const double term2 = sc->term2;
    const long long max_it = sc->max_iter;
    const bool has_delta = (A.delta != 0.0);
    const V vd = (V)A.delta;

    // matrix slices and the state of CG iteration `it` into shared memory
    LocalCsr<V> Bl, Bt, Cl;
    if constexpr (kMatSmem) {
        Bl = load_rows<V>(A.csr, lo, hi, L.g_b, reinterpret_cast<int*>(sm + L.csr_p),
                          reinterpret_cast<int*>(sm + L.csr_i), reinterpret_cast<V*>(sm + L.csr_v));
        Bt = load_rows<V>(A.csc, clo, chi, L.g_bt, reinterpret_cast<int*>(sm + L.csc_p),
                          reinterpret_cast<int*>(sm + L.csc_i), reinterpret_cast<V*>(sm + L.csc_v));
        Cl = load_rows<V>(A.c, lo, hi, L.g_c, reinterpret_cast<int*>(sm + L.c_p),
                          reinterpret_cast<int*>(sm + L.c_i), reinterpret_cast<V*>(sm + L.c_v));
    } else {
        // larger systems: the slices stay in HBM / L2 and are read every
        // iteration (each barrier invalidates L1)
        Bl = global_rows<V>(A.csr, lo, hi, L.g_b);
        Bt = global_rows<V>(A.csc, clo, chi, L.g_bt);
        Cl = global_rows<V>(A.c, lo, hi, L.g_c);
    }
    {
        const V* r = (it & 1) ? A.r1 : A.r0;
        const V* p = (it & 1) ? A.p1 : A.p0;
        for (int i = tid; i < A.m; i += kResThreads) pf[i] = p[i];
        for (int i = lo + tid; i < hi; i += kResThreads) {
            xl[i - lo] = A.x[i];
            rl[i - lo] = r[i];
            dl[i - lo] = ld_ro(A.dsinv + i);
            pvl[i - lo] = ld_ro(A.pivpos + i);
        }
        for (int e = tid; e < k * k; e += kResThreads) Wm[e] = ld_ro(A.W + e);
        for (int l = tid; l < k; l += kResThreads) {
            pv[l] = ld_ro(A.piv + l);
            rP[l] = r[pv[l]];
            a[l] = A.a[l];
            // this CTA's entries of row l of C^T (row indices ascending)
            const int b = ld_ro(A.ct.ptr + l), e = ld_ro(A.ct.ptr + l + 1);
            const int qb = lower_bound_i(A.ct.idx, b, e, lo);
            ctb[l] = qb;
            ctp[l + 1] = lower_bound_i(A.ct.idx, b, e, hi) - qb;
        }
        if (tid == 0) {
            s_inv_rz = (rz_old != 0.0) ? 1.0 / rz_old : 0.0;
            // pivots are in increasing row order: this CTA's pivot rows are l in [plo, phi)
            s_plo = lower_bound_i(A.piv, 0, k, lo);
            s_phi = lower_bound_i(A.piv, 0, k, hi);
        }
    }
    __syncthreads();
    if (tid == 0) {
        ctp[0] = 0;
        for (int l = 0; l < k; ++l) ctp[l + 1] += ctp[l];
    }
    __syncthreads();
    for (int l = warp; l < k; l += kResWarps) {
        const int o = ctp[l], cnt = ctp[l + 1] - o, qb = ctb[l];
        for (int j = lane; j < cnt; j += 32) {
            cti[o + j] = ld_ro(A.ct.idx + qb + j) - lo;
            ctv[o + j] = ld_ro(A.ct.val + qb + j);
        }
    }
    // every CTA has started and loaded its state before any CTA stores into it
    cl.sync();
    const int plo = s_plo, phi = s_phi;

    int done = 0;
    double prr = 0.0;  // this CTA's r.r of the last step (iv); reduced with the next r_N.z_N
    for (int u = 0;; ++u) {
        // (i) z_N on own rows; r_N.z_N and the previous r.r in one block
        // reduction; C^T z_N partials
        double prz = 0.0;
        rows_local<V, !kMatSmem>(
            Cl, [&](int l) { return (V)a[l]; },
            [&](int i, V s) {
                if (pvl[i - lo] < 0) {
                    const V ri = rl[i - lo];
                    const V zi = dl[i - lo] * (ri - s);
                    zl[i - lo] = zi;
                    prz = fma((double)ri, (double)zi, prz);
                }
            });
        block_sum2(prz, prr, red2);  // also: zl complete
        if (tid < cs) {
            *cl.map_shared_rank(s_rz + rank, tid) = prz;
            *cl.map_shared_rank(s_rr + rank, tid) = prr;
        }
        // C^T z_N over this CTA's rows, one thread per (pivot l, CTA c): the
        // cs threads of a pivot form the same sum in the same warp
        // instructions, and each stores it into one CTA
        for (int t = tid; t < k * cs; t += kResThreads) {
            const int l = t / cs, c = t - l * cs;
            V acc = V(0);
            for (int q = ctp[l]; q < ctp[l + 1]; ++q) acc = fma_t(ctv[q], zl[cti[q]], acc);
            *cl.map_shared_rank(kpart + (size_t)rank * k + l, c) = (double)acc;
        }
        cl.sync();
        // w = r_P - sum over CTAs of C^T z_N: a half warp per pivot, one lane
        // per CTA.  (Every FP64 warp instruction holds a sub-partition's FP64
        // pipe for ~64 cycles however few lanes are active, so the scalar work
        // is spread over the warps as short trees, not long serial chains.)
        for (int l0 = 2 * warp; l0 < k; l0 += 2 * kResWarps) {
            const int l = l0 + (lane >> 4), c = lane & 15;
            const double v = half_sum((l < k && c < cs) ? kpart[(size_t)c * k + l] : 0.0);
            if (l < k && c == 0) {
                const double wl = (double)rP[l] - v;
                w[l] = wl;
                awp[l] = a[l] * wl;
            }
        }
        __syncthreads();
        // r.r of the previous step, rz = r_N.z_N + a.w (the CTAs' r_N.z_N
        // and the a_l w_l in one warp sum), beta
        if (warp == 0) {
            const double rr_new = half_sum(lane < cs ? s_rr[lane] : 0.0);
            double v = lane < cs ? s_rz[lane] : 0.0;
            for (int l = lane; l < k; l += 32) v += awp[l];
            const double rz_new = warp_sum(v);
            if (lane == 0) {
                s_sc[0] = rr_new;
                s_sc[1] = rz_new;
                s_sc[2] = (it == 0) ? 0.0 : rz_new * s_inv_rz;
            }
        }
        __syncthreads();
        if (u > 0) {
            rr = s_sc[0];
            if (!(rr == rr)) done = 3;
            else if (rr < term2 || rr == 0.0) done = 1;
            else if (it >= max_it) done = 2;
            if (done != 0) break;
        }
        if (u == iters) break;

        // (ii) z_P = W w on own pivot rows (W symmetric: column l = row l; a
        // half warp per pivot), p = z + beta p on own rows
        rz = s_sc[1];
        if (!(rz > 0.0)) {
            done = 3;
            break;
        }
        beta = s_sc[2];
        for (int l0 = plo + 2 * warp; l0 < phi; l0 += 2 * kResWarps) {
            const int l = l0 + (lane >> 4), c = lane & 15;
            double acc = 0.0;
            if (l < phi)
                for (int c2 = c; c2 < k; c2 += 16) acc = fma(Wm[c2 * k + l], w[c2], acc);
            acc = half_sum(acc);
            if (l < phi && c == 0) zl[pv[l] - lo] = (V)acc;
        }
        __syncthreads();
        {
            const bool first = (it == 0);
            const V vb = (V)beta;
            for (int i = lo + tid; i < hi; i += kResThreads) {
                const V zi = zl[i - lo];
                pf[i] = first ? zi : fma_t(vb, pf[i], zi);
            }
        }
        __syncthreads();
        push_slice(cl, pf, lo, hi, rank, cs);
        cl.sync();

        // (iii) t = B^T p on own columns.  FP64: to L2, from where every CTA
        // gathers the t it needs after the barrier -- measured cheaper than
        // copying all of t (8n bytes) into every CTA's shared memory through
        // DSMEM (~32 GB/s per SM).  FP32: half the bytes, and the DSMEM copy
        // wins where the copy fits in shared memory.
        if constexpr (kTinL2) {
            rows_local<V, !kMatSmem>(Bt, [&](int i) { return pf[i]; }, [&](int j, V s) { A.t[j] = s; });
        } else {
            rows_local<V, !kMatSmem>(Bt, [&](int i) { return pf[i]; }, [&](int j, V s) { tf[j] = s; });
            __syncthreads();
        }
        // 1 / rz for the next beta
        if (warp == kResWarps - 1 && lane == 0) s_inv_rz = 1.0 / rz;
        if constexpr (!kTinL2) push_slice(cl, tf, clo, chi, rank, cs);
        cl.sync();

        // (iv) q = B t + delta p on own rows, p.q partial, q on own pivot rows
        double ppq = 0.0;
        rows_local<V, kTinL2 || !kMatSmem>(
            Bl, [&](int j) { return kTinL2 ? __ldcg(A.t + j) : tf[j]; },
            [&](int i, V s) {
                const V pi = pf[i];
                const V qi = has_delta ? fma_t(vd, pi, s) : s;
                ql[i - lo] = qi;
                ppq = fma((double)pi, (double)qi, ppq);
            });
        ppq = block_sum(ppq, red);  // also: ql complete
        if (tid < cs) *cl.map_shared_rank(s_pq + rank, tid) = ppq;
        for (int t = tid; t < (phi - plo) * cs; t += kResThreads) {
            const int l = plo + t / cs, c = t % cs;
            *cl.map_shared_rank(qP + l, c) = ql[pv[l] - lo];
        }
        cl.sync();
        if (warp == 0) {
            const double pq = half_sum(lane < cs ? s_pq[lane] : 0.0);
            if (lane == 0) {
                s_sc[3] = pq;
                s_sc[4] = rz / pq;
            }
        }
        __syncthreads();
        if (!(s_sc[3] > 0.0)) {
            done = 3;
            break;
        }
        alpha = s_sc[4];
        rz_old = rz;
        const V va = (V)alpha;
        prr = 0.0;
        for (int i = lo + tid; i < hi; i += kResThreads) {
            const V pi = pf[i], qi = ql[i - lo];
            xl[i - lo] = fma_t(va, pi, xl[i - lo]);
            const V ri = fma_t(-va, qi, rl[i - lo]);
            rl[i - lo] = ri;
            prr = fma((double)ri, (double)ri, prr);
        }
        // r_P as the owners computed it (same operands, same rounding), then
        // a = W r_P, a half warp per pivot
        if (warp == 0)
            for (int l = lane; l < k; l += 32) rP[l] = fma_t(-va, qP[l], rP[l]);
        __syncthreads();
        for (int l0 = 2 * warp; l0 < k; l0 += 2 * kResWarps) {
            const int l = l0 + (lane >> 4), c = lane & 15;
            double acc = 0.0;
            if (l < k)
                for (int c2 = c; c2 < k; c2 += 16) acc = fma(Wm[c2 * k + l], (double)rP[c2], acc);
            acc = half_sum(acc);
            if (l < k && c == 0) a[l] = acc;
        }
        __syncthreads();
        ++it;
    }
    // no CTA leaves while another can still store into its shared memory
    cl.sync();
    {
        V* r = (it & 1) ? A.r1 : A.r0;
        V* p = (it & 1) ? A.p1 : A.p0;
        for (int i = lo + tid; i < hi; i += kResThreads) {
            A.x[i] = xl[i - lo];
            r[i] = rl[i - lo];
            p[i] = pf[i];
        }
        if (rank == 0) {
            for (int l = tid; l < k; l += kResThreads) A.a[l] = a[l];
            if (tid == 0) {
                sc->it = it;
                sc->rr = rr;
                sc->rz = rz;
                sc->rz_old = rz_old;
                sc->alpha = alpha;
                sc->beta = beta;
                if (done == 3) sc->status = kStatusNumeric;
                if (done != 0) sc->done = done;
            }
        }
    }
}

cudaLaunchConfig_t resident_config(int cs, size_t smem, cudaStream_t st, cudaLaunchAttribute* at) {
    cudaLaunchConfig_t cfg = {};
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(kResThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cfg;
}

}  // namespace

namespace {

// Largest number of nonzeros in one CTA's slice of `per` consecutive rows.
int64_t slice_max(const int32_t* ptr, int rows, int per) {
    int64_t mx = 0;
    for (int lo = 0; lo < rows; lo += per) {
        const int hi = std::min(rows, lo + per);
        mx = std::max<int64_t>(mx, (int64_t)ptr[hi] - ptr[lo]);
    }
    return mx;
}

}  // namespace

ResLayout resident_layout(int m, int n, int k, int cs, int vbytes, const int32_t* rp, const int32_t* cp,
                          const int32_t* crp, bool mat_smem, bool t_smem) {
    ResLayout L = {};
    L.mat_smem = mat_smem ? 1 : 0;
    L.t_smem = t_smem ? 1 : 0;
    // slices of whole 16-byte words, so DSMEM copies move 16 bytes per store
    L.lr = (((m + cs - 1) / cs) + 3) & ~3;
    L.lc = (((n + cs - 1) / cs) + 3) & ~3;
    const size_t nnz_b = (size_t)slice_max(rp, m, L.lr), nnz_bt = (size_t)slice_max(cp, n, L.lc);
    const size_t nnz_c = (size_t)slice_max(crp, m, L.lr);
    // lanes per row: each FP64 warp instruction costs the same pipe time
    // however many lanes it uses, so FP64 rows take ~8 nonzeros per lane
    // (fewer shuffle levels); FP32 rows ~4
    const int per_lane = vbytes == 8 ? 8 : 4;
    auto lanes = [&](int64_t nz, int rows) {
        const double avg = rows > 0 ? (double)nz / rows : 0.0;
        int g = 1;
        while (g < 32 && g * per_lane < avg) g *= 2;
        return g;
    };
    L.g_b = lanes(rp[m], m);
    L.g_bt = lanes(cp[n], n);
    L.g_c = lanes(crp[m], m);
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += (bytes + 15) & ~(size_t)15;
        return at;
    };
    const size_t kk = (size_t)(k > 0 ? k : 1), vb = (size_t)vbytes, lr = (size_t)L.lr, lc = (size_t)L.lc;
    L.a = take(8 * kk);
    L.w = take(8 * kk);
    L.awp = take(8 * kk);
    L.kpart = take(8 * kk * cs);
    L.s_rz = take(8 * (size_t)cs);
    L.s_rr = take(8 * (size_t)cs);
    L.s_pq = take(8 * (size_t)cs);
    L.W = take(8 * kk * kk);
    L.pf = take(vb * m);
    L.tf = take(t_smem ? vb * n : 16);
    L.xl = take(vb * lr);
    L.rl = take(vb * lr);
    L.zl = take(vb * lr);
    L.ql = take(vb * lr);
    L.dl = take(vb * lr);
    L.rp = take(vb * kk);
    L.qp = take(vb * kk);
    L.pvl = take(4 * lr);
    L.piv = take(4 * kk);
    L.ct_p = take(4 * (kk + 1));
    L.ct_b = take(4 * kk);
    L.ct_i = take(4 * std::max<size_t>(nnz_c, 1));
    L.ct_v = take(vb * std::max<size_t>(nnz_c, 1));
    if (mat_smem) {
        L.csr_p = take(4 * (lr + 1));
        L.csr_i = take(4 * std::max<size_t>(nnz_b, 1));
        L.csr_v = take(vb * std::max<size_t>(nnz_b, 1));
        L.csc_p = take(4 * (lc + 1));
        L.csc_i = take(4 * std::max<size_t>(nnz_bt, 1));
        L.csc_v = take(vb * std::max<size_t>(nnz_bt, 1));
        L.c_p = take(4 * (lr + 1));
        L.c_i = take(4 * std::max<size_t>(nnz_c, 1));
        L.c_v = take(vb * std::max<size_t>(nnz_c, 1));
    }
    L.total = o;
    return L;
}

// The kernel for a layout: FP64 always exchanges t through L2 (measured
// faster), FP32 through shared memory where t fits there.
template <class V>
const void* resident_fn(bool mat_smem, bool t_smem) {
    if constexpr (sizeof(V) == 8) {
        return mat_smem ? (const void*)k_cg_resident<V, true, false> : (const void*)k_cg_resident<V, false, false>;
    } else {
        if (mat_smem) return t_smem ? (const void*)k_cg_resident<V, true, true> : (const void*)k_cg_resident<V, true, false>;
        return t_smem ? (const void*)k_cg_resident<V, false, true> : (const void*)k_cg_resident<V, false, false>;
    }
}

// Cluster size (16, else 8) at which k_cg_resident fits the system in shared
// memory and the GPU can co-schedule the cluster; 0 if none.  Tries the
// matrix slices in shared memory first, then (for at most kResidentL2Work
// per iteration) in L2.  rp, cp, crp: host row pointers of B, B^T and C.
// *L gets the layout.
template <class V>
int cg_resident_configure(int m, int n, int k, const int32_t* rp, const int32_t* cp, const int32_t* crp,
                          ResLayout* L) {
    if (k > kResidentMaxPivots) return 0;
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    const int64_t work = 2 * ((int64_t)rp[m] + crp[m]);
    const size_t static_bytes = 2 * sizeof(double) * kResThreads + 128;
    for (int variant = 0; variant < 4; ++variant) {
        const bool mat_smem = variant < 2, t_smem = (variant & 1) == 0;
        if (!mat_smem && work > kResidentL2Work) break;
        if (t_smem && sizeof(V) == 8) continue;
        const void* fn = resident_fn<V>(mat_smem, t_smem);
        for (int cs : {16, 8}) {
            const ResLayout lay = resident_layout(m, n, k, cs, (int)sizeof(V), rp, cp, crp, mat_smem, t_smem);
            if (lay.total + static_bytes > (size_t)optin) continue;
            if (raise_smem_limit(fn, (int)lay.total) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            if (cs > 8 && cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            cudaLaunchAttribute at[1];
            cudaLaunchConfig_t cfg = resident_config(cs, lay.total, nullptr, at);
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg) == cudaSuccess && nclusters >= 1) {
                *L = lay;
                return cs;
            }
            cudaGetLastError();
        }
    }
    return 0;
}

// Up to `iters` CG iterations in one launch of one cluster of `cs` CTAs.
template <class V>
cudaError_t cg_launch_resident(const CgArgs<V>& A, const ResLayout& L, int cs, int iters, cudaStream_t st) {
    const void* fn = resident_fn<V>(L.mat_smem != 0, L.t_smem != 0);
    const cudaError_t e = raise_smem_limit(fn, (int)L.total);
    if (e != cudaSuccess) return e;
    cudaLaunchAttribute at[1];
    cudaLaunchConfig_t cfg = resident_config(cs, L.total, st, at);
    void* args[] = {(void*)&A, (void*)&L, (void*)&iters};
    return cudaLaunchKernelExC(&cfg, fn, args);
}

template int cg_resident_configure<double>(int, int, int, const int32_t*, const int32_t*, const int32_t*,
                                          ResLayout*);
template int cg_resident_configure<float>(int, int, int, const int32_t*, const int32_t*, const int32_t*,
                                         ResLayout*);
template cudaError_t cg_launch_resident<double>(const CgArgs<double>&, const ResLayout&, int, int, cudaStream_t);
template cudaError_t cg_launch_resident<float>(const CgArgs<float>&, const ResLayout&, int, int, cudaStream_t);

}  // namespace help
