// Preconditioned conjugate gradient on G x = b, G = B B^T + delta I,
// B = A D^-1/2 -- the loop of ConjugateGradient (PCG.cpp:296-395) with the
// partial-Cholesky preconditioner of PCG.cpp:183-196 applied in block form.
//
// Each iteration is six kernels, captured once into a CUDA graph that runs
// several iterations per launch; the host only polls a device flag between
// graph launches.  Scalars (alpha, beta, the stopping test) are formed on the
// device: every kernel that ends a reduction has each block write its partial
// sum, and the last block to finish (ticket counter) adds the partials in
// block order -- so the run is deterministic -- and publishes the scalar for
// the next kernel.  Every kernel first reads the `done` flag and returns at
// once when the solve has finished, so a graph launched past convergence
// costs only empty launches.  No kernel waits on another block.
//
// Preconditioner M = [L11 0; L21 I] diag(D1, D_S) [L11 0; L21 I]^T on the k
// pivot rows P is applied without the dense L21 the reference materialises
// (PCG.cpp:143-155).  With C = G[N, P] (N = non-pivot rows), W = G11^-1:
//     a   = W r_P            (end of the previous iteration)
//     z_N = D_S^-1 (r_N - C a)
//     w   = r_P - C^T z_N
//     z_P = W w
// and r_P . z_P = a . w (W symmetric), so beta is known before p is formed.
//   k_p2 : z_N, r_N.z_N                      k_p3 : w, a.w  -> rz, beta
//   k_p4 : z_P, p_new = z + beta p           k_a  : t = B^T p_new
//   k_b  : q = B t + delta p_new, p.q -> alpha
//   k_c  : x += alpha p, r -= alpha q, r.r -> stop?, a = W r_P
// Vectors are V (double, or float for the inner solves of mixed precision);
// dot products, alpha/beta and the pivot-block work stay in double.
#include <cooperative_groups.h>

#include <algorithm>
#include <map>
#include <mutex>

#include "common.cuh"
#include "kernels.h"
#include "spmv.cuh"

namespace cg = cooperative_groups;

namespace help {

namespace {

constexpr int kCgThreads = 256;

// Sum of the per-block partials (in block order) by the calling block.
HELP_DEVINL double sum_parts(const double* p, const double* p2, int nb, double* red) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += p2 ? p[b] + p2[b] : p[b];
    return block_sum(s, red);
}

// Writes this block's partial and returns true in the last block to finish.
// The barrier first: the ticket announces every write of the block (k_p3's
// w entries come from any of its warps), so no thread may still be writing
// when thread 0 fences and takes it.
HELP_DEVINL bool publish_partial(double v, double* part, unsigned int* ticket) {
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        part[blockIdx.x] = v;
        __threadfence();
        const unsigned int t = atomicAdd(ticket, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last) __threadfence();
    return s_last != 0;
}

HELP_DEVINL bool cg_done(const CgScalars* sc) { return *(volatile const int*)&sc->done != 0; }

// out(c, (W y)_c) for the rows c of W owned by this block's warps (k x k, row-major).
template <class YF, class OUT>
HELP_DEVINL void gemv_rows(int k, const double* __restrict__ W, const YF& yf, const OUT& out, double* s_vec) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    const bool active = (long long)blockIdx.x * nw < k;
    if (active)
        for (int c = tid; c < k; c += blockDim.x) s_vec[c] = yf(c);
    __syncthreads();
    if (active) {
        for (int c = blockIdx.x * nw + warp; c < k; c += gridDim.x * nw) {
            const double* Wr = W + (size_t)c * k;
            double acc = 0.0;
            for (int c2 = lane; c2 < k; c2 += 32) acc = fma(ld_ro(Wr + c2), s_vec[c2], acc);
            acc = warp_sum(acc);
            if (lane == 0) out(c, acc);
        }
    }
    __syncthreads();
}

// ---- initial: r.r and a = W r_P of the starting residual (buffer 0)
template <class V>
__global__ void __launch_bounds__(kCgThreads) k_init(const CgArgs<V> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* s_vec = reinterpret_cast<double*>(smem_raw);
    __shared__ double red[kCgThreads];
    const V* r = A.r0;
    double rr = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < A.m; i += (long long)gridDim.x * blockDim.x) {
        const double v = (double)r[i];
        rr = fma(v, v, rr);
    }
    rr = block_sum(rr, red);
    gemv_rows(A.k, A.W, [&](int c) { return (double)r[A.piv[c]]; }, [&](int c, double s) { A.a[c] = s; }, s_vec);
    if (publish_partial(rr, A.part_rr, &A.sc->ticket[0])) {
        const double tot = sum_parts(A.part_rr, nullptr, gridDim.x, red);
        if (threadIdx.x == 0) {
            CgScalars* sc = A.sc;
            sc->ticket[0] = 0;
            sc->rr0 = tot;
            sc->rr = tot;
            sc->term2 = tot * sc->tol2;
            sc->it = 0;
            sc->status = 0;
            if (!(tot == tot)) {
                sc->status = kStatusNumeric;
                sc->done = 3;
            } else if (tot == 0.0 || sc->max_iter <= 0) {
                sc->done = (tot == 0.0) ? 1 : 2;
            } else {
                sc->done = 0;
            }
        }
    }
}

// ---- P2: z_N = D_S^-1 (r_N - C a), partial r_N . z_N
// a (k values) is gathered once per nonzero of C: copied into each block's
// shared memory when C is large against the copies (A.stage_a, set by the
// host; k <= kStageA).  Measured on config 2 (k = 1,024, 10M entries in C):
// FP32 iteration 315 -> 298 us, FP64 unchanged (FP64-issue-bound).
constexpr int kStageA = 8192;
template <class V>
__global__ void __launch_bounds__(kCgThreads) k_p2(const CgArgs<V> A) {
    if (cg_done(A.sc)) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V* s_a = reinterpret_cast<V*>(smem_raw);
    __shared__ double red[kCgThreads];
    const V* r = (A.sc->it & 1) ? A.r1 : A.r0;
    const bool staged = A.stage_a != 0;
    if (staged) {
        for (int c = threadIdx.x; c < A.k; c += blockDim.x) s_a[c] = (V)A.a[c];
        __syncthreads();
    }
    double rz = 0.0;
    spmv_rows<V>(
        A.c, [&](int c) { return staged ? s_a[c] : (V)A.a[c]; },
        [&](int i, V s) {
            if (A.pivpos[i] < 0) {
                const V ri = r[i];
                const V zi = A.dsinv[i] * (ri - s);
                A.z[i] = zi;
                rz = fma((double)ri, (double)zi, rz);
            }
        },
        [&](int i, V s) {  // long rows: their r.z terms are added by k_p3's last block
            if (A.pivpos[i] < 0) A.z[i] = A.dsinv[i] * (r[i] - s);
        },
        red);
    rz = block_sum(rz, red);
    if (threadIdx.x == 0) A.part_rz[blockIdx.x] = rz;
}

// Fixed-order sum over the long rows of M of term(row), by the calling block.
template <class V, class T>
HELP_DEVINL double long_rows_sum(const SpmvView<V>& M, const T& term, double* red) {
    double s = 0.0;
    for (int j = threadIdx.x; j < M.n_long; j += blockDim.x) s += term(M.long_rows[j]);
    return block_sum(s, red);
}

// ---- P3: w = r_P - C^T z_N; last block: rz = r_N.z_N + a.w, beta
template <class V>
__global__ void __launch_bounds__(kCgThreads) k_p3(const CgArgs<V> A) {
    if (cg_done(A.sc)) return;
    __shared__ double red[kCgThreads];
    const V* r = (A.sc->it & 1) ? A.r1 : A.r0;
    spmv_rows<V>(
        A.ct, [&](int i) { return A.z[i]; },
        [&](int c, V s) { A.w[c] = (double)r[A.piv[c]] - (double)s; }, red);
    if (publish_partial(0.0, A.part_aw, &A.sc->ticket[1])) {
        // every block has written its w entries.  rz = k_p2's partials (same
        // grid) + a . w over all k (= r_P . z_P) + the r.z terms of C's long
        // rows: each thread sums its share of the three in a fixed order, then
        // one block reduction
        double acc = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) acc += A.part_rz[b];
        for (int c = threadIdx.x; c < A.k; c += blockDim.x) acc = fma(A.a[c], __ldcg(A.w + c), acc);
        for (int j = threadIdx.x; j < A.c.n_long; j += blockDim.x) {
            const int i = A.c.long_rows[j];
            if (A.pivpos[i] < 0) acc = fma((double)__ldcg(r + i), (double)__ldcg(A.z + i), acc);
        }
        const double rz = block_sum(acc, red);
        if (threadIdx.x == 0) {
            CgScalars* sc = A.sc;
            sc->ticket[1] = 0;
            if (!(rz > 0.0)) {  // M^-1 not positive on r, or NaN
                sc->status = kStatusNumeric;
                sc->done = 3;
            } else {
                sc->beta = (sc->it == 0) ? 0.0 : rz / sc->rz_old;
                sc->rz = rz;
            }
        }
    }
}

// ---- P4: z_P = W w, p_new = z + beta p
template <class V>
__global__ void __launch_bounds__(kCgThreads) k_p4(const CgArgs<V> A) {
    if (cg_done(A.sc)) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* s_vec = reinterpret_cast<double*>(smem_raw);
    const long long it = A.sc->it;
    const V* p = (it & 1) ? A.p1 : A.p0;
    V* pn = (it & 1) ? A.p0 : A.p1;
    const bool first = (it == 0);
    const V vb = (V)A.sc->beta;
    gemv_rows(A.k, A.W, [&](int c) { return A.w[c]; },
              [&](int c, double s) {
                  const int i = A.piv[c];
                  const V zc = (V)s;
                  pn[i] = first ? zc : fma_t(vb, p[i], zc);
              },
              s_vec);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < A.m; i += (long long)gridDim.x * blockDim.x) {
        if (A.pivpos[i] < 0) {
            const V zi = A.z[i];
            pn[i] = first ? zi : fma_t(vb, p[i], zi);
        }
    }
}

// ---- A: t = B^T p_new
template <class V>
__global__ void __launch_bounds__(kCgThreads) k_a(const CgArgs<V> A) {
    if (cg_done(A.sc) || A.precond_only) return;
    __shared__ double red[kCgThreads];
    const V* pn = (A.sc->it & 1) ? A.p0 : A.p1;
    spmv_rows<V>(A.csc, [&](int i) { return pn[i]; }, [&](int j, V s) { A.t[j] = s; }, red);
}

// ---- B: q = B t + delta p_new, partial p.q; last block: alpha
template <class V>
__global__ void __launch_bounds__(kCgThreads) k_b(const CgArgs<V> A) {
    if (cg_done(A.sc) || A.precond_only) return;
    __shared__ double red[kCgThreads];
    const V* pn = (A.sc->it & 1) ? A.p0 : A.p1;
    const V vd = (V)A.delta;
    const bool has_delta = (A.delta != 0.0);
    double pq = 0.0;
    spmv_rows<V>(
        A.csr, [&](int j) { return A.t[j]; },
        [&](int i, V s) {
            const V pi = pn[i];
            const V qi = has_delta ? fma_t(vd, pi, s) : s;
            A.q[i] = qi;
            pq = fma((double)pi, (double)qi, pq);
        },
        [&](int i, V s) { A.q[i] = has_delta ? fma_t(vd, pn[i], s) : s; }, red);
    pq = block_sum(pq, red);
    if (publish_partial(pq, A.part_pq, &A.sc->ticket[2])) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) acc += __ldcg(A.part_pq + b);
        for (int j = threadIdx.x; j < A.csr.n_long; j += blockDim.x) {
            const int i = A.csr.long_rows[j];
            acc = fma((double)__ldcg(pn + i), (double)__ldcg(A.q + i), acc);
        }
        const double tot = block_sum(acc, red);
        if (threadIdx.x == 0) {
            CgScalars* sc = A.sc;
            sc->ticket[2] = 0;
            if (!(tot > 0.0)) {  // G not positive on p (breakdown) or NaN
                sc->status = kStatusNumeric;
                sc->done = 3;
            } else {
                sc->alpha = sc->rz / tot;
                sc->rz_old = sc->rz;
            }
        }
    }
}

// ---- C: x += alpha p, r_new = r - alpha q, r.r, a = W r_new_P; last block: stop?
template <class V>
__global__ void __launch_bounds__(kCgThreads) k_c(const CgArgs<V> A) {
    if (cg_done(A.sc) || A.precond_only) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* s_vec = reinterpret_cast<double*>(smem_raw);
    __shared__ double red[kCgThreads];
    const long long it = A.sc->it;
    const V* r = (it & 1) ? A.r1 : A.r0;
    V* rn = (it & 1) ? A.r0 : A.r1;
    const V* pn = (it & 1) ? A.p0 : A.p1;
    const V va = (V)A.sc->alpha;
    double rr = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < A.m; i += (long long)gridDim.x * blockDim.x) {
        const V pi = pn[i], qi = A.q[i];
        A.x[i] = fma_t(va, pi, A.x[i]);
        const V ri = fma_t(-va, qi, r[i]);
        rn[i] = ri;
        rr = fma((double)ri, (double)ri, rr);
    }
    rr = block_sum(rr, red);
    gemv_rows(A.k, A.W,
              [&](int c) {
                  const int i = A.piv[c];
                  return (double)fma_t(-va, A.q[i], r[i]);
              },
              [&](int c, double s) { A.a[c] = s; }, s_vec);
    if (publish_partial(rr, A.part_rr, &A.sc->ticket[3])) {
        const double tot = sum_parts(A.part_rr, nullptr, gridDim.x, red);
        if (threadIdx.x == 0) {
            CgScalars* sc = A.sc;
            sc->ticket[3] = 0;
            sc->rr = tot;
            sc->it = it + 1;  // buffers flip for the next iteration
            if (!(tot == tot)) {
                sc->status = kStatusNumeric;
                sc->done = 3;
            } else if (tot < sc->term2 || tot == 0.0) {
                sc->done = 1;
            } else if (sc->it >= sc->max_iter) {
                sc->done = 2;
            }
        }
    }
}

template <class V>
size_t gemv_smem(const CgArgs<V>& A) {
    return (size_t)(A.k > 0 ? A.k : 1) * sizeof(double);
}

// ---------------------------------------------------------------- one cluster
//
// For small systems the six launches of an iteration cost more than their
// work.  k_cg_cluster runs whole iterations inside one thread-block cluster
// (8 or 16 CTAs of 256 threads, one per SM): the same six phases, separated
// by hardware cluster barriers (barrier.cluster arrive.release /
// wait.acquire), with the dot products reduced through distributed shared
// memory -- every CTA reads the CTAs' partials in rank order, so all of them
// form bit-identical alpha, beta and stopping decisions and leave the loop
// together.  Vectors written inside the kernel are read with ld.global.cg
// (L2, coherent across the cluster's SMs); only the matrix and W go through
// the read-only path.  No CTA ever waits on a flag.

// 256 threads: measured on config 0 (m = 2,000, 30k nonzeros) at 27.7 us per
// iteration against 30.7 (512) and 39.8 (1024), the block reductions and
// barriers of the wide CTAs costing more than their extra parallelism.
constexpr int kClusterThreads = 256;

// Sum over the cluster's CTAs (rank order) of s_part[slot] (+ s_part[slot2]).
// Call after a cluster barrier that follows every CTA's write of its slots.
HELP_DEVINL double cluster_total(cg::cluster_group& cl, double* s_part, int slot, int slot2, double* s_out) {
    if (threadIdx.x < 32) {
        const unsigned int lane = threadIdx.x;
        double v = 0.0;
        if (lane < cl.num_blocks()) {
            const double* rp = cl.map_shared_rank(s_part, lane);
            v = rp[slot];
            if (slot2 >= 0) v += rp[slot2];
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double t = __shfl_down_sync(0xffffffffu, v, o);
            if ((lane & (2 * o - 1)) == 0) v += t;
        }
        if (lane == 0) *s_out = v;
    }
    __syncthreads();
    return *s_out;
}

template <class V>
__global__ void __launch_bounds__(kClusterThreads) k_cg_cluster(const CgArgs<V> A, int iters) {
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* s_vec = reinterpret_cast<double*>(smem_raw);
    __shared__ double red[kClusterThreads];
    __shared__ double s_part[4];
    __shared__ double s_tot[4];
    CgScalars* sc = A.sc;
    if (*(volatile const int*)&sc->done != 0) return;  // same value in every CTA (written before this launch)
    const int tid = threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long it = sc->it;
    double rz_old = sc->rz_old, rz = sc->rz, rr = sc->rr, alpha = sc->alpha, beta = sc->beta;
    const double term2 = sc->term2;
    const long long max_it = sc->max_iter;
    const bool has_delta = (A.delta != 0.0);
    const V vd = (V)A.delta;
    int done = 0;
    for (int u = 0; u < iters && done == 0; ++u) {
        const V* r = (it & 1) ? A.r1 : A.r0;
        V* rn = (it & 1) ? A.r0 : A.r1;
        const V* p = (it & 1) ? A.p1 : A.p0;
        V* pn = (it & 1) ? A.p0 : A.p1;
        // P2: z_N = D_S^-1 (r_N - C a)
        double prz = 0.0;
        spmv_rows<V>(
            A.c, [&](int c) { return (V)__ldcg(A.a + c); },
            [&](int i, V s) {
                if (A.pivpos[i] < 0) {
                    const V ri = __ldcg(r + i);
                    const V zi = A.dsinv[i] * (ri - s);
                    A.z[i] = zi;
                    prz = fma((double)ri, (double)zi, prz);
                }
            },
            [&](int i, V s) {
                if (A.pivpos[i] < 0) A.z[i] = A.dsinv[i] * (__ldcg(r + i) - s);
            },
            red);
        prz = block_sum(prz, red);
        if (tid == 0) s_part[0] = prz;
        cl.sync();
        // P3: w = r_P - C^T z_N
        spmv_rows<V>(
            A.ct, [&](int i) { return __ldcg(A.z + i); },
            [&](int c, V s) { A.w[c] = (double)__ldcg(r + A.piv[c]) - (double)s; }, red);
        cl.sync();
        {
            // a . w over all k and the long rows' r.z terms, the same in every CTA
            double acc = 0.0;
            for (int c = tid; c < A.k; c += blockDim.x) acc = fma(__ldcg(A.a + c), __ldcg(A.w + c), acc);
            for (int j = tid; j < A.c.n_long; j += blockDim.x) {
                const int i = A.c.long_rows[j];
                if (A.pivpos[i] < 0) acc = fma((double)__ldcg(r + i), (double)__ldcg(A.z + i), acc);
            }
            const double own = block_sum(acc, red);
            rz = cluster_total(cl, s_part, 0, -1, &s_tot[0]) + own;
        }
        if (!(rz > 0.0)) {
            done = 3;
            break;
        }
        beta = (it == 0) ? 0.0 : rz / rz_old;
        // P4: z_P = W w, p_new = z + beta p
        {
            const bool first = (it == 0);
            const V vb = (V)beta;
            gemv_rows(A.k, A.W, [&](int c) { return __ldcg(A.w + c); },
                      [&](int c, double s) {
                          const int i = A.piv[c];
                          const V zc = (V)s;
                          pn[i] = first ? zc : fma_t(vb, __ldcg(p + i), zc);
                      },
                      s_vec);
            for (long long i = blockIdx.x * (long long)blockDim.x + tid; i < A.m; i += stride) {
                if (A.pivpos[i] < 0) {
                    const V zi = __ldcg(A.z + i);
                    pn[i] = first ? zi : fma_t(vb, __ldcg(p + i), zi);
                }
            }
        }
        cl.sync();
        // A: t = B^T p_new
        spmv_rows<V>(A.csc, [&](int i) { return __ldcg(pn + i); }, [&](int j, V s) { A.t[j] = s; }, red);
        cl.sync();
        // B: q = B t + delta p_new
        double ppq = 0.0;
        spmv_rows<V>(
            A.csr, [&](int j) { return __ldcg(A.t + j); },
            [&](int i, V s) {
                const V pi = __ldcg(pn + i);
                const V qi = has_delta ? fma_t(vd, pi, s) : s;
                A.q[i] = qi;
                ppq = fma((double)pi, (double)qi, ppq);
            },
            [&](int i, V s) { A.q[i] = has_delta ? fma_t(vd, __ldcg(pn + i), s) : s; }, red);
        ppq = block_sum(ppq, red);
        if (tid == 0) s_part[2] = ppq;
        cl.sync();
        const double pql =
            long_rows_sum(A.csr, [&](int i) { return (double)__ldcg(pn + i) * (double)__ldcg(A.q + i); }, red);
        const double pq = cluster_total(cl, s_part, 2, -1, &s_tot[1]) + pql;
        if (!(pq > 0.0)) {
            done = 3;
            break;
        }
        alpha = rz / pq;
        rz_old = rz;
        // C: x += alpha p_new, r_new = r - alpha q, a = W r_new_P
        {
            const V va = (V)alpha;
            double prr = 0.0;
            for (long long i = blockIdx.x * (long long)blockDim.x + tid; i < A.m; i += stride) {
                const V pi = __ldcg(pn + i), qi = __ldcg(A.q + i);
                A.x[i] = fma_t(va, pi, __ldcg(A.x + i));
                const V ri = fma_t(-va, qi, __ldcg(r + i));
                rn[i] = ri;
                prr = fma((double)ri, (double)ri, prr);
            }
            prr = block_sum(prr, red);
            gemv_rows(A.k, A.W,
                      [&](int c) {
                          const int i = A.piv[c];
                          return (double)fma_t(-va, __ldcg(A.q + i), __ldcg(r + i));
                      },
                      [&](int c, double s) { A.a[c] = s; }, s_vec);
            if (tid == 0) s_part[3] = prr;
        }
        cl.sync();
        rr = cluster_total(cl, s_part, 3, -1, &s_tot[2]);
        ++it;
        if (!(rr == rr)) done = 3;
        else if (rr < term2 || rr == 0.0) done = 1;
        else if (it >= max_it) done = 2;
    }
    // no CTA may exit while another can still read its shared memory
    cl.sync();
    if (cl.block_rank() == 0 && tid == 0) {
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

}  // namespace

cudaError_t raise_smem_limit(const void* fn, int bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, int> limit;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    int& cur = limit[{fn, dev}];
    if (bytes <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

template <class V>
cudaError_t cg_configure(int k_max) {
    const int smem = (k_max > 0 ? k_max : 1) * (int)sizeof(double);
    cudaError_t e = raise_smem_limit((const void*)k_init<V>, smem);
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_p4<V>, smem);
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_c<V>, smem);
    if (e == cudaSuccess) e = raise_smem_limit((const void*)k_p2<V>, (int)(sizeof(V) * kStageA));
    return e;
}

template <class V>
cudaError_t cg_launch_init(const CgArgs<V>& A, int blocks, cudaStream_t st) {
    k_init<V><<<blocks, kCgThreads, gemv_smem(A), st>>>(A);
    return cudaGetLastError();
}

// One iteration's six kernels (captured into a graph by the caller).
template <class V>
cudaError_t cg_launch_iteration(const CgArgs<V>& A, int blocks, cudaStream_t st) {
    const size_t sm = gemv_smem(A);
    k_p2<V><<<blocks, kCgThreads, A.stage_a ? sizeof(V) * (size_t)A.k : 0, st>>>(A);
    k_p3<V><<<blocks, kCgThreads, 0, st>>>(A);
    k_p4<V><<<blocks, kCgThreads, sm, st>>>(A);
    k_a<V><<<blocks, kCgThreads, 0, st>>>(A);
    k_b<V><<<blocks, kCgThreads, 0, st>>>(A);
    k_c<V><<<blocks, kCgThreads, sm, st>>>(A);
    return cudaGetLastError();
}

int cg_threads() { return kCgThreads; }

int cg_blocks_per_sm() {
    static const int per_sm = [] {
        int lo = 0;
        auto take = [&](const void* f, size_t smem) {
            int b = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f, kCgThreads, smem) == cudaSuccess && b > 0)
                lo = lo ? std::min(lo, b) : b;
        };
        // dynamic shared memory: the k-vector copies are small against the
        // register limit at the pivot counts of the graph path
        take((const void*)k_p2<double>, 0);
        take((const void*)k_p3<double>, 0);
        take((const void*)k_p4<double>, 0);
        take((const void*)k_a<double>, 0);
        take((const void*)k_b<double>, 0);
        take((const void*)k_c<double>, 0);
        take((const void*)k_p2<float>, 0);
        take((const void*)k_p3<float>, 0);
        take((const void*)k_p4<float>, 0);
        take((const void*)k_a<float>, 0);
        take((const void*)k_b<float>, 0);
        take((const void*)k_c<float>, 0);
        cudaGetLastError();
        return lo > 0 ? lo : 8;
    }();
    return per_sm;
}

// Cluster size for k_cg_cluster: 16 CTAs where the GPU can co-schedule such a
// cluster with this shared memory, else 8 (the portable size); 0 if neither.
template <class V>
int cg_cluster_configure(int k_max) {
    const int smem = (k_max > 0 ? k_max : 1) * (int)sizeof(double);
    if (raise_smem_limit((const void*)k_cg_cluster<V>, smem) != cudaSuccess) return 0;
    for (int cs : {16, 8}) {
        if (cs > 8 && cudaFuncSetAttribute(k_cg_cluster<V>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                          cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(kClusterThreads);
        cfg.dynamicSmemBytes = smem;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, k_cg_cluster<V>, &cfg) == cudaSuccess && nclusters >= 1)
            return cs;
        cudaGetLastError();
    }
    return 0;
}

// Up to `iters` CG iterations in one launch of one cluster of `cs` CTAs.
template <class V>
cudaError_t cg_launch_cluster(const CgArgs<V>& A, int cs, int iters, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = gemv_smem(A);
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_cg_cluster<V>, A, iters);
}

template cudaError_t cg_configure<double>(int);
template cudaError_t cg_configure<float>(int);
template cudaError_t cg_launch_init<double>(const CgArgs<double>&, int, cudaStream_t);
template cudaError_t cg_launch_init<float>(const CgArgs<float>&, int, cudaStream_t);
template cudaError_t cg_launch_iteration<double>(const CgArgs<double>&, int, cudaStream_t);
template cudaError_t cg_launch_iteration<float>(const CgArgs<float>&, int, cudaStream_t);
template int cg_cluster_configure<double>(int);
template int cg_cluster_configure<float>(int);
template cudaError_t cg_launch_cluster<double>(const CgArgs<double>&, int, int, cudaStream_t);
template cudaError_t cg_launch_cluster<float>(const CgArgs<float>&, int, int, cudaStream_t);

}  // namespace help
