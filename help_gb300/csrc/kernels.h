// Host-callable launchers of the device kernels (one declaration list for
// api.cu).  All launches are asynchronous on the given stream.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "spmv.cuh"

namespace help {

// The dynamic shared-memory limit of a kernel is a property of the function
// (per device), shared by every context and host thread in the process:
// only ever raise it, so a context sizing a smaller system never lowers the
// limit under another context's launch (or graph capture).
cudaError_t raise_smem_limit(const void* fn, int bytes);

struct TopkStateDev {
    unsigned long long prefix;  // high bits of the threshold key decided so far
    unsigned long long mask;
    int remaining;              // rows still to take at or below the prefix
    int n_greater;              // rows strictly above the threshold
};

// Device-side scalars of one CG run (one set per context).
struct CgScalars {
    double rr0, rr, term2, rz, rz_old, alpha, beta;
    double tol2;          // set by the host: stop when r.r < tol2 * r0.r0
    long long it;
    long long max_iter;   // set by the host
    int done;             // 0 running, 1 converged, 2 iteration cap, 3 breakdown
    int status;
    unsigned int ticket[4];
};

// Device control block (one per context).
struct DevCtrl {
    int status;
    int regularised;
    CgScalars cg;
    TopkStateDev topk;
    int totals[8];
};

template <class V>
struct CgArgs {
    int m, n, k;
    SpmvView<V> csr, csc, c, ct;  // B, B^T, C = G[N, P], C^T
    const int* piv;
    const int* pivpos;
    const double* W;
    const V* dsinv;
    double delta;
    V* x;
    V* r0;
    V* r1;
    V* z;
    V* p0;
    V* p1;
    V* q;
    V* t;
    double* a;
    double* w;
    double* part_rr;  // gridDim doubles each
    double* part_rz;
    double* part_aw;
    double* part_pq;
    int precond_only;  // stop after the first preconditioner application (z in p1)
    int stage_a;       // k_p2 copies a into shared memory (k <= 8192, C large against blocks x k)
    CgScalars* sc;
};

template <class V>
cudaError_t cg_configure(int k_max);
template <class V>
cudaError_t cg_launch_init(const CgArgs<V>& A, int blocks, cudaStream_t st);
template <class V>
cudaError_t cg_launch_iteration(const CgArgs<V>& A, int blocks, cudaStream_t st);
int cg_threads();
// The fewest CTAs per SM any graph CG kernel (both precisions) keeps resident:
// the CG grid is at most this many x SMs, one wave.
int cg_blocks_per_sm();
// Single-cluster CG (small systems): cluster size 16 / 8 / 0 = unavailable.
template <class V>
int cg_cluster_configure(int k_max);
template <class V>
cudaError_t cg_launch_cluster(const CgArgs<V>& A, int cs, int iters, cudaStream_t st);

// Single-cluster CG with the vectors and the matrix slices in shared memory
// (pcg_resident.cu), for systems with at most kResidentMaxPivots pivots whose
// rows of B and B^T all hold <= 32 G nonzeros.  Byte offsets into the
// kernel's dynamic shared memory; lr / lc rows / columns per CTA.
constexpr int kResidentMaxPivots = 64;
// matrix slices read from L2 every iteration (when they do not fit shared
// memory) up to this much work per iteration, 2 (nnz(A) + nnz(C)): beyond
// it the whole-GPU graph's 152 SMs win over one cluster's 16 (measured FP64
// us per CG iteration, resident / graph: 29 / 43 at 120k nonzeros, 36 / 38
// at 117k (MCF), 42 / 43 at 150k with k = 64, 64 / 46 at 300k)
constexpr int64_t kResidentL2Work = 320000;
struct ResLayout {
    int lr, lc;
    int mat_smem;        // 1: matrix slices in shared memory, 0: read from L2
    int t_smem;          // 1: t = B^T p copied into every CTA (FP32), 0: exchanged through L2
    int g_b, g_bt, g_c;  // lanes per row of B, B^T, C
    size_t a, w, awp, kpart, s_rz, s_rr, s_pq, W, pf, tf, xl, rl, zl, ql, dl, rp, qp, pvl, piv, ct_p, ct_b, ct_i, ct_v,
        csr_p, csr_i, csr_v, csc_p, csc_i, csc_v, c_p, c_i, c_v, total;
};
ResLayout resident_layout(int m, int n, int k, int cs, int vbytes, const int32_t* rp, const int32_t* cp,
                          const int32_t* crp, bool mat_smem, bool t_smem);
template <class V>
int cg_resident_configure(int m, int n, int k, const int32_t* rp, const int32_t* cp, const int32_t* crp,
                          ResLayout* L);
template <class V>
cudaError_t cg_launch_resident(const CgArgs<V>& A, const ResLayout& L, int cs, int iters, cudaStream_t st);

// ---- standalone SpMV over items (vec.cu)
enum SpmvEpi {
    kEpiStore = 0,     // y[row] = s
    kEpiRhs = 1,       // y[row] = s - aux[row]                (A D^-1 b1 - b2)
    kEpiBacksub = 2,   // y[row] = s2[row] * (aux[row] - s)    (D^-1 (b1 - A^T x2))
    kEpiResid = 3,     // y[row] = aux[row] - (s + delta * aux2[row])  (rhs - G x)
    kEpiAddDelta = 4,  // y[row] = s + delta * aux[row]
    kEpiAcc = 5        // y[row] = aux[row] + delta * s        (delta = +-1: the HSD driver's A x / A^T y updates)
};
template <class V>
cudaError_t spmv_launch(int epi, const SpmvView<V>& M, const V* x, V* y, const V* aux, const V* aux2,
                        const double* s2, double delta, int blocks, int threads, cudaStream_t stream);

// ---- vector kernels (vec.cu)
cudaError_t vec_scale_mul(const double* a, const double* b, double* out, int64_t n, cudaStream_t st);  // out = a*b
// dst[q] = src[map[q]] (0 where map[q] < 0): a matrix's values into its sliced layout
template <class V>
cudaError_t sell_gather(const int* map, const V* src, V* dst, int64_t n, int num_sms, cudaStream_t st);
cudaError_t vec_to_f32(const double* a, float* out, int64_t n, cudaStream_t st);
cudaError_t vec_add_f32(double* x, const float* e, int64_t n, cudaStream_t st);  // x += e
cudaError_t vec_to_f32_scaled(const double* a, double scale, float* out, int64_t n, cudaStream_t st);
cudaError_t vec_add_f32_scaled(double* x, const float* e, double scale, int64_t n, cudaStream_t st);
cudaError_t vec_fill(double* x, double v, int64_t n, cudaStream_t st);
// dst = src (either may be host memory the device reaches directly)
cudaError_t vec_copy(const double* src, double* dst, int64_t n, int num_sms, cudaStream_t st);
// The fewest CTAs per SM any standalone SpMV kernel keeps resident: the grid
// of a standalone pass is this many x SMs, one wave.
int spmv_blocks_per_sm();
cudaError_t vec_fill_f32(float* x, float v, int64_t n, cudaStream_t st);
// Deterministic sum of squares into out[0] (uses `part` of >= 1024 doubles).
cudaError_t vec_sumsq(const double* x, int64_t n, double* part, double* out, cudaStream_t st);
// Deterministic x . y into out[0] (same scratch as vec_sumsq); x *= a.
cudaError_t vec_dot(const double* x, const double* y, int64_t n, double* part, double* out, cudaStream_t st);
cudaError_t vec_scale(double* x, double a, int64_t n, cudaStream_t st);

// ---- renew pipeline (renew.cu)
// s = d^-1/2 (status <- numeric error if some d_j is not positive and finite)
cudaError_t renew_inv_sqrt(const double* d, double* s, int n, int* status, cudaStream_t st);
// B = A diag(s) in both layouts (FP32 copies when bv32 / bvT32 are not null)
// and diag = rowsum(B .* B) + delta (status <- numeric error if some diag <= 0).
cudaError_t renew_scale_values(const double* s, const int* rp, const int* ci, const double* av, double* bv,
                               float* bv32, const int* cp, const double* avT, double* bvT, float* bvT32,
                               double* diag, double delta, int m, int n, int64_t nnz, int* status, cudaStream_t st);
// Top-k rows by key (diag >= 0); pivots ascending in piv[0..k), pivpos[m] = position or -1.
// flags: 3*m ints of scratch.
cudaError_t topk_select(const double* diag, int m, int k, unsigned long long* keys, unsigned int* hist,
                        int* flags, int* scan_tmp, TopkStateDev* tst, int* status, int* piv, int* pivpos,
                        cudaStream_t st);
size_t scan_tmp_elems(int64_t n);
// Exclusive scan of n int32 (in place allowed); writes the total to *total_dev if not null.
cudaError_t exclusive_scan(const int* in, int* out, int64_t n, int* tmp, int* total_dev, cudaStream_t st);
cudaError_t pivot_lists_count(const int* cp, const int* ri, const int* pivpos, int n, int* cnt, cudaStream_t st);
cudaError_t pivot_lists_fill(const int* cp, const int* ri, const double* bvT, const int* pivpos, int n,
                             const int* bp_ptr, int* bp_c, double* bp_v, cudaStream_t st);
size_t gcols_smem_bytes(int k);
int gcols_warps(int k);
// Row-wise G[i, P] (pass 0: counts per non-pivot row into cnt; pass 1: fill C rows / dense G11).
cudaError_t gcols_rows(int pass, const int* rp, const int* ci, const double* bv, const int* bp_ptr, const int* bp_c,
                       const double* bp_v, const int* pivpos, int m, int k, double delta, int* cnt, const int* c_rp,
                       int* c_ci, double* c_v, double* g11, int num_sms, cudaStream_t st);
// Deterministic transpose of C (m rows, k columns): per-block counts, scan, fill.
int ct_rows_per_block();
cudaError_t ct_count(const int* c_rp, const int* c_ci, int m, int k, int* blk_cnt, cudaStream_t st);
cudaError_t ct_fill(const int* c_rp, const int* c_ci, const double* c_v, int m, int k, const int* blk_off,
                    int* ct_ci, double* ct_v, cudaStream_t st);
cudaError_t ct_row_ptr(const int* blk_off, int k, int nblk, const int* total_dev, int* ct_rp, cudaStream_t st);
// Copy values to FP32.
cudaError_t vals_to_f32(const double* a, float* out, int64_t n, cudaStream_t st);
// D_S^-1 for non-pivot rows (1/diag when k == 0); 0 for pivot rows.
cudaError_t schur_diag(const int* c_rp, const int* c_ci, const double* c_v, const double* W, const double* diag,
                       const int* pivpos, int m, int k, double floor_rel, double* dsinv, float* dsinv32,
                       cudaStream_t st);

// ---- dense pivot block (dense.cu): W = G11^-1 through Cholesky; returns the
// number of regularised pivots in *regularised (device int).
size_t dense_work_elems(int k);
cudaError_t dense_spd_inverse(double* g11, double* W, double* work, int k, int* regularised, cudaStream_t st);

// ---- explicit A diag(w) A^T (adat.cu)
// Rows of A D A^T with more contributions than the per-warp shared-memory
// sort holds: kmax - i + 1 per heavy row, then the count (out_ci == null) or
// fill pass over dense accumulator slots (acc, stamp: slots x R; bits:
// slots x ceil(R / 32) words, zero; stamp all -1 before the first use).
cudaError_t adat_heavy_range(const int* heavy, int nh, const int* rp, const int* ci, const int* cp, const int* ri,
                             int* range, cudaStream_t st);
cudaError_t adat_heavy(const int* heavy, int nh, const int* rp, const int* ci, const double* av, const int* cp,
                       const int* ri, const double* avT, const double* wv, double* acc, int* stamp, unsigned* bits,
                       size_t R, int slots, int* hcnt, const int* out_rp, int* out_ci, double* out_v, cudaStream_t st);
cudaError_t adat_count(const int* rp, const int* ci, const int* cp, const int* ri, int m, int* cnt,
                       cudaStream_t st);
cudaError_t adat_fill(const int* rp, const int* ci, const double* av, const int* cp, const int* ri,
                      const double* avT, const double* wv, int m, const int* out_rp, int* out_ci, double* out_v,
                      cudaStream_t st);

}  // namespace help
