/*
 * help_gpu.h -- C ABI of libhelp_gpu.so, the GB300 normal-equations backend.
 *
 * The reference (Tian-Xie/HELP) selects its normal-equations backend at link
 * time through four C++ functions declared in LP.h:157-160 and implemented
 * for the PCG backend in UsePCG_CPU.cpp:26-183 + PCG.cpp:38-395.  This
 * library provides the same four operations as plain C entry points (no
 * globals, no torch types: plain pointers, sizes and an opaque context) so a
 * C++ shim (help_gb300/csrc/UsePCG_GPU.cpp) can re-export them under the
 * reference's own names, and any FFI can bind them directly.
 *
 * Boundary contract (same as the reference's):
 *   - all vectors passed to construct/renew/solve are HOST arrays owned by the
 *     caller; the library keeps its own device copies of A and all scratch;
 *   - d is D = X^-1 Z itself (not inverted);
 *   - solve writes x_1 (n) and x_2 (m) in full;
 *   - single-threaded caller, no re-entrancy on one context: calls on one
 *     context must not overlap on the GPU either (help_pcg_matvec_dev on
 *     two streams), as they share its scratch (long-row partial sums).
 * Every entry point returns HELP_OK (0) or a negative HELP_E* code; the
 * reference's backends exit() on fatal errors instead (Helper.cpp:24-35), the
 * UsePCG_GPU.cpp shim keeps that behaviour.
 */
#ifndef HELP_GPU_H
#define HELP_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    HELP_OK = 0,
    HELP_E_ARG = -1,         /* bad argument or call order                        */
    HELP_E_CUDA = -2,        /* CUDA runtime error (message via help_pcg_last_error) */
    HELP_E_NOMEM = -3,       /* device or host allocation failed                  */
    HELP_E_NUMERIC = -4,     /* non-positive / non-finite d, breakdown, NaN        */
    HELP_E_TIMEOUT = -5,     /* a device-side wait ran past its limit              */
    HELP_E_NOT_CONVERGED = -6 /* the solve's last CG run stopped at its iteration cap
                                 without meeting cg_tol (x_1, x_2 are still written);
                                 HELP_OK instead when options.cap_ok is set          */
};

enum {
    HELP_PREC_FP64 = 0,      /* plain FP64 PCG: the drop-in form                      */
    HELP_PREC_MIXED = 1      /* FP32 CG inside FP64 iterative refinement              */
};

typedef struct help_pcg help_pcg;  /* opaque: one matrix resident on one GPU */

typedef struct help_pcg_options {
    int32_t device;          /* CUDA device ordinal                                     */
    int32_t pivots;          /* k, partial-Cholesky pivot count (reference: 10, PCG.h:20) */
    int32_t precision;       /* HELP_PREC_FP64 or HELP_PREC_MIXED                        */
    double cg_tol;           /* stop when ||r|| < cg_tol*||r0|| (reference 1e-20, PCG.h:19) */
    int64_t cg_max_iter;     /* iteration cap per CG run (the reference has none)         */
    double delta;            /* regularisation: solves (A D^-1 A^T + delta I) (ref: 0)   */
    /* mixed precision */
    double ir_tol;           /* FP64 normal-equation residual target ||r||/||rhs||      */
    int32_t ir_max_outer;    /* refinement steps before falling back to FP64 PCG        */
    double inner_tol;        /* relative residual reduction asked of each FP32 CG run   */
    int64_t inner_max_iter;  /* cap per FP32 CG run                                     */
    /* warm start and fallback (the learned correction is attached separately,
       help_pcg_attach_mlp, and brings its own warm start) */
    int32_t warm_start;      /* 1: start CG from the previous solve's x_2 of this renew */
    int32_t fallback;        /* mixed form only -- 1: when FP32 refinement stalls or hits
                                its cap, finish with plain FP64 PCG; 0: stop there        */
    int32_t cg_path;         /* 0 auto: the shared-memory-resident cluster kernel when
                                the vectors fit one cluster's shared memory (<= 64
                                pivots, rows of <= 32 G nonzeros), else one thread-block
                                cluster over L2 when the system is small, else the
                                multi-kernel graph; 1 always the graph; 2 the cluster
                                kernel over L2; 3 the resident kernel where it fits
                                (else as 0)                                              */
    int32_t cap_ok;          /* 0 (default): a solve whose last CG run stopped at its
                                iteration cap returns HELP_E_NOT_CONVERGED; 1: it returns
                                HELP_OK and stats.converged = 0 (for callers that treat
                                an inexact Newton direction as usable)                   */
    double mixed_max_d_spread; /* mixed form: FP32 refinement only while max(d)/min(d) of
                                the renew is at most this (default 1e8) and the CG runs
                                on the bandwidth-bound graph path; otherwise plain FP64
                                PCG to ir_tol, chosen before any FP32 work              */
} help_pcg_options;

typedef struct help_pcg_stats {
    int64_t cg_iterations;       /* last solve: all CG iterations (inner + fallback)  */
    int64_t cg_iterations_total; /* since construct                                   */
    int32_t ir_outer;            /* last solve: refinement steps (mixed)              */
    int32_t fell_back;           /* last solve: 1 if plain FP64 PCG had to finish it   */
    int32_t converged;           /* last solve: stopping rule met                      */
    int32_t pivots;              /* k actually used                                    */
    double rel_residual;         /* last solve: FP64 ||rhs - G x_2|| / ||rhs||         */
    double renew_ms, solve_ms;   /* last renew / solve wall time                       */
    int64_t nnz_c;               /* entries of the pivot-column block G[:,P] (non-pivot rows) */
    int32_t solves, renews;
    /* device time of the CG graph launches (CUDA events on the launching stream) */
    double cg_kernel_ms;         /* last solve, all CG launches                        */
    double cg_kernel_ms_total;   /* since construct                                    */
    int64_t cg_iterations_fp32;  /* last solve: iterations run in FP32 (mixed)          */
    int32_t cg_launches;         /* last solve                                          */
    int32_t dense_regularised;   /* last renew: pivots raised to the floor in G11       */
    int32_t cg_path_used;        /* last CG run: 1 multi-kernel graph, 2 single cluster,
                                    3 single cluster with shared-memory-resident vectors */
    int32_t cluster_ctas;        /* CTAs per cluster of the single-cluster path (0 = unavailable) */
    int32_t learned_warm;        /* last solve: started from the model's warm start     */
    int32_t learned_fallbacks;   /* since construct: model-assisted solves redone plain */
    int32_t fp32_chosen;         /* last solve (mixed): 1 FP32 refinement ran, 0 FP64 up front */
    double d_spread;             /* last renew: max(d) / min(d)                         */
} help_pcg_stats;

/* Fills *opt with the defaults (FP64, k = 10, cg_tol = 1e-20 as the reference). */
void help_pcg_default_options(help_pcg_options* opt);

/* Creates a context bound to opt->device; no matrix yet. */
int help_pcg_create(const help_pcg_options* opt, help_pcg** out);
/* Frees the context (calls help_pcg_destruct if needed). */
void help_pcg_free(help_pcg* ctx);

/* LinearEquation_Construct (UsePCG_CPU.cpp:26-68): A (m x n) given column-wise
 * (CSC, zero-based, rows sorted inside columns).  Uploads A once as both
 * CSC and CSR and plans the SpMV work partition. */
int help_pcg_construct(help_pcg* ctx, int32_t m, int32_t n, const int32_t* col_ptr,
                       const int32_t* row_ind, const double* val);

/* RenewLinearEquation (UsePCG_CPU.cpp:78-80; the reference rebuilds its
 * preconditioner inside every solve instead, PCG.cpp:301 -> :38-177):
 * uploads d, forms B = A D^-1/2, picks the k pivots, builds G[:,P], factors
 * the pivot block and the Schur diagonal.  Call once per interior-point
 * iteration, before the solves that use this d. */
int help_pcg_renew(help_pcg* ctx, const double* d);

/* SolveLinearEquation (UsePCG_CPU.cpp:91-183):
 *   [D A^T; A 0] [x_1; x_2] = [b_1; b_2]
 *   (A D^-1 A^T) x_2 = A D^-1 b_1 - b_2,   x_1 = D^-1 (b_1 - A^T x_2)
 * d must be the array last passed to help_pcg_renew (renews if it is not). */
int help_pcg_solve(help_pcg* ctx, const double* d, const double* b_1, const double* b_2,
                   double* x_1, double* x_2);

/* LinearEquation_Destruct (UsePCG_CPU.cpp:70-75): releases the device matrix. */
int help_pcg_destruct(help_pcg* ctx);

int help_pcg_get_stats(const help_pcg* ctx, help_pcg_stats* out);
const char* help_pcg_last_error(const help_pcg* ctx);

/* ---- building blocks of the path, exposed for parity tests and the isolated
 * ADA^T v benchmark.  Host arrays unless the name ends in _dev. ---- */

enum { HELP_OP_A = 0, HELP_OP_AT = 1, HELP_OP_ADAT = 2, HELP_OP_B = 3, HELP_OP_BT = 4 };

/* y = A x (CSRMV_N, Helper.cpp:57-68), y = A^T x (CSRMV_T, Helper.cpp:71-81)
 * or y = (A D^-1 A^T + delta I) x (PCG.cpp:346-358), D from the last renew.
 * HELP_OP_B / HELP_OP_BT are the two passes of the last one, with
 * B = A D^-1/2: y = B x (x has n entries) and y = B^T x (x has m entries). */
int help_pcg_matvec(help_pcg* ctx, int32_t op, const double* x, double* y);
/* Same on device pointers, on `stream` (a cudaStream_t, NULL = default);
 * fp32 != 0 runs the FP32 copy of B (x, y are then float*). */
int help_pcg_matvec_dev(help_pcg* ctx, int32_t op, int32_t fp32, const void* x, void* y,
                        void* stream);
/* dest += sign * A v (transpose 0: v has n entries, dest m) or
 * dest += sign * A^T v (transpose 1: v has m entries, dest n), sign = +1 or
 * -1, host arrays, with the device copy of A -- the HSD iteration's own
 * products (ATimes, Helper.cpp:110-152, called at HSDSolver.cpp:97, :108
 * and from the direction computation), offered to the driver as the
 * optional matvec of its backend table.  Each row's products are summed on
 * the device and added to dest once. */
int help_pcg_matvec_acc(help_pcg* ctx, int32_t transpose, int32_t sign, const double* v, double* dest);

/* The learned part's solve slots (the i-th solve after a renew takes slot
 * min(i, 3); each slot's solution seeds the same slot's warm start and
 * features at the next renew): slots[i] is the slot of solve i for i < n
 * (n <= 4, slots in [0, 4)), the default beyond.  The paired backend
 * maps context 0's solves to slots {0, 2} and context 1's to {1}, the slots
 * those systems take on one context. */
int help_pcg_set_solve_slots(help_pcg* ctx, const int32_t* slots, int32_t n);
/* dst's solution of dst_slot in the current renew := src's of src_slot (both
 * constructed with the same matrix on the same device; nothing without an
 * attached model).  The paired backend gives context 1 context 0's solution
 * of the bottom system (slot 0) before each renew, whose features -- and so
 * the Schur-diagonal correction -- it reads. */
int help_pcg_share_solution(help_pcg* dst, int32_t dst_slot, help_pcg* src, int32_t src_slot);

/* Two contexts on one GPU for the HSD driver's paired solves (help_lp.h,
 * help_ne_backend.solve2).  Each IPM iteration solves the bottom system
 * (LinearEquationBottom, HSDSolver.cpp:226-261) and the first search
 * direction (:281-473) with the same matrix, and neither right-hand side
 * depends on the other's solution: the pair gives each to its own context,
 * on its own host thread and stream, so the two CG runs overlap on the GPU
 * (two single-cluster runs on small systems).  Both contexts are built and
 * renewed from the same arguments; each solve gives what help_pcg_solve on
 * one context gives (the option warm_start is refused; an attached model is
 * followed through help_pcg_set_solve_slots and help_pcg_share_solution).
 * The backend-table entries take the pair as their ctx. */
typedef struct help_pcg_pair help_pcg_pair;
int help_pcg_pair_create(const help_pcg_options* opt, help_pcg_pair** out);
void help_pcg_pair_free(help_pcg_pair* pair);
/* Context 0 or 1 of the pair (stats, products); NULL for any other index. */
help_pcg* help_pcg_pair_context(help_pcg_pair* pair, int32_t which);
int help_pcg_pair_construct(void* pair, int32_t m, int32_t n, const int32_t* col_ptr, const int32_t* row_ind,
                            const double* val);
int help_pcg_pair_renew(void* pair, const double* d);
/* One solve, on context 0. */
int help_pcg_pair_solve(void* pair, const double* d, const double* b_1, const double* b_2, double* x_1,
                        double* x_2);
/* (b_1a, b_2a) on context 0 and (b_1b, b_2b) on context 1, at the same time;
 * the first error code of the two (context 0's first). */
int help_pcg_pair_solve2(void* pair, const double* d, const double* b_1a, const double* b_2a, double* x_1a,
                         double* x_2a, const double* b_1b, const double* b_2b, double* x_1b, double* x_2b);
int help_pcg_pair_destruct(void* pair);
/* help_pcg_matvec_acc on context 0. */
int help_pcg_pair_matvec(void* pair, int32_t transpose, int32_t sign, const double* v, double* dest);
/* z = M^-1 r with the last renew's partial-Cholesky preconditioner
 * (Preconditioner, PCG.cpp:183-196), vectors in the original row order. */
int help_pcg_precond_apply(help_pcg* ctx, const double* r, double* z);
/* Pivot rows (ascending, k of them), diag(A D^-1 A^T) and the Schur diagonal
 * D_S used for non-pivot rows (PCG.cpp:41-46, :100-102). Any pointer may be NULL. */
int help_pcg_get_pivots(help_pcg* ctx, int32_t* pivots, double* diag_g, double* diag_s);
/* One PCG run on (A D^-1 A^T + delta I) x = b from x = 0 with the current
 * preconditioner (ConjugateGradient, PCG.cpp:296-395); returns iterations in
 * *iters; stats cg_iterations / cg_kernel_ms / cg_launches describe this run. */
int help_pcg_cg(help_pcg* ctx, const double* b, double* x, int64_t* iters);
/* The same run in FP32 (vectors and matrices in FP32, dot products and the
 * pivot block in FP64) on a context created with HELP_PREC_MIXED: the inner
 * solver of the mixed form, alone. */
int help_pcg_cg_f32(help_pcg* ctx, const double* b, double* x, int64_t* iters);

/* Explicit A diag(w) A^T, upper triangle incl. diagonal, CSR with columns
 * sorted in each row (ADAt_Allocate + ADAt_Calc, Helper.cpp:215-377; the
 * reference keeps discovery order inside a row).  Two-call protocol: with
 * col == NULL only *nnz is returned; then pass arrays of that size. */
int help_adat_assemble(help_pcg* ctx, const double* w, int32_t* row_ptr, int32_t* col, double* val,
                       int64_t* nnz);

/* ---- learned part (no counterpart in the reference) ----
 *
 * A 16 -> 64 -> 64 -> 2 MLP (ReLU, BF16 weights and activations, FP32
 * accumulation on the tensor cores) reads per-row features of the normal
 * equations after each renew and gives, per row, (0) the log-factor of a
 * correction of the preconditioner's Schur diagonal D_S (clamped to +-2) and
 * (1) a scale of the warm start: solve s of a renew starts from
 * alpha * (out[:,1] .* x_2 of solve s of the previous renew), alpha the
 * G-norm-optimal scalar.  The plain partial-Cholesky PCG is its fallback: a
 * solve that hits the iteration cap or whose FP64 residual check fails is
 * redone cold with the uncorrected preconditioner.
 *
 * Features (row i of A, d = D):  0 log10 diag(A D^-1 A^T)_ii,  1-4 mean /
 * std / min / max of log10 d_j over the row,  5 log2(1 + row length),
 * 6 log10(D_S,i / diag_i) (0 on pivot rows),  7 pivot flag,  8 x_2 of the
 * same solve slot in the previous renew over its RMS,  9 / 10 mean /
 * largest |change| of log10 d_j over the row since the previous renew;
 * 11-15 zero.  Solve slot s > 0 runs the model on its own features.  Each is normalised
 * as (f - mean) * scale with the model's constants, then rounded to BF16.
 *
 * Parameters (FP32, HELP_MLP_PARAMS floats): W1[64][16], b1[64], W2[64][64],
 * b2[64], W3[2][64], b3[2] (row-major, out x in), then the normalisation
 * mean[16], scale[16].  Training minimises sum w (out - target)^2 / sum w
 * over rows x 2 entries with Adam (0.9, 0.999, 1e-8) on the trainable part. */
#define HELP_MLP_IN 16
#define HELP_MLP_HIDDEN 64
#define HELP_MLP_OUT 2
#define HELP_MLP_OFF_W1 0
#define HELP_MLP_OFF_B1 1024
#define HELP_MLP_OFF_W2 1088
#define HELP_MLP_OFF_B2 5184
#define HELP_MLP_OFF_W3 5248
#define HELP_MLP_OFF_B3 5376
#define HELP_MLP_OFF_MEAN 5378
#define HELP_MLP_OFF_SCALE 5394
#define HELP_MLP_PARAMS 5410

typedef struct help_mlp help_mlp;
int help_mlp_create(int32_t device, help_mlp** out);
int help_mlp_free(help_mlp* mlp);
const char* help_mlp_last_error(const help_mlp* mlp);
/* host arrays of HELP_MLP_PARAMS floats; set also resets the Adam state */
int help_mlp_set_params(help_mlp* mlp, const float* params);
int help_mlp_get_params(help_mlp* mlp, float* params);
/* device arrays: x BF16 [rows][16], out FP32 [rows][2]; runs on `stream` */
int help_mlp_forward(help_mlp* mlp, const void* x, int64_t rows, float* out, void* stream);
/* device x, target, weight ([rows][2]); host loss and grad (HELP_MLP_OFF_MEAN floats) */
int help_mlp_loss_grad(help_mlp* mlp, const void* x, const float* target, const float* weight, int64_t rows,
                       double* loss, float* grad);
/* one Adam step with learning rate lr on that loss (loss before the step) */
int help_mlp_train_step(help_mlp* mlp, const void* x, const float* target, const float* weight, int64_t rows,
                        float lr, double* loss);
/* Use `mlp` in this context's solves from the next renew on (NULL: plain PCG).
 * The model must live on the context's device and outlive the attachment. */
int help_pcg_attach_mlp(help_pcg* ctx, help_mlp* mlp);
/* Raw (unnormalised) FP32 features of the current renew for solve slot
 * `slot` (0 .. 3, the order of the solves after a renew) into the device
 * array x [m][16]; the previous renew's solution of that slot and its d are
 * used when a model was attached during it. */
int help_pcg_features(help_pcg* ctx, int32_t slot, float* x);

/* ---- no-allocation product (no counterpart in the reference) ----
 *
 * y = A D^-1 A^T x for callers that cannot allocate device memory (code
 * running under another runtime's memory pool or an allocator that forbids
 * new allocations, paths that must not allocate after start-up, hosts that
 * only receive device pointers).  Everything is the caller's device memory --
 * A as CSR (row_ptr[m+1], col_ind[nnz], val[nnz]) and as CSC
 * (col_ptr[n+1], row_ind[nnz], val_t[nnz]), d[n], x[m], y[m] -- except the
 * intermediate D^-1 A^T x, which lives in a fixed device array of 2^20
 * doubles (8 MiB) that every GPU loading the library keeps until the process
 * exits.  No cudaMalloc, cudaFree or allocating library call is made.
 *   - n larger than 2^20 is rejected with HELP_E_ARG;
 *   - the CUDA runtime loads the library's device code on first use, so the
 *     first call on each device is the one that reserves the array (8 MiB of
 *     device memory taken then): make it at start-up, with that device
 *     current, before any stream capture and before the memory pool that
 *     forbids allocation is set up; later calls allocate nothing;
 *   - every call on a device shares the array, so calls that overlap on the
 *     GPU (other streams, other host threads) race: serialise them;
 *   - nothing has to start at zero: the first pass writes every entry of the
 *     array that the second pass reads, and y is written in full;
 *   - runs on `stream` (NULL = the legacy default stream) on the current device.
 */
int help_adat_matvec_noalloc(int32_t m, int32_t n, int64_t nnz, const int32_t* row_ptr,
                             const int32_t* col_ind, const double* val, const int32_t* col_ptr,
                             const int32_t* row_ind, const double* val_t, const double* d,
                             const double* x, double* y, void* stream);

#ifdef __cplusplus
}
#endif
#endif
