/*
 * oracle.h -- CPU restatement of the reference's normal-equations PCG path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is compared
 * against and the timed CPU baseline in bench.py; nothing in help_gb300/
 * links, loads or calls it.  Each function cites the reference file:line it
 * restates (Tian-Xie/HELP).  The operation order of every floating-point
 * loop follows the reference (with its MKL calls given their plain BLAS
 * meaning), so on the same inputs the restatement reproduces the reference
 * built from its own sources bit for bit (pinned in tests/test_oracle_pin.py).
 *
 * Matrices are zero-based CSR: row_ptr[m+1], col_ind[nnz], val[nnz].
 */
#ifndef HELP_ORACLE_H
#define HELP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* y = beta*y + alpha*A*x over rows [beg[i], end[i]) -- Helper.cpp:57-68 (CSRMV_N) */
void oracle_csrmv_n(int m, int n, double alpha, const double* val, const int* col, const int* beg,
                    const int* end, const double* x, double beta, double* y);
/* y = beta*y + alpha*A^T*x as a scatter over rows -- Helper.cpp:71-81 (CSRMV_T) */
void oracle_csrmv_t(int m, int n, double alpha, const double* val, const int* col, const int* beg,
                    const int* end, const double* x, double beta, double* y);

/* Symbolic upper triangle of A A^T in the reference's discovery order
 * (Helper.cpp:215-271): pass row_ptr_out[m+1]; col_out may be NULL to count.
 * Returns nnz of the triangle. */
int64_t oracle_adat_symbolic(int m, int n, const int* row_ptr, const int* col_ind, const int* col_ptr,
                             const int* row_ind, int* row_ptr_out, int* col_out);
/* Numeric A diag(d) A^T on that pattern (Helper.cpp:331-348). */
void oracle_adat_numeric(int m, int n, const int* row_ptr, const int* col_ind, const double* val,
                         const int* col_ptr, const int* row_ind, const double* valT, const double* d,
                         const int* pat_ptr, const int* pat_col, double* out);
/* The same with `threads` POSIX threads (the reference's OpenMP row loop);
 * returns the threads used, -1 on allocation failure. */
int oracle_adat_numeric_threads(int m, int n, const int* row_ptr, const int* col_ind, const double* val,
                                const int* col_ptr, const int* row_ind, const double* valT, const double* d,
                                const int* pat_ptr, const int* pat_col, double* out, int threads);

/* Pivot rules for the partial Cholesky. */
enum {
    ORACLE_PIVOT_GREEDY = 0, /* reference: argmax of the Schur-updated diagonal (PCG.cpp:54-59) */
    ORACLE_PIVOT_GIVEN = 1   /* pivots given in order (the GPU library's top-k set)            */
};

typedef struct oracle_pchol {
    int m, k;
    int* perm;      /* m: permuted position -> original row (PCG_PERM)           */
    double* L;      /* m*k row-major by ORIGINAL row: PARTIAL_CHOL_L[row][c]      */
    double* D;      /* k: PARTIAL_CHOL_D                                          */
    double* diag_s; /* m by ORIGINAL row: DIAG_S after the k downdates            */
    double* l11inv; /* k*k: L11^-1 (unit lower), PCG.cpp:119-133                  */
    int* beg;       /* m: permuted row starts of A (csrRowPtrA_BEG, PCG.cpp:106)  */
    int* end;       /* m                                                          */
} oracle_pchol;

/* RenewPartialCholesky -- PCG.cpp:38-177, with the pivot count k a parameter
 * (the reference fixes k = PART_CHOL_COLS = 10, PCG.h:20).  `given` holds k
 * pivot rows for ORACLE_PIVOT_GIVEN.  Returns 0 on success. */
int oracle_pchol_build(int m, int n, const int* row_ptr, const int* col_ind, const double* val,
                       const double* d, double gamma, double delta, int k, int rule, const int* given,
                       oracle_pchol* out);
void oracle_pchol_free(oracle_pchol* pc);

/* M^-1 r in the permuted row order -- PCG.cpp:183-196 */
void oracle_precond_apply(const oracle_pchol* pc, const double* r, double* out);

/* Preconditioned CG on (A (D + gamma I)^-1 A^T + delta I) x = b -- PCG.cpp:296-395.
 * Stops when ||r|| < tol*||r0|| (reference: tol = PREC_THRESHOLD = 1e-20,
 * PCG.h:19) or after max_iter iterations (the reference has no cap).
 * Returns the number of iterations, negative on error. */
int64_t oracle_pcg(int m, int n, const int* row_ptr, const int* col_ind, const double* val,
                   const double* d, double gamma, double delta, const double* b, double* x, int k,
                   int rule, const int* given, double tol, int64_t max_iter);

/* Normal-equations backend with the reference boundary's semantics
 * (UsePCG_CPU.cpp:26-183); usable as help_ne_backend callbacks. */
typedef struct oracle_ne oracle_ne;
oracle_ne* oracle_ne_create(int k, int rule, double tol, int64_t max_iter);
int oracle_ne_construct(void* ctx, int32_t m, int32_t n, const int32_t* col_ptr, const int32_t* row_ind,
                        const double* val);
int oracle_ne_renew(void* ctx, const double* d);
int oracle_ne_solve(void* ctx, const double* d, const double* b_1, const double* b_2, double* x_1,
                    double* x_2);
int oracle_ne_destruct(void* ctx);
void oracle_ne_free(oracle_ne* ne);
int64_t oracle_ne_last_iters(const oracle_ne* ne);
int64_t oracle_ne_total_iters(const oracle_ne* ne);

/* The GPU library's pivot rule restated: the k rows with the largest
 * diagonal of A (D + gamma I)^-1 A^T + delta I, ties to the lower row index,
 * returned in increasing row order.  Returns the number chosen (min(k, m)). */
int oracle_topk_pivots(int m, const double* diag, int k, int* pivots);
/* diag(A (D + gamma I)^-1 A^T) + delta  (PCG.cpp:41-46) */
void oracle_diag_adat(int m, const int* row_ptr, const int* col_ind, const double* val, const double* d,
                      double gamma, double delta, double* diag);

#ifdef __cplusplus
}
#endif
#endif
