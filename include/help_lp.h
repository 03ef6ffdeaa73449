/*
 * help_lp.h -- host-side C ABI of libhelp_lp.so: seeded LP instance generators,
 * the MPS writer that feeds the same instances to the reference program, and
 * the homogeneous self-dual (HSD) interior-point driver that calls a
 * normal-equations backend through the four entry points the reference's
 * HSDSolver.cpp calls (LP.h:157-160).
 *
 * Everything here is plain C: int32 indices, double values, caller-visible
 * arrays allocated with malloc and released by help_lp_free().
 */
#ifndef HELP_LP_H
#define HELP_LP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Instance families (the five benchmark configurations map onto these). */
enum {
    HELP_LP_RANDOM = 0,   /* k nonzeros per column at uniform-random distinct rows   */
    HELP_LP_ZIPF = 1,     /* k nonzeros per column, rows from a Zipf rank law        */
    HELP_LP_MCF = 2,      /* multicommodity flow on a 4-neighbour grid graph         */
    HELP_LP_BLOCK = 3     /* block-angular: diagonal random blocks + linking rows    */
};

typedef struct help_lp_spec {
    int32_t kind;
    int32_t m, n, nnz_per_col;      /* RANDOM / ZIPF                                */
    double zipf_s;                  /* ZIPF: exponent of the rank law               */
    int32_t zipf_offset;            /* ZIPF: rank offset that flattens the head     */
    int32_t grid, commodities;      /* MCF: grid side, number of commodities        */
    int32_t pairs_per_commodity;    /* MCF: source/sink pairs routed per commodity  */
    int32_t blocks, block_rows, block_cols, link_rows;  /* BLOCK                    */
    double link_prob;               /* BLOCK: P(column appears in a linking row)    */
    int32_t mcf_ungrounded;         /* MCF: keep every node row (rank K short); 0
                                       grounds node 0 of each commodity            */
} help_lp_spec;

/*
 * A standard-form LP  min c^T x  s.t.  A x = b, x >= 0, stored column-major
 * (CSC, row indices sorted inside each column).  All values lie on a 1e-6
 * decimal grid so the MPS text written by help_lp_write_mps() parses back to
 * bit-identical doubles.  Inequality rows (MCF capacity rows) are already
 * closed with slack columns appended after the structural columns, in row
 * order, exactly as the reference's bound/row standardisation does
 * (Crushing.cpp:71-99); n_struct counts the columns before the slacks and
 * row_type[i] is 'E' or 'L' for the MPS writer.
 */
typedef struct help_lp {
    int32_t m, n, n_struct;
    int64_t nnz;
    int32_t* col_ptr;   /* n + 1   */
    int32_t* row_ind;   /* nnz     */
    double* val;        /* nnz     */
    double* b;          /* m       */
    double* c;          /* n       */
    char* row_type;     /* m       */
} help_lp;

/* Returns 0 on success, a negative code on bad parameters or allocation failure. */
int help_lp_generate(const help_lp_spec* spec, uint64_t seed, help_lp* out);
void help_lp_free(help_lp* lp);

/* Writes the instance (structural columns only, inequality rows as 'L') in
 * the fixed-column MPS layout the reference parser reads (MPSRead.cpp:18,
 * card positions 4/14/24).  Returns 0 on success. */
int help_lp_write_mps(const help_lp* lp, const char* path);

/* Reads an MPS file (fixed or free layout: fields separated by blanks, names
 * without blanks) into the standard form above, as the reference's MPSRead
 * (MPSRead.cpp:76-219) and row standardisation (Crushing.cpp:71-99) do for
 * the problems the HSD driver takes: rows N (the first is the objective,
 * minimised), E, L, G; L and G rows get a slack column (+1 / -1) appended
 * after the structural columns in row order; entries of unknown rows and
 * entries below 1e-8 in magnitude are dropped (MPSRead.cpp:148-163); rows are
 * sorted inside each column and a repeated (row, column) entry is an error.
 * RANGES and every bound other than x >= 0 (LO 0, PL) are rejected, as are
 * integer markers.  Returns 0, -1 bad arguments, -2 I/O error or out of
 * memory, -3 format error (help_lp_last_error() tells which line and why). */
int help_lp_read_mps(const char* path, help_lp* out);

/* Binary fast path for large instances (no text parsing): a 64-byte header
 * ("HELPLP01", m, n, n_struct, nnz as int64) followed by col_ptr (int32,
 * n+1), row_ind (int32, nnz), val (f64, nnz), b (f64, m), c (f64, n),
 * row_type (m bytes), little-endian.  Return codes as help_lp_read_mps. */
int help_lp_write_bin(const help_lp* lp, const char* path);
int help_lp_read_bin(const char* path, help_lp* out);

/* Linear-dependency presolve (the purpose of the reference's
 * Presolve_Lindep.cpp:316, off there by default, LP.h:72): *out gets in
 * without the rows that are linear combinations of the other rows, after
 * checking that b agrees to 1e-8 sqrt(1 + |b|_2^2).  A triangular crash
 * peels the rows that have a column of their own; the rows it defers are
 * reduced against the peeled ones and eliminated (Markowitz order, threshold
 * pivoting, a dense finish for the last <= 4096 rows).  A row is dependent
 * when none of its entries is left above tol x its largest entry (the
 * reference's TOLAPIV is 1e-8).  removed (m flags, may be NULL) marks the
 * dropped rows.  Returns the number of rows dropped, -1 bad arguments, -2 out
 * of memory, -3 b disagrees (the LP is primal infeasible), -4 the presolve
 * does not apply: the elimination fills in past its limits (4 x nnz + 16 m
 * entries or 64 x nnz + 2^28 entry updates with more than 4096 rows left;
 * random sparse A at 10^4 rows and more), *out left empty. */
int help_lp_remove_dependent_rows(const help_lp* in, double tol, help_lp* out, int32_t* removed);

/* Message of the last failed read on this thread ("" if none). */
const char* help_lp_last_error(void);

/* Row-major copy (CSR, column indices sorted inside each row) of a CSC matrix. */
int help_csc_to_csr(int32_t m, int32_t n, const int32_t* col_ptr, const int32_t* row_ind,
                    const double* val, int32_t* row_ptr, int32_t* col_ind, double* val_out);

/* ------------------------------------------------------------------------ */
/* HSD interior-point driver                                                 */
/* ------------------------------------------------------------------------ */

/*
 * The four normal-equations entry points, as function pointers, so one
 * driver binary can run against any backend (the GPU library, or the CPU
 * restatement used as the measured baseline).  Semantics follow the
 * reference boundary (LP.h:157-160, UsePCG_CPU.cpp:26-183):
 *   construct(ctx, m, n, csc...)  -- LinearEquation_Construct
 *   renew(ctx, d)                 -- RenewLinearEquation, d = X^-1 Z (not inverted)
 *   solve(ctx, d, b1, b2, x1, x2) -- SolveLinearEquation for
 *                                    [D A^T; A 0][x1; x2] = [b1; b2]
 *   destruct(ctx)                 -- LinearEquation_Destruct
 * Each returns 0 on success.
 */
typedef struct help_ne_backend {
    void* ctx;
    int (*construct)(void* ctx, int32_t m, int32_t n, const int32_t* col_ptr,
                     const int32_t* row_ind, const double* val);
    int (*renew)(void* ctx, const double* d);
    int (*solve)(void* ctx, const double* d, const double* b_1, const double* b_2,
                 double* x_1, double* x_2);
    int (*destruct)(void* ctx);
    /* Optional (may be NULL): dest += sign * A v (transpose 0) or
     * dest += sign * A^T v (transpose 1) with the backend's copy of A -- the
     * driver's own products (ATimes, Helper.cpp:110-152) done where A
     * already lives.  NULL: the driver's host loops (the reference's order). */
    int (*matvec)(void* ctx, int32_t transpose, int32_t sign, const double* v, double* dest);
    /* Optional (may be NULL): two solves with the matrix of the last renew,
     * (b_1a, b_2a) -> (x_1a, x_2a) and (b_1b, b_2b) -> (x_1b, x_2b), each giving
     * what solve gives for it, run at the same time where the backend can.
     * The driver then solves the bottom system (LinearEquationBottom,
     * HSDSolver.cpp:226-261) and the first direction of an iteration
     * (SearchDirection, :281-473) together: neither right-hand side depends on
     * the other's solution.  NULL: one solve after the other, as the reference. */
    int (*solve2)(void* ctx, const double* d, const double* b_1a, const double* b_2a, double* x_1a,
                  double* x_2a, const double* b_1b, const double* b_2b, double* x_1b, double* x_2b);
} help_ne_backend;

typedef struct help_hsd_options {
    int32_t max_iterations;     /* reference: Max_Iterations = 10000 (LP.h:86)   */
    double gap_tol;             /* reference: 1e-8 (LP.h:89)                     */
    double pinf_tol, dinf_tol;  /* reference: 1e-8 (LP.h:90-91)                  */
    int32_t verbose;            /* print the reference's per-iteration table     */
    /* Optional per-iteration callback (iteration, primal obj, dual obj, rel gap,
     * primal infeasibility, dual infeasibility); may be NULL. */
    void (*on_iter)(void* user, int32_t iter, const double* stats6);
    void* user;
    /* Remove the dependent rows first (help_lp_remove_dependent_rows, tol
     * 1e-8), as the reference does when PRESOLVE_LINDEP is set (LP.h:72, 0
     * there; Presolve.cpp:1254-1260): the backend then sees the reduced
     * matrix, y_out still has m entries (0 on the dropped rows).  Where the
     * presolve does not apply (its -4) the LP is solved as it is. */
    int32_t presolve_lindep;
    /* Wall-clock cap in seconds (0: none; the reference has none): checked
     * before each iteration's renew; when it has run out the driver stops
     * with status 2, as at the iteration limit. */
    double max_seconds;
} help_hsd_options;

typedef struct help_hsd_result {
    int32_t status;             /* 0 OK, 1 stalled, 2 iteration limit, 3 unknown (LP.h:163-167) */
    int32_t iterations;         /* rows of the reference table printed (Iter + 1 at exit) */
    int32_t solves;             /* normal-equation solves issued                 */
    int32_t renews;
    double primal_obj, dual_obj, rel_gap, primal_infeas, dual_infeas;
    double tau, kappa;
    double wall_s, backend_s;   /* total and time spent inside backend calls     */
    int32_t lp_status;          /* 0 OK, 1 primal infeasible found by the presolve
                                   (the reference's LP_Status, LP.h:77-80; no
                                   HSD iteration is run then)                   */
    int32_t rows_removed;       /* dependent rows the presolve dropped           */
} help_hsd_result;

void help_hsd_default_options(help_hsd_options* opt);

/* Runs the HSD method (the reference's HSD_Main, HSDSolver.cpp:869-883) on an
 * all-lower-bounded standard-form LP.  x_out (n) / y_out (m) may be NULL.
 * Returns 0, -1 bad arguments, the backend's construct code when that
 * fails, -2 when a later backend call failed, -3 host out of memory (the
 * backend may then still hold its construct). */
int help_hsd_solve(const help_lp* lp, const help_ne_backend* be, const help_hsd_options* opt,
                   help_hsd_result* res, double* x_out, double* y_out);

#ifdef __cplusplus
}
#endif
#endif
