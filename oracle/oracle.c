/*
 * oracle.c -- CPU restatement of the reference's normal-equations PCG path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library and the timed CPU
 * baseline; the product library never links it.  Compiled with
 * -ffp-contract=off so every multiply-add rounds the way the reference's
 * plain loops do.  See oracle.h for the interface.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- SpMV */

/* Helper.cpp:57-68 */
void oracle_csrmv_n(int m, int n, double alpha, const double* val, const int* col, const int* beg,
                    const int* end, const double* x, double beta, double* y) {
    (void)n;
    for (int i = 0; i < m; i++) y[i] *= beta;
    for (int i = 0; i < m; i++) {
        double tmp = 0;
        for (int j = beg[i]; j < end[i]; j++) tmp += val[j] * x[col[j]];
        y[i] += tmp * alpha;
    }
}

/* Helper.cpp:71-81 */
void oracle_csrmv_t(int m, int n, double alpha, const double* val, const int* col, const int* beg,
                    const int* end, const double* x, double beta, double* y) {
    for (int i = 0; i < n; i++) y[i] *= beta;
    for (int i = 0; i < m; i++) {
        double tmp = alpha * x[i];
        for (int j = beg[i]; j < end[i]; j++) y[col[j]] += val[j] * tmp;
    }
}

/* Plain-BLAS meaning of the MKL sparse routine the reference calls
 * (mkl_dcsrmv, used at PCG.cpp:190-195 and UsePCG_CPU.cpp:112, :174). */
static void blas_csrmv(char trans, int rows, int cols, double alpha, const double* val, const int* ind,
                       const int* ptr, const double* x, double beta, double* y) {
    if (trans == 'N') {
        for (int i = 0; i < rows; i++) {
            double s = 0.0;
            for (int p = ptr[i]; p < ptr[i + 1]; p++) s += val[p] * x[ind[p]];
            y[i] = (beta == 0.0 ? 0.0 : beta * y[i]) + alpha * s;
        }
    } else {
        for (int j = 0; j < cols; j++) y[j] = (beta == 0.0 ? 0.0 : beta * y[j]);
        for (int i = 0; i < rows; i++) {
            const double a = alpha * x[i];
            for (int p = ptr[i]; p < ptr[i + 1]; p++) y[ind[p]] += val[p] * a;
        }
    }
}

static double blas_dot(int n, const double* x, const double* y) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += x[i] * y[i];
    return s;
}
static double blas_nrm2(int n, const double* x) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += x[i] * x[i];
    return sqrt(s);
}
static void blas_axpy(int n, double a, const double* x, double* y) {
    for (int i = 0; i < n; i++) y[i] += a * x[i];
}

/* ---------------------------------------------------------------- ADA^T */

/* For every CSR(A) entry, its position inside its column of CSC(A).  Rows are
 * sorted inside columns, so scanning rows in order fills each column in order. */
static int* csr_to_csc_link(int m, int n, const int* row_ptr, const int* col_ind, const int* col_ptr) {
    int* fill = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int* link = (int*)malloc(sizeof(int) * (size_t)(row_ptr[m] > 0 ? row_ptr[m] : 1));
    if (!fill || !link) {
        free(fill);
        free(link);
        return NULL;
    }
    for (int j = 0; j < n; j++) fill[j] = col_ptr[j];
    for (int i = 0; i < m; i++)
        for (int p = row_ptr[i]; p < row_ptr[i + 1]; p++) link[p] = fill[col_ind[p]]++;
    free(fill);
    return link;
}

/* Helper.cpp:215-271: row i collects every row k >= i sharing a column with
 * it, in the order met walking row i's columns and each column downward. */
int64_t oracle_adat_symbolic(int m, int n, const int* row_ptr, const int* col_ind, const int* col_ptr,
                             const int* row_ind, int* row_ptr_out, int* col_out) {
    int* link = csr_to_csc_link(m, n, row_ptr, col_ind, col_ptr);
    int* flag = (int*)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    if (!link || !flag) {
        free(link);
        free(flag);
        return -1;
    }
    for (int k = 0; k < m; k++) flag[k] = -1;
    int64_t nnz = 0;
    row_ptr_out[0] = 0;
    for (int i = 0; i < m; i++) {
        for (int p = row_ptr[i]; p < row_ptr[i + 1]; p++) {
            const int j = col_ind[p];
            for (int q = link[p]; q < col_ptr[j + 1]; q++) {
                const int k = row_ind[q];
                if (flag[k] != i) {
                    flag[k] = i;
                    if (col_out) col_out[nnz] = k;
                    nnz++;
                }
            }
        }
        row_ptr_out[i + 1] = (int)nnz;
    }
    free(link);
    free(flag);
    return nnz;
}

/* Helper.cpp:331-348 (and the CSR-linked variant :350-377, same order). */
/* One row of ADAt_Calc (Helper.cpp:350-377): the dense accumulator is zeroed
 * on the row's pattern, each row entry walks its column from the row down,
 * the pattern is read back. */
static void adat_numeric_row(int i, const int* row_ptr, const int* col_ind, const double* val, const int* col_ptr,
                             const int* row_ind, const double* valT, const double* d, const int* pat_ptr,
                             const int* pat_col, const int* link, double* acc, double* out) {
    for (int p = pat_ptr[i]; p < pat_ptr[i + 1]; p++) acc[pat_col[p]] = 0;
    for (int p = row_ptr[i]; p < row_ptr[i + 1]; p++) {
        const int j = col_ind[p];
        const double vd = val[p] * d[j];
        for (int q = link[p]; q < col_ptr[j + 1]; q++) acc[row_ind[q]] += vd * valT[q];
    }
    for (int p = pat_ptr[i]; p < pat_ptr[i + 1]; p++) out[p] = acc[pat_col[p]];
}

void oracle_adat_numeric(int m, int n, const int* row_ptr, const int* col_ind, const double* val,
                         const int* col_ptr, const int* row_ind, const double* valT, const double* d,
                         const int* pat_ptr, const int* pat_col, double* out) {
    oracle_adat_numeric_threads(m, n, row_ptr, col_ind, val, col_ptr, row_ind, valT, d, pat_ptr, pat_col, out, 1);
}

/* The reference runs ADAt_Calc's row loop under `omp parallel for` with one
 * dense accumulator per thread (Helper.cpp:210-211, :352-356); here POSIX
 * threads take chunks of 256 rows from a shared counter.  Rows are
 * independent, so the result is the same for every thread count. */
typedef struct {
    int m;
    const int *row_ptr, *col_ind, *col_ptr, *row_ind, *pat_ptr, *pat_col, *link;
    const double *val, *valT, *d;
    double* out;
    int next;
    int failed;
} adat_job;

static void* adat_worker(void* arg) {
    adat_job* J = (adat_job*)arg;
    double* acc = (double*)malloc(sizeof(double) * (size_t)(J->m > 0 ? J->m : 1));
    if (!acc) {
        __atomic_store_n(&J->failed, 1, __ATOMIC_RELAXED);
        return NULL;
    }
    for (;;) {
        const int b = __atomic_fetch_add(&J->next, 256, __ATOMIC_RELAXED);
        if (b >= J->m) break;
        const int e = b + 256 < J->m ? b + 256 : J->m;
        for (int i = b; i < e; i++)
            adat_numeric_row(i, J->row_ptr, J->col_ind, J->val, J->col_ptr, J->row_ind, J->valT, J->d, J->pat_ptr,
                             J->pat_col, J->link, acc, J->out);
    }
    free(acc);
    return NULL;
}

int oracle_adat_numeric_threads(int m, int n, const int* row_ptr, const int* col_ind, const double* val,
                                const int* col_ptr, const int* row_ind, const double* valT, const double* d,
                                const int* pat_ptr, const int* pat_col, double* out, int threads) {
    int* link = csr_to_csc_link(m, n, row_ptr, col_ind, col_ptr);
    if (!link) return -1;
    adat_job J = {m, row_ptr, col_ind, col_ptr, row_ind, pat_ptr, pat_col, link, val, valT, d, out, 0, 0};
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    int started = 0;
    for (int t = 1; t < threads; t++)
        if (pthread_create(&tid[started], NULL, adat_worker, &J) == 0) started++;
    adat_worker(&J);
    for (int t = 0; t < started; t++) pthread_join(tid[t], NULL);
    free(link);
    return J.failed ? -1 : started + 1;
}

/* ---------------------------------------------------------------- partial Cholesky */

void oracle_diag_adat(int m, const int* row_ptr, const int* col_ind, const double* val, const double* d,
                      double gamma, double delta, double* diag) {
    for (int i = 0; i < m; i++) {
        diag[i] = delta;
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; j++) diag[i] += val[j] * val[j] / (d[col_ind[j]] + gamma);
    }
}

void oracle_pchol_free(oracle_pchol* pc) {
    if (!pc) return;
    free(pc->perm);
    free(pc->L);
    free(pc->D);
    free(pc->diag_s);
    free(pc->l11inv);
    free(pc->beg);
    free(pc->end);
    memset(pc, 0, sizeof(*pc));
}

/* PCG.cpp:38-177.  Step 1 diagonal, step 2 k pivots with a left-looking
 * LDL^T column update and Schur-diagonal downdate, step 3 the permuted row
 * pointers, step 4.1 L11^-1 by elimination.  Step 4.2's explicit Inv1/Inv2
 * CSR matrices are applied implicitly by oracle_precond_apply in the same
 * arithmetic order. */
int oracle_pchol_build(int m, int n, const int* row_ptr, const int* col_ind, const double* val,
                       const double* d, double gamma, double delta, int k_req, int rule, const int* given,
                       oracle_pchol* out) {
    memset(out, 0, sizeof(*out));
    const int K = k_req < m ? k_req : m;
    if (K < 0 || m <= 0) return -1;
    out->m = m;
    out->k = K;
    out->perm = (int*)malloc(sizeof(int) * (size_t)m);
    out->L = (double*)calloc((size_t)m * (size_t)(K > 0 ? K : 1), sizeof(double));
    out->D = (double*)calloc((size_t)(K > 0 ? K : 1), sizeof(double));
    out->diag_s = (double*)malloc(sizeof(double) * (size_t)m);
    out->l11inv = (double*)calloc((size_t)(K > 0 ? K : 1) * (size_t)(K > 0 ? K : 1), sizeof(double));
    out->beg = (int*)malloc(sizeof(int) * (size_t)m);
    out->end = (int*)malloc(sizeof(int) * (size_t)m);
    double* U = (double*)calloc((size_t)m * (size_t)(K > 0 ? K : 1), sizeof(double));
    double* temp_gr = (double*)calloc((size_t)m, sizeof(double));
    double* scatter = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    int* where = (int*)malloc(sizeof(int) * (size_t)m);
    if (!out->perm || !out->L || !out->D || !out->diag_s || !out->l11inv || !out->beg || !out->end || !U ||
        !temp_gr || !scatter || !where) {
        free(U);
        free(temp_gr);
        free(scatter);
        free(where);
        oracle_pchol_free(out);
        return -2;
    }
    double* DS = out->diag_s;
    int* perm = out->perm;
    double* L = out->L;
    double* D = out->D;
#define LL(row, c) L[(size_t)(row) * (size_t)K + (size_t)(c)]
#define UU(row, c) U[(size_t)(row) * (size_t)K + (size_t)(c)]

    /* Step 1: PCG.cpp:41-46 */
    oracle_diag_adat(m, row_ptr, col_ind, val, d, gamma, delta, DS);

    /* Step 2: PCG.cpp:49-103 */
    for (int i = 0; i < m; i++) perm[i] = i, where[i] = i;
    for (int k = 0; k < K; k++) {
        int col_max_ind = k;
        if (rule == ORACLE_PIVOT_GREEDY) {
            for (int i = k + 1; i < m; i++)
                if (DS[perm[i]] > DS[perm[col_max_ind]]) col_max_ind = i;
        } else {
            col_max_ind = where[given[k]];
        }
        {
            const int a = perm[k], b = perm[col_max_ind];
            perm[k] = b;
            perm[col_max_ind] = a;
            where[b] = k;
            where[a] = col_max_ind;
        }
        const int col_max = perm[k];
        for (int j = row_ptr[col_max]; j < row_ptr[col_max + 1]; j++)
            scatter[col_ind[j]] = val[j] / (d[col_ind[j]] + gamma);
        for (int i = k; i < m; i++) {
            const int ii = perm[i];
            temp_gr[ii] = 0;
            for (int j = row_ptr[ii]; j < row_ptr[ii + 1]; j++) temp_gr[ii] += val[j] * scatter[col_ind[j]];
        }
        temp_gr[col_max] += delta;
        for (int j = row_ptr[col_max]; j < row_ptr[col_max + 1]; j++) scatter[col_ind[j]] = 0;

        D[k] = temp_gr[col_max];
        for (int j = k + 1; j < m; j++) UU(perm[j], k) = temp_gr[perm[j]];
        for (int r = 0; r < k; r++) {
            const double tmp = LL(col_max, r);
            D[k] -= UU(col_max, r) * tmp;
            for (int j = k + 1; j < m; j++) UU(perm[j], k) -= UU(perm[j], r) * tmp;
        }
        LL(col_max, k) = 1;
        for (int j = k + 1; j < m; j++) LL(perm[j], k) = UU(perm[j], k) / D[k];
        const double tmp_d = D[k];
        for (int j = k + 1; j < m; j++) DS[perm[j]] -= tmp_d * LL(perm[j], k) * LL(perm[j], k);
    }

    /* Step 3: PCG.cpp:106-110 */
    for (int i = 0; i < m; i++) {
        out->beg[i] = row_ptr[perm[i]];
        out->end[i] = row_ptr[perm[i] + 1];
    }

    /* Step 4.1: PCG.cpp:119-133 (unit-lower L11, inverse by elimination) */
    double* inv = out->l11inv;
    for (int i = 0; i < K; i++)
        for (int j = 0; j < K; j++) inv[(size_t)i * K + j] = (double)(i == j);
    for (int j = 0; j < K; j++)
        for (int i = j + 1; i < K; i++) {
            const double factor = LL(perm[i], j);
            for (int c = 0; c <= j; c++) inv[(size_t)i * K + c] -= inv[(size_t)j * K + c] * factor;
        }
#undef LL
#undef UU
    free(U);
    free(temp_gr);
    free(scatter);
    free(where);
    return 0;
}

/* PCG.cpp:183-196: Ret = Inv2^T Inv1^T D_S^-1 Inv1 Inv2 r, where
 * Inv2 = diag(L11^-1, I) and Inv1 = [I 0; -L21 I] (PCG.cpp:135-176), applied
 * with the operation order of the CSR matrices the reference builds. */
void oracle_precond_apply(const oracle_pchol* pc, const double* r, double* out) {
    const int m = pc->m, K = pc->k;
    const int* perm = pc->perm;
    const double* inv = pc->l11inv;
    double* t1 = (double*)malloc(sizeof(double) * (size_t)m);
    double* t2 = (double*)malloc(sizeof(double) * (size_t)m);
    if (!t1 || !t2) {
        free(t1);
        free(t2);
        return;
    }
    /* t1 = Inv2 r  ('N', beta 0) */
    for (int i = 0; i < K; i++) {
        double s = 0.0;
        for (int j = 0; j <= i; j++) s += inv[(size_t)i * K + j] * r[j];
        t1[i] = 0.0 + 1.0 * s;
    }
    for (int i = K; i < m; i++) {
        double s = 0.0;
        s += 1.0 * r[i];
        t1[i] = 0.0 + 1.0 * s;
    }
    /* t2 = Inv1 t1  ('N', beta 0) */
    for (int i = 0; i < K; i++) {
        double s = 0.0;
        s += 1.0 * t1[i];
        t2[i] = 0.0 + 1.0 * s;
    }
    for (int i = K; i < m; i++) {
        double s = 0.0;
        const double* Lrow = pc->L + (size_t)perm[i] * (size_t)K;
        for (int j = 0; j < K; j++) s += (-Lrow[j]) * t1[j];
        s += 1.0 * t1[i];
        t2[i] = 0.0 + 1.0 * s;
    }
    /* t2 /= DIAG_S[perm[i]] */
    for (int i = 0; i < m; i++) t2[i] /= pc->diag_s[perm[i]];
    /* t1 = Inv1^T t2  ('T', beta 0) */
    for (int j = 0; j < m; j++) t1[j] = 0.0;
    for (int i = 0; i < K; i++) {
        const double a = 1.0 * t2[i];
        t1[i] += 1.0 * a;
    }
    for (int i = K; i < m; i++) {
        const double a = 1.0 * t2[i];
        const double* Lrow = pc->L + (size_t)perm[i] * (size_t)K;
        for (int j = 0; j < K; j++) t1[j] += (-Lrow[j]) * a;
        t1[i] += 1.0 * a;
    }
    /* out = Inv2^T t1  ('T', beta 0) */
    for (int j = 0; j < m; j++) out[j] = 0.0;
    for (int i = 0; i < K; i++) {
        const double a = 1.0 * t1[i];
        for (int j = 0; j <= i; j++) out[j] += inv[(size_t)i * K + j] * a;
    }
    for (int i = K; i < m; i++) {
        const double a = 1.0 * t1[i];
        out[i] += 1.0 * a;
    }
    free(t1);
    free(t2);
}

/* ---------------------------------------------------------------- PCG */

/* PCG.cpp:296-395 */
int64_t oracle_pcg(int m, int n, const int* row_ptr, const int* col_ind, const double* val,
                   const double* d, double gamma, double delta, const double* b, double* x, int k,
                   int rule, const int* given, double tol, int64_t max_iter) {
    oracle_pchol pc;
    if (oracle_pchol_build(m, n, row_ptr, col_ind, val, d, gamma, delta, k, rule, given, &pc)) return -2;
    double* tmp_col = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    double* r = (double*)malloc(sizeof(double) * (size_t)m);
    double* z = (double*)malloc(sizeof(double) * (size_t)m);
    double* p = (double*)malloc(sizeof(double) * (size_t)m);
    double* q = (double*)malloc(sizeof(double) * (size_t)m);
    double* xs = (double*)malloc(sizeof(double) * (size_t)m);
    if (!tmp_col || !r || !z || !p || !q || !xs) {
        free(tmp_col), free(r), free(z), free(p), free(q), free(xs);
        oracle_pchol_free(&pc);
        return -2;
    }
    const int* perm = pc.perm;
    for (int i = 0; i < m; i++) x[i] = 0;
    oracle_csrmv_t(m, n, 1.0, val, col_ind, pc.beg, pc.end, x, 0.0, tmp_col);
    for (int i = 0; i < n; i++) tmp_col[i] /= d[i] + gamma;
    for (int i = 0; i < m; i++) r[i] = b[perm[i]] - delta * x[i];
    oracle_csrmv_n(m, n, -1.0, val, col_ind, pc.beg, pc.end, tmp_col, 1.0, r);
    oracle_precond_apply(&pc, r, z);
    for (int i = 0; i < m; i++) p[i] = z[i];
    const double terminate = blas_nrm2(m, r) * tol;
    int64_t loop = 0;
    for (;;) {
        const double rnorm = blas_nrm2(m, r);
        if (rnorm < terminate) break;
        if (loop >= max_iter) break;
        loop++;
        oracle_csrmv_t(m, n, 1.0, val, col_ind, pc.beg, pc.end, p, 0.0, tmp_col);
        for (int i = 0; i < n; i++) tmp_col[i] /= d[i] + gamma;
        for (int i = 0; i < m; i++) q[i] = delta * p[i];
        oracle_csrmv_n(m, n, 1.0, val, col_ind, pc.beg, pc.end, tmp_col, 1.0, q);
        const double alpha_up = blas_dot(m, z, r);
        const double alpha_down = blas_dot(m, p, q);
        const double alpha = alpha_up / alpha_down;
        blas_axpy(m, alpha, p, x);
        blas_axpy(m, -alpha, q, r);
        oracle_precond_apply(&pc, r, z);
        const double beta_up = blas_dot(m, z, r);
        const double beta = beta_up / alpha_up;
        for (int i = 0; i < m; i++) p[i] *= beta;
        blas_axpy(m, 1.0, z, p);
    }
    for (int i = 0; i < m; i++) xs[perm[i]] = x[i];
    for (int i = 0; i < m; i++) x[i] = xs[i];
    free(tmp_col), free(r), free(z), free(p), free(q), free(xs);
    oracle_pchol_free(&pc);
    return loop;
}

/* ---------------------------------------------------------------- top-k */

int oracle_topk_pivots(int m, const double* diag, int k, int* pivots) {
    const int K = k < m ? k : m;
    int* idx = (int*)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    if (!idx) return -1;
    for (int i = 0; i < m; i++) idx[i] = i;
    /* partial selection sort is enough for test sizes; order (value desc, index asc) */
    for (int a = 0; a < K; a++) {
        int best = a;
        for (int i = a + 1; i < m; i++) {
            const double vi = diag[idx[i]], vb = diag[idx[best]];
            if (vi > vb || (vi == vb && idx[i] < idx[best])) best = i;
        }
        const int t = idx[a];
        idx[a] = idx[best];
        idx[best] = t;
    }
    /* increasing row order */
    for (int a = 1; a < K; a++) {
        const int v = idx[a];
        int b = a - 1;
        while (b >= 0 && idx[b] > v) {
            idx[b + 1] = idx[b];
            b--;
        }
        idx[b + 1] = v;
    }
    for (int a = 0; a < K; a++) pivots[a] = idx[a];
    free(idx);
    return K;
}

/* ---------------------------------------------------------------- backend */

struct oracle_ne {
    int m, n, k, rule;
    double tol;
    int64_t max_iter, last_iters, total_iters;
    int *row_ptr, *col_ind; /* CSR(A)   */
    double* val;
    int *col_ptr, *row_ind; /* CSC(A) = CSR(A^T) */
    double* valT;
    double *tmp_row, *tmp_col, *x2;
    int* given;
};

oracle_ne* oracle_ne_create(int k, int rule, double tol, int64_t max_iter) {
    oracle_ne* ne = (oracle_ne*)calloc(1, sizeof(oracle_ne));
    if (!ne) return NULL;
    ne->k = k;
    ne->rule = rule;
    ne->tol = tol;
    ne->max_iter = max_iter;
    return ne;
}

/* UsePCG_CPU.cpp:26-68: CSR(A^T) straight from the column lists and CSR(A)
 * from the row lists (both sorted). */
int oracle_ne_construct(void* ctx, int32_t m, int32_t n, const int32_t* col_ptr, const int32_t* row_ind,
                        const double* val) {
    oracle_ne* ne = (oracle_ne*)ctx;
    const int nnz = col_ptr[n];
    ne->m = m;
    ne->n = n;
    ne->col_ptr = (int*)malloc(sizeof(int) * (size_t)(n + 1));
    ne->row_ind = (int*)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    ne->valT = (double*)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    ne->row_ptr = (int*)calloc((size_t)m + 1, sizeof(int));
    ne->col_ind = (int*)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    ne->val = (double*)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    ne->tmp_row = (double*)malloc(sizeof(double) * (size_t)m);
    ne->tmp_col = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    ne->x2 = (double*)malloc(sizeof(double) * (size_t)m);
    ne->given = (int*)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    if (!ne->col_ptr || !ne->row_ind || !ne->valT || !ne->row_ptr || !ne->col_ind || !ne->val || !ne->tmp_row ||
        !ne->tmp_col || !ne->x2 || !ne->given)
        return -2;
    memcpy(ne->col_ptr, col_ptr, sizeof(int) * (size_t)(n + 1));
    memcpy(ne->row_ind, row_ind, sizeof(int) * (size_t)nnz);
    memcpy(ne->valT, val, sizeof(double) * (size_t)nnz);
    for (int p = 0; p < nnz; p++) ne->row_ptr[row_ind[p] + 1]++;
    for (int i = 0; i < m; i++) ne->row_ptr[i + 1] += ne->row_ptr[i];
    int* fill = (int*)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    if (!fill) return -2;
    for (int i = 0; i < m; i++) fill[i] = ne->row_ptr[i];
    for (int j = 0; j < n; j++)
        for (int p = col_ptr[j]; p < col_ptr[j + 1]; p++) {
            const int q = fill[row_ind[p]]++;
            ne->col_ind[q] = j;
            ne->val[q] = val[p];
        }
    free(fill);
    return 0;
}

/* UsePCG_CPU.cpp:78-80: a no-op -- the reference rebuilds its preconditioner
 * inside every solve (PCG.cpp:301). */
int oracle_ne_renew(void* ctx, const double* d) {
    (void)ctx;
    (void)d;
    return 0;
}

/* UsePCG_CPU.cpp:91-183 */
int oracle_ne_solve(void* ctx, const double* d, const double* b_1, const double* b_2, double* x_1,
                    double* x_2) {
    oracle_ne* ne = (oracle_ne*)ctx;
    const int m = ne->m, n = ne->n;
    for (int i = 0; i < m; i++) ne->tmp_row[i] = -b_2[i];
    for (int i = 0; i < n; i++) ne->tmp_col[i] = b_1[i] / d[i];
    blas_csrmv('T', n, m, 1.0, ne->valT, ne->row_ind, ne->col_ptr, ne->tmp_col, 1.0, ne->tmp_row);
    const int* given = NULL;
    if (ne->rule == ORACLE_PIVOT_GIVEN) {
        double* diag = (double*)malloc(sizeof(double) * (size_t)m);
        if (!diag) return -2;
        oracle_diag_adat(m, ne->row_ptr, ne->col_ind, ne->val, d, 0.0, 0.0, diag);
        oracle_topk_pivots(m, diag, ne->k, ne->given);
        free(diag);
        given = ne->given;
    }
    const int64_t it = oracle_pcg(m, n, ne->row_ptr, ne->col_ind, ne->val, d, 0.0, 0.0, ne->tmp_row, ne->x2,
                                  ne->k, ne->rule, given, ne->tol, ne->max_iter);
    if (it < 0) return -2;
    ne->last_iters = it;
    ne->total_iters += it;
    for (int i = 0; i < m; i++) x_2[i] = ne->x2[i];
    for (int i = 0; i < n; i++) ne->tmp_col[i] = b_1[i];
    blas_csrmv('N', n, m, -1.0, ne->valT, ne->row_ind, ne->col_ptr, x_2, 1.0, ne->tmp_col);
    for (int i = 0; i < n; i++) x_1[i] = ne->tmp_col[i] / d[i];
    return 0;
}

/* UsePCG_CPU.cpp:70-75 */
int oracle_ne_destruct(void* ctx) {
    oracle_ne* ne = (oracle_ne*)ctx;
    free(ne->row_ptr), free(ne->col_ind), free(ne->val);
    free(ne->col_ptr), free(ne->row_ind), free(ne->valT);
    free(ne->tmp_row), free(ne->tmp_col), free(ne->x2), free(ne->given);
    ne->row_ptr = ne->col_ind = ne->col_ptr = ne->row_ind = ne->given = NULL;
    ne->val = ne->valT = ne->tmp_row = ne->tmp_col = ne->x2 = NULL;
    return 0;
}

void oracle_ne_free(oracle_ne* ne) { free(ne); }
int64_t oracle_ne_last_iters(const oracle_ne* ne) { return ne->last_iters; }
int64_t oracle_ne_total_iters(const oracle_ne* ne) { return ne->total_iters; }
