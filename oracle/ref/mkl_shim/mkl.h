/*
 * Stand-in for the Intel MKL header the reference includes (MKL_Util.h:15-17).
 * MKL is not available on this machine, so each routine the reference's PCG
 * path calls is given its standard BLAS / sparse-BLAS meaning as a plain loop,
 * written from the BLAS definitions.  Used only to build the reference as a
 * test oracle (its PCG path, and LUSOL under its dependent-row presolve).
 *
 * help_ref_nrm2_calls counts cblas_dnrm2 calls: ConjugateGradient calls it
 * once before its loop and once at the top of every pass (PCG.cpp:335, :341),
 * so a solve that ran k CG iterations makes k + 2 calls.
 */
#ifndef HELP_MKL_SHIM_H
#define HELP_MKL_SHIM_H
#include <math.h>

extern long long help_ref_nrm2_calls;

/* y := alpha*op(A)*x + beta*y for a zero-based CSR matrix A (m x k) given by
 * (val, indx, pntrb, pntre); op = 'N' (y has m entries) or 'T' (y has k). */
static inline void mkl_dcsrmv(const char* transa, const int* m, const int* k, const double* alpha,
                              const char* matdescra, const double* val, const int* indx,
                              const int* pntrb, const int* pntre, const double* x,
                              const double* beta, double* y) {
    (void)matdescra;
    const int M = *m, K = *k;
    if (*transa == 'N' || *transa == 'n') {
        for (int i = 0; i < M; i++) {
            double s = 0.0;
            for (int p = pntrb[i]; p < pntre[i]; p++) s += val[p] * x[indx[p]];
            y[i] = (*beta == 0.0 ? 0.0 : *beta * y[i]) + *alpha * s;
        }
    } else {
        for (int j = 0; j < K; j++) y[j] = (*beta == 0.0 ? 0.0 : *beta * y[j]);
        for (int i = 0; i < M; i++) {
            const double a = *alpha * x[i];
            for (int p = pntrb[i]; p < pntre[i]; p++) y[indx[p]] += val[p] * a;
        }
    }
}
static inline double cblas_ddot(int n, const double* x, int incx, const double* y, int incy) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += x[i * incx] * y[i * incy];
    return s;
}
static inline double cblas_dnrm2(int n, const double* x, int incx) {
    help_ref_nrm2_calls++;
    double s = 0.0;
    for (int i = 0; i < n; i++) s += x[i * incx] * x[i * incx];
    return sqrt(s);
}
static inline void cblas_daxpy(int n, double a, const double* x, int incx, double* y, int incy) {
    for (int i = 0; i < n; i++) y[i * incy] += a * x[i * incx];
}
static inline void cblas_dscal(int n, double a, double* x, int incx) {
    for (int i = 0; i < n; i++) x[i * incx] *= a;
}
static inline void cblas_dcopy(int n, const double* x, int incx, double* y, int incy) {
    for (int i = 0; i < n; i++) y[i * incy] = x[i * incx];
}
/* The two further routines LUSOL's BLAS layer calls (lusol/myblas.cpp, used
 * by the reference's dependent-row presolve). */
static inline void cblas_dswap(int n, double* x, int incx, double* y, int incy) {
    for (int i = 0; i < n; i++) {
        const double t = x[i * incx];
        x[i * incx] = y[i * incy];
        y[i * incy] = t;
    }
}
/* zero-based index of the first entry of largest magnitude (0 when n < 1) */
static inline int cblas_idamax(int n, const double* x, int incx) {
    int best = 0;
    double vmax = -1.0;
    for (int i = 0; i < n; i++)
        if (fabs(x[i * incx]) > vmax) {
            vmax = fabs(x[i * incx]);
            best = i;
        }
    return best;
}
#endif
