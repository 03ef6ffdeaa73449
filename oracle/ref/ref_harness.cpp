// Function-level harness over the reference's own PCG-path sources
// (Helper.cpp, PCG.cpp, UsePCG_CPU.cpp, GlobalVar.cpp), compiled unmodified
// against the MKL stand-in.  It loads a CSC matrix into the reference's
// linked-list globals the way Presolve_Init leaves them (rows sorted inside
// columns, columns sorted inside rows; Presolve.cpp:77-113) and exposes the
// hot-path functions with C linkage so tests can compare the CPU restatement
// under oracle/ against the reference itself.
#include "LP.h"
#include "PCG.h"
#include <cstdint>
#include <vector>

long long help_ref_nrm2_calls = 0;

// Defined with external linkage in the reference sources.
extern double DIAG_S[];                                              // PCG.cpp:20
void RenewPartialCholesky(int n_Row, int n_Col, double* csrValA, int* csrColIndA,
                          int* csrRowPtrA, double* d, double gamma, double delta);  // PCG.cpp:38
extern double* csrValA;                                              // UsePCG_CPU.cpp:21
extern int csrRowPtrA[];
extern int* csrColIndA;

extern "C" {

int ref_max_rows() { return MAX_ROWS; }
int ref_max_cols() { return MAX_COLS; }
int ref_pchol_cols() { return PART_CHOL_COLS; }

int ref_load(int m, int n, const int* col_ptr, const int* row_ind, const double* val) {
    const int nnz = col_ptr[n];
    if (m > MAX_ROWS || n > MAX_COLS || nnz > MAX_ELEMENTS) return -1;
    n_Row = m; n_Col = n; n_Element = nnz;
    n_LB = n; n_UB = 0; n_FR = 0;
    for (int j = 0; j < n; ++j) {
        V_Matrix_Col_Head[j] = (col_ptr[j] < col_ptr[j + 1]) ? col_ptr[j] : -1;
        for (int p = col_ptr[j]; p < col_ptr[j + 1]; ++p) {
            V_Matrix_Row[p] = row_ind[p];
            V_Matrix_Col[p] = j;
            V_Matrix_Value[p] = val[p];
            V_Matrix_Col_Next[p] = (p + 1 < col_ptr[j + 1]) ? p + 1 : -1;
            V_Matrix_Col_Prev[p] = (p > col_ptr[j]) ? p - 1 : -1;
        }
    }
    std::vector<int> tail(m, -1);
    for (int i = 0; i < m; ++i) V_Matrix_Row_Head[i] = -1;
    for (int j = 0; j < n; ++j)
        for (int p = col_ptr[j]; p < col_ptr[j + 1]; ++p) {
            const int i = row_ind[p];
            V_Matrix_Row_Next[p] = -1;
            V_Matrix_Row_Prev[p] = tail[i];
            if (tail[i] < 0) V_Matrix_Row_Head[i] = p; else V_Matrix_Row_Next[tail[i]] = p;
            tail[i] = p;
        }
    return 0;
}

int ref_construct() { return LinearEquation_Construct(); }

long long ref_solve(const double* d, const double* b1, const double* b2, double* x1, double* x2) {
    std::vector<double> dd(d, d + n_Col), bb1(b1, b1 + n_Col), bb2(b2, b2 + n_Row);
    const long long before = help_ref_nrm2_calls;
    SolveLinearEquation(dd.data(), bb1.data(), bb2.data(), x1, x2);
    return help_ref_nrm2_calls - before - 2;
}

void ref_csrmv_n(int m, int n, double alpha, const double* val, const int* col, const int* beg,
                 const int* end, const double* x, double beta, double* y) {
    CSRMV_N(m, n, alpha, (double*)val, (int*)col, (int*)beg, (int*)end, (double*)x, beta, y);
}

void ref_csrmv_t(int m, int n, double alpha, const double* val, const int* col, const int* beg,
                 const int* end, const double* x, double beta, double* y) {
    CSRMV_T(m, n, alpha, (double*)val, (int*)col, (int*)beg, (int*)end, (double*)x, beta, y);
}

// RenewPartialCholesky on the CSR(A) built by ref_construct().  L is returned
// row-major as [m][PART_CHOL_COLS] indexed by original row, D as [PART_CHOL_COLS].
int ref_pchol(const double* d, double gamma, double delta, int* perm, double* L, double* D,
              double* diag_s) {
    std::vector<double> dd(d, d + n_Col);
    RenewPartialCholesky(n_Row, n_Col, csrValA, csrColIndA, csrRowPtrA, dd.data(), gamma, delta);
    for (int i = 0; i < n_Row; ++i) {
        perm[i] = PCG_PERM[i];
        diag_s[i] = DIAG_S[i];
        for (int c = 0; c < PART_CHOL_COLS; ++c) L[(size_t)i * PART_CHOL_COLS + c] = PARTIAL_CHOL_L[i][c];
    }
    for (int c = 0; c < PART_CHOL_COLS; ++c) D[c] = PARTIAL_CHOL_D[c];
    return PART_CHOL_COLS;
}

// Preconditioner (PCG.cpp:183-196) on a vector in the permuted row order of
// the last ref_pchol call.
void ref_precond(const double* r, double* out) {
    std::vector<double> rr(r, r + n_Row);
    Preconditioner(n_Row, n_Col, rr.data(), out);
}

// ADAt_Allocate + ADAt_Calc (Helper.cpp:215-271, :331-348): the upper
// triangle of A diag(d) A^T in the reference's discovery order.
int ref_adat(const double* d, int* row_ptr, int* col, double* val, int cap) {
    int nnz = 0;
    double* pv = nullptr;
    int* pc = nullptr;
    ADAt_Allocate(&nnz, &pv, row_ptr, &pc);
    if (nnz > cap) { free(pv); free(pc); return -nnz; }
    ADAt_Calc((double*)d, pv, row_ptr, pc);
    for (int p = 0; p < nnz; ++p) { col[p] = pc[p]; val[p] = pv[p]; }
    free(pv);
    free(pc);
    return nnz;
}

}  // extern "C"
