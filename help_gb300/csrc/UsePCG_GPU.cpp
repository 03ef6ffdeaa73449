// Drop-in GPU normal-equations backend for the HELP interior-point solver.
//
// The reference picks its normal-equations backend at link time: every
// backend defines the four functions declared in LP.h:157-160, and the PCG
// one is UsePCG_CPU.cpp + PCG.cpp.  Build the reference with this file in
// their place and link libhelp_gpu.so:
//
//   g++ -O2 -fopenmp -I<HELP sources> -I<this repo>/include
//       Crushing.cpp GlobalVar.cpp Hash.cpp Helper.cpp HSDSolver.cpp Init.cpp
//       Main.cpp MPSRead.cpp Presolve.cpp Report.cpp UsePCG_GPU.cpp
//       -L<this repo>/help_gb300/_lib -lhelp_gpu -Wl,-rpath,<...>
//   (one command line)
//
// MPSRead, Crushing, Presolve, the HSD iteration and Report are unchanged.
// The matrix is read from the same globals UsePCG_CPU.cpp reads
// (V_Matrix_Col_Head / _Next / _Row / _Value, LP.h:105-109) and handed to the
// GPU once; RenewLinearEquation builds the preconditioner once per
// interior-point iteration (the CPU backend rebuilds it inside each of the
// three solves, PCG.cpp:301).  Errors go through the reference's CheckError,
// which releases the backend and exits (Helper.cpp:24-35).
//
// Options come from the environment (defaults = the reference's PCG:
// 10 pivots, FP64, relative tolerance 1e-20): HELP_GPU_PIVOTS,
// HELP_GPU_PRECISION (fp64 | mixed), HELP_GPU_CG_TOL, HELP_GPU_CG_MAX_ITER,
// HELP_GPU_DEVICE, HELP_GPU_CAP_OK (1: a solve that stops at the iteration
// cap hands back its inexact direction instead of failing; the reference's
// CG has no cap).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "LP.h"
#include "help_gpu.h"

static help_pcg* g_help_ctx = nullptr;

static void help_check(int rc, const char* what) {
    if (rc != HELP_OK) {
        std::printf("help_gpu: %s failed: %s\n", what, help_pcg_last_error(g_help_ctx));
        CheckError(rc, (char*)what);
    }
}

int LinearEquation_Construct() {
    help_pcg_options opt;
    help_pcg_default_options(&opt);
    if (const char* s = std::getenv("HELP_GPU_PIVOTS")) opt.pivots = std::atoi(s);
    if (const char* s = std::getenv("HELP_GPU_PRECISION")) opt.precision = std::strcmp(s, "mixed") ? HELP_PREC_FP64 : HELP_PREC_MIXED;
    if (const char* s = std::getenv("HELP_GPU_CG_TOL")) opt.cg_tol = std::atof(s);
    if (const char* s = std::getenv("HELP_GPU_CG_MAX_ITER")) opt.cg_max_iter = std::atoll(s);
    if (const char* s = std::getenv("HELP_GPU_DEVICE")) opt.device = std::atoi(s);
    if (const char* s = std::getenv("HELP_GPU_CAP_OK")) opt.cap_ok = std::atoi(s);
    help_check(help_pcg_create(&opt, &g_help_ctx), "help_pcg_create");
    // CSC of A from the column lists (rows are sorted inside each column
    // after Presolve_Init, Presolve.cpp:77-113)
    std::vector<int32_t> col_ptr(n_Col + 1, 0), row_ind;
    std::vector<double> val;
    for (int j = 0; j < n_Col; j++) {
        col_ptr[j] = (int32_t)row_ind.size();
        for (int p = V_Matrix_Col_Head[j]; p != -1; p = V_Matrix_Col_Next[p]) {
            row_ind.push_back(V_Matrix_Row[p]);
            val.push_back(V_Matrix_Value[p]);
        }
    }
    col_ptr[n_Col] = (int32_t)row_ind.size();
    help_check(help_pcg_construct(g_help_ctx, n_Row, n_Col, col_ptr.data(), row_ind.data(), val.data()),
               "help_pcg_construct");
    return 0;
}

int LinearEquation_Destruct() {
    if (g_help_ctx) {
        help_pcg_free(g_help_ctx);
        g_help_ctx = nullptr;
    }
    return 0;
}

void RenewLinearEquation(double* d) { help_check(help_pcg_renew(g_help_ctx, d), "help_pcg_renew"); }

int SolveLinearEquation(double* d, double* b_1, double* b_2, double* x_1, double* x_2) {
    help_check(help_pcg_solve(g_help_ctx, d, b_1, b_2, x_1, x_2), "help_pcg_solve");
    return 0;
}
