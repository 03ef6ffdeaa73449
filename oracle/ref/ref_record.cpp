// Recording wrapper around the reference's own SolveLinearEquation
// (UsePCG_CPU.cpp:91-183).  The recipe compiles UsePCG_CPU.cpp with
// -DSolveLinearEquation=help_ref_inner_solve, so the reference's HSD driver
// (HSDSolver.cpp:186) lands here; each call is forwarded unchanged and, when
// HELP_REF_RECORD names a directory, its inputs, outputs and CG iteration
// count are appended to <dir>/solves.bin:
//   int32 m, int32 n, int64 cg_iters, d[n], b_1[n], b_2[m], x_1[n], x_2[m]
// CG iterations are counted through the cblas_dnrm2 stand-in (k + 2 calls).
//
// The same recipe renames RenewLinearEquation and LinearEquation_Destruct, so
// the HSD loop's renews (HSDSolver.cpp:627, :768) are counted here and its
// final iterate is read when HSD_Main destructs the backend
// (HSDSolver.cpp:881): with HELP_REF_FINAL naming a file, the last printed
// row's values (HSD_Calc_Newton_Parameters, HSDSolver.cpp:752-753) are
// written there at full precision, one `key value` pair per line (%.17g).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>

extern int n_Row, n_Col;
extern double HSD_primal_obj, HSD_dual_obj, HSD_relative_gap, HSD_primal_infeas, HSD_dual_infeas;
extern double HSD_tau, HSD_kappa;
extern int HSD_Status;
long long help_ref_nrm2_calls = 0;
static long long help_ref_renews = 0, help_ref_solves = 0, help_ref_cg_total = 0;
int help_ref_inner_solve(double* d, double* b_1, double* b_2, double* x_1, double* x_2);
void help_ref_inner_renew(double* d);
int help_ref_inner_destruct();

void RenewLinearEquation(double* d) {
    ++help_ref_renews;
    help_ref_inner_renew(d);
}

int LinearEquation_Destruct() {
    const char* path = std::getenv("HELP_REF_FINAL");
    if (path && *path) {
        FILE* f = std::fopen(path, "w");
        if (f) {
            std::fprintf(f, "status %d\n", HSD_Status);
            // one renew per iteration that did not stop, plus the one in the
            // starting-point set-up (HSDSolver.cpp:627): the last printed Iter
            std::fprintf(f, "iterations %lld\n", help_ref_renews);
            std::fprintf(f, "solves %lld\n", help_ref_solves);
            std::fprintf(f, "cg_iterations %lld\n", help_ref_cg_total);
            std::fprintf(f, "primal_obj %.17g\n", HSD_primal_obj);
            std::fprintf(f, "dual_obj %.17g\n", HSD_dual_obj);
            std::fprintf(f, "rel_gap %.17g\n", HSD_relative_gap);
            std::fprintf(f, "primal_infeas %.17g\n", HSD_primal_infeas);
            std::fprintf(f, "dual_infeas %.17g\n", HSD_dual_infeas);
            std::fprintf(f, "tau %.17g\n", HSD_tau);
            std::fprintf(f, "kappa %.17g\n", HSD_kappa);
            std::fclose(f);
        }
    }
    return help_ref_inner_destruct();
}

int SolveLinearEquation(double* d, double* b_1, double* b_2, double* x_1, double* x_2) {
    const int m = n_Row, n = n_Col;
    std::vector<double> d0(d, d + n), b10(b_1, b_1 + n), b20(b_2, b_2 + m);
    const long long before = help_ref_nrm2_calls;
    const int rc = help_ref_inner_solve(d, b_1, b_2, x_1, x_2);
    const int64_t iters = (int64_t)(help_ref_nrm2_calls - before - 2);
    ++help_ref_solves;
    help_ref_cg_total += iters;
    const char* dir = std::getenv("HELP_REF_RECORD");
    if (dir && *dir) {
        char path[4096];
        std::snprintf(path, sizeof(path), "%s/solves.bin", dir);
        FILE* f = std::fopen(path, "ab");
        if (f) {
            const int32_t hdr[2] = {m, n};
            std::fwrite(hdr, sizeof(int32_t), 2, f);
            std::fwrite(&iters, sizeof(int64_t), 1, f);
            std::fwrite(d0.data(), sizeof(double), n, f);
            std::fwrite(b10.data(), sizeof(double), n, f);
            std::fwrite(b20.data(), sizeof(double), m, f);
            std::fwrite(x_1, sizeof(double), n, f);
            std::fwrite(x_2, sizeof(double), m, f);
            std::fclose(f);
        }
    }
    return rc;
}
