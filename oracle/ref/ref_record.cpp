// Recording wrapper around the reference's own SolveLinearEquation
// (UsePCG_CPU.cpp:91-183).  The recipe compiles UsePCG_CPU.cpp with
// -DSolveLinearEquation=help_ref_inner_solve, so the reference's HSD driver
// (HSDSolver.cpp:186) lands here; each call is forwarded unchanged and, when
// HELP_REF_RECORD names a directory, its inputs, outputs and CG iteration
// count are appended to <dir>/solves.bin:
//   int32 m, int32 n, int64 cg_iters, d[n], b_1[n], b_2[m], x_1[n], x_2[m]
// CG iterations are counted through the cblas_dnrm2 stand-in (k + 2 calls).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>

extern int n_Row, n_Col;
long long help_ref_nrm2_calls = 0;
int help_ref_inner_solve(double* d, double* b_1, double* b_2, double* x_1, double* x_2);

int SolveLinearEquation(double* d, double* b_1, double* b_2, double* x_1, double* x_2) {
    const int m = n_Row, n = n_Col;
    std::vector<double> d0(d, d + n), b10(b_1, b_1 + n), b20(b_2, b_2 + m);
    const long long before = help_ref_nrm2_calls;
    const int rc = help_ref_inner_solve(d, b_1, b_2, x_1, x_2);
    const int64_t iters = (int64_t)(help_ref_nrm2_calls - before - 2);
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
