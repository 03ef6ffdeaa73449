// Test oracle: runs the reference's own dependent-row presolve
// (Presolve_Lindep.cpp with its vendored LUSOL; switched off inside the
// reference program, PRESOLVE_LINDEP = 0 at LP.h:72) on one MPS file, after
// the reference's own MPS reader, crushing and presolve set-up -- the steps
// Main.cpp:43-85 and Presolve.cpp:1252-1256 take before it.  The last line
// printed is JSON: rows after crushing, dependent rows found (empty ones
// included), LP status (0 ok, 1 primal infeasible), the presolve's own wall
// time, and the disabled rows.
#include <chrono>
#include <cstdio>
#include <cstring>

#include "LP.h"
#include "Presolve.h"

void Presolve_Init();   // Presolve.cpp:77
extern int Count_LDP;   // Presolve_Lindep.cpp:24

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s file.mps\n", argv[0]);
        return 2;
    }
    if (Prog_Init()) return 3;
    std::strncpy(Filename, argv[1], MAX_FILENAME - 1);
    if (MPS_ReadFile()) return 4;
    if (CRUSH_Main()) return 5;
    if (LP_Status != LP_STATUS_OK) {
        std::printf("{\"rows\": %d, \"dependent\": -1, \"status\": %d, \"disabled\": []}\n", n_Row, LP_Status);
        return 0;
    }
    Presolve_Init();
    const auto t0 = std::chrono::steady_clock::now();
    Presolve_Linear_Dependent_Main();
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("{\"rows\": %d, \"dependent\": %d, \"status\": %d, \"seconds\": %.6f, \"disabled\": [", n_Row,
                Count_LDP, LP_Status, secs);
    bool first = true;
    for (int i = 0; i < n_Row; ++i)
        if (Row_Disable[i]) {
            std::printf(first ? "%d" : ", %d", i);
            first = false;
        }
    std::printf("]}\n");
    return 0;
}
