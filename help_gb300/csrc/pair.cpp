// Two help_pcg contexts behind one backend table, for the HSD driver's paired
// solves (help_ne_backend.solve2 in help_lp.h; declarations in help_gpu.h).
//
// The reference's HSD iteration (HSDSolver.cpp:737-867) solves the bottom
// system (LinearEquationBottom, :226-261) and then the first search direction
// (SearchDirection, :281-473) one after the other, though neither right-hand
// side depends on the other system's solution.  The pair runs them at the
// same time: context 1 on a second host thread, context 0 on the caller's.
// Each context has its own stream and buffers, so the two CG runs overlap on
// the GPU -- on small systems two single-cluster kernels on different SMs.
// Construct and renew run on both contexts with the same arguments (renew on
// two threads as well), so each solve gives what one context gives.  With a
// model attached (the learned part) the solve slots follow the systems as on
// one context -- context 0's solves take slots 0 (bottom) and 2 (corrector),
// context 1's slot 1 (predictor) -- and before each renew context 1 receives
// context 0's bottom solution, whose features set the Schur-diagonal
// correction: every warm start, feature and correction is one context's.
#include <thread>

#include "../../include/help_gpu.h"
#include "guard.h"

struct help_pcg_pair {
    help_pcg* c[2] = {nullptr, nullptr};
};

namespace {

help_pcg_pair* as_pair(void* p) { return static_cast<help_pcg_pair*>(p); }

// f(0) on this thread and f(1) on a second one; the first nonzero code (0's first)
template <class F>
int both(F&& f) {
    int rc1 = 0;
    std::thread t([&] { rc1 = f(1); });
    const int rc0 = f(0);
    t.join();
    return rc0 ? rc0 : rc1;
}

}  // namespace

extern "C" {

int help_pcg_pair_create(const help_pcg_options* opt, help_pcg_pair** out) {
    return c_guard(HELP_E_NOMEM, [&]() -> int {
        if (!out) return HELP_E_ARG;
        *out = nullptr;
        // a warm start depends on the order of the solves, which the pair changes
        if (opt && opt->warm_start) return HELP_E_ARG;
        help_pcg_pair* p = new help_pcg_pair();
        static const int32_t slots0[2] = {0, 2}, slots1[1] = {1};
        for (int i = 0; i < 2; ++i) {
            int rc = help_pcg_create(opt, &p->c[i]);
            if (rc == HELP_OK) rc = i == 0 ? help_pcg_set_solve_slots(p->c[0], slots0, 2)
                                           : help_pcg_set_solve_slots(p->c[1], slots1, 1);
            if (rc != HELP_OK) {
                help_pcg_pair_free(p);
                return rc;
            }
        }
        *out = p;
        return HELP_OK;
    });
}

void help_pcg_pair_free(help_pcg_pair* pair) {
    if (!pair) return;
    for (help_pcg* c : pair->c)
        if (c) help_pcg_free(c);
    delete pair;
}

help_pcg* help_pcg_pair_context(help_pcg_pair* pair, int32_t which) {
    return (pair && (which == 0 || which == 1)) ? pair->c[which] : nullptr;
}

int help_pcg_pair_construct(void* pair, int32_t m, int32_t n, const int32_t* col_ptr, const int32_t* row_ind,
                            const double* val) {
    help_pcg_pair* p = as_pair(pair);
    if (!p) return HELP_E_ARG;
    return c_guard(HELP_E_NOMEM,
                   [&]() -> int { return both([&](int i) -> int { return help_pcg_construct(p->c[i], m, n, col_ptr, row_ind, val); }); });
}

int help_pcg_pair_renew(void* pair, const double* d) {
    help_pcg_pair* p = as_pair(pair);
    if (!p) return HELP_E_ARG;
    return c_guard(HELP_E_NOMEM, [&]() -> int {
        // the bottom system's solution of the renew ending now, which the next
        // renew's features read on context 1 as on context 0
        const int rc = help_pcg_share_solution(p->c[1], 0, p->c[0], 0);
        if (rc != HELP_OK) return rc;
        return both([&](int i) -> int { return help_pcg_renew(p->c[i], d); });
    });
}

int help_pcg_pair_solve(void* pair, const double* d, const double* b_1, const double* b_2, double* x_1,
                        double* x_2) {
    help_pcg_pair* p = as_pair(pair);
    if (!p) return HELP_E_ARG;
    return help_pcg_solve(p->c[0], d, b_1, b_2, x_1, x_2);
}

int help_pcg_pair_solve2(void* pair, const double* d, const double* b_1a, const double* b_2a, double* x_1a,
                         double* x_2a, const double* b_1b, const double* b_2b, double* x_1b, double* x_2b) {
    help_pcg_pair* p = as_pair(pair);
    if (!p) return HELP_E_ARG;
    return c_guard(HELP_E_NOMEM, [&]() -> int {
        return both([&](int i) -> int {
            return i == 0 ? help_pcg_solve(p->c[0], d, b_1a, b_2a, x_1a, x_2a)
                          : help_pcg_solve(p->c[1], d, b_1b, b_2b, x_1b, x_2b);
        });
    });
}

int help_pcg_pair_destruct(void* pair) {
    help_pcg_pair* p = as_pair(pair);
    if (!p) return HELP_E_ARG;
    const int rc0 = help_pcg_destruct(p->c[0]), rc1 = help_pcg_destruct(p->c[1]);
    return rc0 ? rc0 : rc1;
}

int help_pcg_pair_matvec(void* pair, int32_t transpose, int32_t sign, const double* v, double* dest) {
    help_pcg_pair* p = as_pair(pair);
    if (!p) return HELP_E_ARG;
    return help_pcg_matvec_acc(p->c[0], transpose, sign, v, dest);
}

}  // extern "C"
