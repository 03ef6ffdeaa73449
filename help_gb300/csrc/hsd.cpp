// Homogeneous self-dual interior-point driver: the caller of the
// normal-equations boundary, restated from the reference's HSDSolver.cpp so
// the backend can be driven end to end (and timed) where the reference
// program itself is not available.  It calls the backend only through the
// four boundary operations (help_ne_backend), exactly where HSD_Main /
// HSD_Solving call LinearEquation_Construct / RenewLinearEquation /
// SolveLinearEquation / LinearEquation_Destruct.
//
// Scope: standard-form LPs whose columns all have lower bound 0 and no upper
// bound (n_LB = n, n_UB = n_FR = 0 in the reference's column classes,
// Presolve.cpp:1101-1140) -- every instance family in help_lp.h is of that
// form once its inequality rows carry slack columns.  The reference's
// upper-bound and free-variable terms vanish identically for such LPs; the
// arithmetic that remains follows HSDSolver.cpp operation by operation (loop
// orders included) so the iterates match the reference program's.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/help_lp.h"
#include "guard.h"

namespace {

// LP.h:82-91
const double STEPSIZE_GAMMA = 0.99995;
const double STEPSIZE_BETA = 1e-8;
const double Mu_Tolerance = 1e-12;
const double Infeasibility_Tolerance = 1e-8;
const double Variable_Tolerance = 1e-12;
// LP.h:163-167
const int HSD_STATUS_OK = 0;
const int HSD_STATUS_STALLED = 1;
const int HSD_STATUS_ITER_LIMIT = 2;
const int HSD_STATUS_UNKNOWN_ERROR = 3;

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Helper.cpp:48-55
double DotProduct(int n, const double* a, const double* b) {
    double Ret = 0;
    for (int i = 0; i < n; i++) Ret += a[i] * b[i];
    return Ret;
}

// Helper.cpp:83-104
void SetScaledVector(int n, double alpha, const double* src, double* dest) {
    if (alpha == 1) {
        for (int i = 0; i < n; i++) dest[i] = src[i];
    } else if (alpha == -1) {
        for (int i = 0; i < n; i++) dest[i] = -src[i];
    } else if (alpha == 0) {
        for (int i = 0; i < n; i++) dest[i] = 0;
    } else {
        for (int i = 0; i < n; i++) dest[i] = alpha * src[i];
    }
}

struct Hsd {
    const help_lp* lp;
    const help_ne_backend* be;
    const help_hsd_options* opt;
    int m, n;
    std::vector<double> x, y, z, D, r_p, r_d;
    double tau = 1, kappa = 1, rho = 1, inf0 = 1;
    double sum_r_norm = 0, primal_obj = 0, dual_obj = 0, comp_gap = 0, relative_gap = 0;
    double primal_infeas = 0, dual_infeas = 0, infe = 0, D_g = 0, r_g = 0, mu = 0, rfval = 0;
    int status = HSD_STATUS_OK;
    std::vector<double> hat_r_xz, dx, dy, dz, dx_b, dy_b, dz_b;
    double hat_r_tk = 0, dtau = 0, dkappa = 0;
    std::vector<double> Dir_p, Dir_q, Dir_u, Dir_v, Dir_RHS1, Dir_RHS2, SLE_RHS1, SLE_RHS2, LEBOT_RHS1, LEBOT_RHS2;
    std::vector<double> SLE2_RHS1, SLE2_RHS2;  // the second system of a paired solve (backend solve2)
    std::vector<double> masked;  // hrxz where x < z, for the device product
    double backend_s = 0;
    int solves = 0, renews = 0;
    int be_error = 0;

    // Helper.cpp:110-152 over the column lists (CSC keeps the same order),
    // or the backend's device copy of A when it offers one
    void ATimes(int transpose, int sign, const double* v, double* dest) {
        if (be->matvec) {
            const double t = now_s();
            if (be->matvec(be->ctx, transpose, sign, v, dest) != 0) be_error = 1;
            backend_s += now_s() - t;
            return;
        }
        const int32_t* cp = lp->col_ptr;
        const int32_t* ri = lp->row_ind;
        const double* av = lp->val;
        if (!transpose) {
            for (int Col = 0; Col < n; Col++) {
                const double vCol = v[Col];
                if (sign == 1)
                    for (int j = cp[Col]; j < cp[Col + 1]; j++) dest[ri[j]] += av[j] * vCol;
                else
                    for (int j = cp[Col]; j < cp[Col + 1]; j++) dest[ri[j]] -= av[j] * vCol;
            }
        } else {
            for (int Col = 0; Col < n; Col++) {
                double destCol = dest[Col];
                if (sign == 1)
                    for (int j = cp[Col]; j < cp[Col + 1]; j++) destCol += av[j] * v[ri[j]];
                else
                    for (int j = cp[Col]; j < cp[Col + 1]; j++) destCol -= av[j] * v[ri[j]];
                dest[Col] = destCol;
            }
        }
    }

    void Renew() {
        const double t = now_s();
        if (be->renew(be->ctx, D.data()) != 0) be_error = 1;
        backend_s += now_s() - t;
        renews++;
    }
    void Solve(const double* b1, const double* b2, double* x1, double* x2) {
        const double t = now_s();
        if (be->solve(be->ctx, D.data(), b1, b2, x1, x2) != 0) be_error = 1;
        backend_s += now_s() - t;
        solves++;
    }
    void Solve2(const double* b1a, const double* b2a, double* x1a, double* x2a, const double* b1b, const double* b2b,
                double* x1b, double* x2b) {
        const double t = now_s();
        if (be->solve2(be->ctx, D.data(), b1a, b2a, x1a, x2a, b1b, b2b, x1b, x2b) != 0) be_error = 1;
        backend_s += now_s() - t;
        solves += 2;
    }

    // HSDSolver.cpp:53-150
    void CalcNewtonParameters() {
        const double* c = lp->c;
        const double* b = lp->b;
        double xz_min = tau * kappa;
        double xz_sum = xz_min;
        for (int i = 0; i < n; i++) {
            D[i] = z[i] / x[i];
            const double tmp = z[i] * x[i];
            xz_min = std::min(xz_min, tmp);
            xz_sum += tmp;
            if (D[i] <= 0.0) {
                status = HSD_STATUS_STALLED;
                if (opt->verbose) std::printf("HSD_Calc_Newton_Parameters: Negative Iterate.\n");
                return;
            }
        }
        const double Tmp = 0;
        D_g = kappa / tau + rho * Tmp / (tau * tau);
        mu = xz_sum / (1.0 + n);
        rfval = (1.0 + n) * xz_min / xz_sum;
        SetScaledVector(m, tau, b, r_p.data());
        ATimes(0, -1, x.data(), r_p.data());
        for (int i = 0; i < n; i++) r_d[i] = z[i] - c[i] * tau;
        ATimes(1, 1, y.data(), r_d.data());
        const double cTx = DotProduct(n, c, x.data());
        const double bTy = DotProduct(m, b, y.data()) + 0.0;
        r_g = kappa + cTx - bTy;
        const double rp2 = DotProduct(m, r_p.data(), r_p.data());
        const double rd2 = DotProduct(n, r_d.data(), r_d.data());
        const double rg2 = r_g * r_g;
        sum_r_norm = rp2 + rd2 + rg2;
        primal_obj = 0.0 + cTx / tau;
        dual_obj = 0.0 + bTy / tau;
        comp_gap = xz_sum;
        relative_gap = std::fabs(primal_obj - dual_obj) / (1.0 + std::fabs(dual_obj));
        primal_infeas = std::sqrt(rp2) / (tau + std::sqrt(DotProduct(n, x.data(), x.data())));
        dual_infeas = std::sqrt(rd2) /
                      (tau + std::sqrt(DotProduct(n, z.data(), z.data()) + 0.0 + 0.0 + DotProduct(m, y.data(), y.data())));
        infe = tau / (kappa * inf0);
    }

    // HSDSolver.cpp:156-208 (no upper-bounded columns)
    void SolveLE(const double* s, const double* t, double* p, double* q) {
        for (int i = 0; i < n; i++) SLE_RHS1[i] = s[i];
        for (int i = 0; i < m; i++) SLE_RHS2[i] = t[i];
        Solve(SLE_RHS1.data(), SLE_RHS2.data(), p, q);
        for (int i = 0; i < m; i++) q[i] = -q[i];
    }
    // Two SolveLE at once (backend solve2): each system as SolveLE does it
    void SolveLE2(const double* sa, const double* ta, double* pa, double* qa, const double* sb, const double* tb,
                  double* pb, double* qb) {
        for (int i = 0; i < n; i++) SLE_RHS1[i] = sa[i];
        for (int i = 0; i < m; i++) SLE_RHS2[i] = ta[i];
        for (int i = 0; i < n; i++) SLE2_RHS1[i] = sb[i];
        for (int i = 0; i < m; i++) SLE2_RHS2[i] = tb[i];
        Solve2(SLE_RHS1.data(), SLE_RHS2.data(), pa, qa, SLE2_RHS1.data(), SLE2_RHS2.data(), pb, qb);
        for (int i = 0; i < m; i++) qa[i] = -qa[i];
        for (int i = 0; i < m; i++) qb[i] = -qb[i];
    }

    // HSDSolver.cpp:212-220
    double MixDots(const double* p, const double* q) const {
        double Ret = -DotProduct(n, lp->c, p);
        Ret += DotProduct(m, lp->b, q) + 0.0;
        return Ret;
    }

    // HSDSolver.cpp:226-261
    double LinearEquationBottom() {
        for (int i = 0; i < n; i++) LEBOT_RHS1[i] = lp->c[i];
        for (int i = 0; i < m; i++) LEBOT_RHS2[i] = -lp->b[i];
        SolveLE(LEBOT_RHS1.data(), LEBOT_RHS2.data(), Dir_p.data(), Dir_q.data());
        return MixDots(Dir_p.data(), Dir_q.data());
    }

    // HSDSolver.cpp:281-473, in three parts so that a backend with solve2 can
    // take the direction's system together with the bottom one: the
    // right-hand side (DirRhs, returns UP), the solve, the rest (DirFinish).
    int SearchDirection(double eta, double DOT, double* hrxz, double hrtk, double* ddx, double& ddtau, double* ddy,
                        double* ddz, double& ddkappa) {
        const double UP = DirRhs(eta, hrxz, hrtk);
        SolveLE(Dir_RHS1.data(), Dir_RHS2.data(), Dir_u.data(), Dir_v.data());
        return DirFinish(eta, DOT, hrxz, hrtk, UP, ddx, ddtau, ddy, ddz, ddkappa);
    }

    // LinearEquationBottom and the first SearchDirection of an iteration.
    // Neither right-hand side depends on the other system's solution, so with
    // the backend's solve2 both systems are solved at once; every value the
    // driver computes is the same as in the sequential order.
    int BottomAndDirection(double eta, double* hrxz, double hrtk, double* ddx, double& ddtau, double* ddy,
                           double* ddz, double& ddkappa, double& DOT) {
        if (!be->solve2) {
            DOT = LinearEquationBottom();
            return SearchDirection(eta, DOT, hrxz, hrtk, ddx, ddtau, ddy, ddz, ddkappa);
        }
        for (int i = 0; i < n; i++) LEBOT_RHS1[i] = lp->c[i];
        for (int i = 0; i < m; i++) LEBOT_RHS2[i] = -lp->b[i];
        const double UP = DirRhs(eta, hrxz, hrtk);
        SolveLE2(LEBOT_RHS1.data(), LEBOT_RHS2.data(), Dir_p.data(), Dir_q.data(), Dir_RHS1.data(), Dir_RHS2.data(),
                 Dir_u.data(), Dir_v.data());
        DOT = MixDots(Dir_p.data(), Dir_q.data());
        return DirFinish(eta, DOT, hrxz, hrtk, UP, ddx, ddtau, ddy, ddz, ddkappa);
    }

    double DirRhs(double eta, double* hrxz, double hrtk) {
        const double* c = lp->c;
        SetScaledVector(n, eta, r_d.data(), Dir_RHS1.data());
        SetScaledVector(m, eta, r_p.data(), Dir_RHS2.data());
        for (int i = 0; i < n; i++) hrxz[i] /= std::max(x[i], z[i]);
        for (int i = 0; i < n; i++)
            if (x[i] >= z[i]) Dir_RHS1[i] += hrxz[i];
        if (be->matvec) {
            // the same product, A (hrxz where x < z), on the backend's copy
            // of A: a scatter over every nonzero on the host otherwise (the
            // driver's largest host cost at 10^8 nonzeros); row sums in the
            // device's order, as for the driver's other products
            for (int i = 0; i < n; i++) masked[i] = (x[i] < z[i]) ? hrxz[i] : 0.0;
            ATimes(0, -1, masked.data(), Dir_RHS2.data());
        } else {
            for (int i = 0; i < n; i++)
                if (x[i] < z[i]) {
                    for (int j = lp->col_ptr[i]; j < lp->col_ptr[i + 1]; j++)
                        Dir_RHS2[lp->row_ind[j]] -= lp->val[j] * hrxz[i];
                }
        }
        double UP = eta * r_g + hrtk / tau;
        for (int i = 0; i < n; i++)
            if (x[i] < z[i]) UP += c[i] * hrxz[i];
        return UP;
    }

    int DirFinish(double eta, double DOT, const double* hrxz, double hrtk, double UP, double* ddx, double& ddtau,
                  double* ddy, double* ddz, double& ddkappa) {
        const double* c = lp->c;
        const double* b = lp->b;
        const double DOWN = D_g - DOT;
        if (DOWN <= 1e-13)
            ddtau = 0;
        else
            ddtau = (UP - MixDots(Dir_u.data(), Dir_v.data())) / std::max(D_g, DOWN);
        for (int i = 0; i < n; i++) {
            const double Temp = Dir_u[i] - Dir_p[i] * ddtau;
            if (x[i] >= z[i]) {
                ddx[i] = Temp;
                ddz[i] = hrxz[i] - z[i] * Temp / x[i];
            } else {
                ddx[i] = hrxz[i] + Temp;
                ddz[i] = -z[i] * Temp / x[i];
            }
        }
        for (int i = 0; i < m; i++) ddy[i] = Dir_v[i] - Dir_q[i] * ddtau;
        ddkappa = (hrtk - kappa * ddtau) / tau;
        SetScaledVector(n, eta, r_d.data(), Dir_RHS1.data());
        for (int i = 0; i < n; i++) Dir_RHS1[i] += -c[i] * ddtau + ddz[i];
        ATimes(1, 1, ddy, Dir_RHS1.data());
        for (int i = 0; i < m; i++) Dir_RHS2[i] = eta * r_p[i] + b[i] * ddtau;
        ATimes(0, -1, ddx, Dir_RHS2.data());
        const double r_p_norm = DotProduct(m, Dir_RHS2.data(), Dir_RHS2.data()) + 0.0;
        const double r_d_norm = DotProduct(n, Dir_RHS1.data(), Dir_RHS1.data()) + 0.0;
        const double Tmp = 0;
        double r_g_norm = eta * r_g + ddkappa - MixDots(ddx, ddy) - rho * Tmp * ddtau / (tau * tau);
        r_g_norm = r_g_norm * r_g_norm;
        if (r_p_norm + r_d_norm <= 1e-10 || r_p_norm + r_d_norm + r_g_norm <= sum_r_norm * 0.1) return 1;
        return 0;
    }

    // HSDSolver.cpp:478-488
    double Stepsize(const double* v, const double* dv) const {
        double Ret = 1.0;
        for (int i = 0; i < n; i++)
            if (dv[i] < -Variable_Tolerance && v[i] + Ret * dv[i] < 0.0) Ret = -v[i] / dv[i];
        return Ret;
    }

    // HSDSolver.cpp:491-514
    int CheckStepsize(double alpha_p, double alpha_tau, double alpha_d, double alpha_kappa, double beta) const {
        double xz_min = (tau + alpha_tau * dtau) * (kappa + alpha_kappa * dkappa);
        double xz_sum = xz_min;
        for (int i = 0; i < n; i++) {
            const double tmp = (x[i] + alpha_p * dx[i]) * (z[i] + alpha_d * dz[i]);
            xz_min = std::min(xz_min, tmp);
            xz_sum += tmp;
        }
        const double mu_ = xz_sum / (1.0 + n);
        return (xz_min / mu_ >= beta);
    }

    // HSDSolver.cpp:521-535
    void GetStepsize(double& p_size, double& d_size) const {
        p_size = Stepsize(x.data(), dx.data());
        d_size = Stepsize(z.data(), dz.data());
        if (dtau < -Variable_Tolerance) {
            p_size = std::min(p_size, -tau / dtau);
            d_size = std::min(d_size, -tau / dtau);
        }
        if (dkappa < -Variable_Tolerance) {
            p_size = std::min(p_size, -kappa / dkappa);
            d_size = std::min(d_size, -kappa / dkappa);
        }
    }

    // HSDSolver.cpp:537-594
    void UpdateStep(double eta, double p_step, double d_step) {
        (void)eta;
        double tau_step, kappa_step;
        const int PGD = (p_step * dtau) > (d_step * dtau);
        if (PGD) {
            tau_step = d_step;
            kappa_step = p_step;
        } else {
            tau_step = p_step;
            kappa_step = d_step;
        }
        double rstep = STEPSIZE_GAMMA;
        const double threshold = std::max(std::min(std::sqrt(STEPSIZE_BETA), rfval * 0.01), STEPSIZE_BETA);
        while (!CheckStepsize(rstep * p_step, rstep * tau_step, rstep * d_step, rstep * kappa_step, threshold))
            rstep *= 0.95;
        p_step *= rstep;
        tau_step *= rstep;
        d_step *= rstep;
        kappa_step *= rstep;
        const double tau_p = tau + p_step * dtau;
        const double tau_d = tau + d_step * dtau;
        double p_factor, d_factor;
        if (PGD) {
            p_factor = tau_d / tau_p;
            d_factor = 1;
        } else {
            p_factor = 1;
            d_factor = tau_p / tau_d;
        }
        for (int i = 0; i < n; i++) {
            x[i] = (x[i] + p_step * dx[i]) * p_factor;
            z[i] = (z[i] + d_step * dz[i]) * d_factor;
        }
        for (int i = 0; i < m; i++) y[i] = (y[i] + d_step * dy[i]) * d_factor;
        tau += tau_step * dtau;
        kappa = (kappa + kappa_step * dkappa) * p_factor * d_factor;
    }

    // HSDSolver.cpp:596-717
    void GetInitPoint() {
        status = HSD_STATUS_OK;
        for (int i = 0; i < n; i++) x[i] = z[i] = 1.0;
        for (int i = 0; i < m; i++) y[i] = 0.0;
        tau = kappa = 1.0;
        const double n_All = 1.0 + n;
        const double mu_ = (DotProduct(n, x.data(), z.data()) + 0.0 + tau * kappa) / n_All;
        inf0 = tau / kappa;
        rho = 1.0;
        CalcNewtonParameters();
        if (status != HSD_STATUS_OK) return;
        Renew();
        double phi = 1.0;
        const double eta = 1.0;
        for (int i = 0; i < n; i++) hat_r_xz[i] = -x[i] * z[i] + mu_;
        hat_r_tk = -tau * kappa + mu_;
        double DOT = 0.0;
        const int Newton_Success = BottomAndDirection(eta, hat_r_xz.data(), hat_r_tk, dx.data(), dtau, dy.data(),
                                                      dz.data(), dkappa, DOT);
        double p_step = 0, d_step = 0;
        if (Newton_Success)
            GetStepsize(p_step, d_step);
        else {
            if (opt->verbose) std::printf("HSD_GetInitPoint: Warning: Inaccurate Newton Direction.\n");
            phi = 0.0;
        }
        const double gamma = 10.0;
        const double alpha_p = std::max(0.0, 1.0 - std::min(p_step, d_step)) * gamma * mu_;
        const double dmu = std::max((DotProduct(n, dx.data(), dz.data()) + 0.0 + dtau * dkappa) / n_All, 0.0);
        for (int i = 0; i < n; i++) hat_r_xz[i] = -x[i] * z[i] + alpha_p - phi * (dx[i] * dz[i] - dmu);
        hat_r_tk = -tau * kappa + alpha_p - phi * (dtau * dkappa - dmu);
        double dtau_b = 0, dkappa_b = 0;
        const int IMP_Success =
            SearchDirection(eta, DOT, hat_r_xz.data(), hat_r_tk, dx_b.data(), dtau_b, dy_b.data(), dz_b.data(), dkappa_b);
        if (!IMP_Success) {
            if (opt->verbose) std::printf("HSD_GetInitPoint: Warning: Inaccurate Improved Direction.\n");
            if (!Newton_Success) {
                if (opt->verbose)
                    std::printf("HSD_GetInitPoint: Warning: Failed to generate Newton-like starting point.\n");
                return;
            }
        } else {
            dx = dx_b;
            dy = dy_b;
            dz = dz_b;
            dtau = dtau_b;
            dkappa = dkappa_b;
            GetStepsize(p_step, d_step);
        }
        if (p_step < Variable_Tolerance && d_step < Variable_Tolerance) {
            if (opt->verbose)
                std::printf("HSD_GetInitPoint: Warning: Newton-like starting point with 0 stepsize, stop here.\n");
            return;
        }
        UpdateStep(eta, p_step, d_step);
    }

    // HSDSolver.cpp:737-867; returns the number of table rows printed.
    int Solving() {
        GetInitPoint();
        const double mu0 = (DotProduct(n, x.data(), z.data()) + 0.0 + tau * kappa) / (1.0 + n);
        mu = mu0;
        if (opt->verbose) {
            std::printf("+------+------------------+------------------+----------+----------+----------+\n");
            std::printf("| Iter |      P. Obj.     |      D. Obj.     |  Rel.Gap | P.Infeas | D.Infeas |\n");
            std::printf("+------+------------------+------------------+----------+----------+----------+\n");
        }
        int Iter;
        const double t_start = now_s();
        for (Iter = 0; Iter < opt->max_iterations; Iter++) {
            rho = std::max(mu / mu0, 1e-12);
            CalcNewtonParameters();
            if (opt->verbose) {
                std::printf("| %4d | %16.7le | %16.7le | %8.1le | %8.1le | %8.1le |\n", Iter, primal_obj, dual_obj,
                            relative_gap, primal_infeas, dual_infeas);
                std::printf("+------+------------------+------------------+----------+----------+----------+\n");
                std::fflush(stdout);
            }
            if (opt->on_iter) {
                const double s6[6] = {primal_obj, dual_obj, relative_gap, primal_infeas, dual_infeas, mu};
                opt->on_iter(opt->user, Iter, s6);
            }
            if (status != HSD_STATUS_OK || (mu <= Mu_Tolerance * mu0 && infe < Infeasibility_Tolerance) ||
                (relative_gap <= opt->gap_tol && primal_infeas <= opt->pinf_tol && dual_infeas <= opt->dinf_tol))
                break;
            if (be_error) break;
            if (opt->max_seconds > 0.0 && now_s() - t_start > opt->max_seconds) {
                status = HSD_STATUS_ITER_LIMIT;  // a wall-clock cap the reference lacks
                break;
            }
            Renew();
            const double phi = 1.0;
            double eta = 1.0;
            for (int i = 0; i < n; i++) hat_r_xz[i] = -x[i] * z[i];
            hat_r_tk = -tau * kappa;
            double DOT = 0.0;
            const int Newton_Success = BottomAndDirection(eta, hat_r_xz.data(), hat_r_tk, dx.data(), dtau, dy.data(),
                                                          dz.data(), dkappa, DOT);
            double p_step = 0.0, d_step = 0.0, gamma;
            if (Newton_Success) {
                GetStepsize(p_step, d_step);
                double new_mu = (tau + p_step * dtau) * (kappa + d_step * dkappa);
                for (int i = 0; i < n; i++) new_mu += (x[i] + p_step * dx[i]) * (z[i] + d_step * dz[i]);
                new_mu /= 1.0 + n;
                gamma = new_mu / mu;
                gamma = std::min(gamma * gamma * gamma, 0.2 * std::min(gamma, 1.0));
                if (mu < 1e-3) gamma = std::max(gamma, mu);
                gamma = std::max(1e-6, gamma);
            } else {
                if (opt->verbose) std::printf("HSD_Solving: Inaccurate Newton Direction, Stalled.\n");
                status = HSD_STATUS_STALLED;
                break;
            }
            eta = 1.0 - gamma;
            const double alpha_p = gamma * mu;
            const double dmu = std::max((DotProduct(n, dx.data(), dz.data()) + 0.0 + dtau * dkappa) / (1.0 + n), 0.0);
            for (int i = 0; i < n; i++) hat_r_xz[i] = -x[i] * z[i] + alpha_p - phi * (dx[i] * dz[i] - dmu);
            hat_r_tk = -tau * kappa + alpha_p - phi * (dtau * dkappa - dmu);
            double dtau_b = 0, dkappa_b = 0;
            const int IMP_Success = SearchDirection(eta, DOT, hat_r_xz.data(), hat_r_tk, dx_b.data(), dtau_b,
                                                    dy_b.data(), dz_b.data(), dkappa_b);
            if (IMP_Success) {
                dx = dx_b;
                dy = dy_b;
                dz = dz_b;
                dtau = dtau_b;
                dkappa = dkappa_b;
                GetStepsize(p_step, d_step);
            }
            if (p_step < Variable_Tolerance && d_step < Variable_Tolerance) {
                if (opt->verbose) std::printf("HSD_Solving: Warning: Newton-like starting point with 0 stepsize, stop here.\n");
                status = HSD_STATUS_UNKNOWN_ERROR;
                break;
            }
            UpdateStep(eta, p_step, d_step);
        }
        if (Iter >= opt->max_iterations) status = HSD_STATUS_ITER_LIMIT;
        return Iter + (Iter < opt->max_iterations ? 1 : 0);
    }
};

}  // namespace

extern "C" {

void help_hsd_default_options(help_hsd_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->max_iterations = 10000;
    o->gap_tol = 1e-8;
    o->pinf_tol = 1e-8;
    o->dinf_tol = 1e-8;
}

static int hsd_solve(const help_lp* lp, const help_ne_backend* be, const help_hsd_options* opt_in,
                     help_hsd_result* res, double* x_out, double* y_out) {
    if (!lp || !be || !res || !be->construct || !be->renew || !be->solve || !be->destruct) return -1;
    help_hsd_options dflt;
    help_hsd_default_options(&dflt);
    const help_hsd_options* opt = opt_in ? opt_in : &dflt;
    std::memset(res, 0, sizeof(*res));
    if (lp->m == 0 || lp->n == 0) return 0;  // HSDSolver.cpp:871-875
    const double t0 = now_s();
    Hsd h;
    h.lp = lp;
    h.be = be;
    h.opt = opt;
    h.m = lp->m;
    h.n = lp->n;
    const size_t m = lp->m, n = lp->n;
    for (auto* v : {&h.x, &h.z, &h.D, &h.r_d, &h.hat_r_xz, &h.dx, &h.dz, &h.dx_b, &h.dz_b, &h.Dir_p, &h.Dir_u,
                    &h.Dir_RHS1, &h.SLE_RHS1, &h.LEBOT_RHS1})
        v->assign(n, 0.0);
    if (be->matvec) h.masked.assign(n, 0.0);
    if (be->solve2) {
        h.SLE2_RHS1.assign(n, 0.0);
        h.SLE2_RHS2.assign(m, 0.0);
    }
    for (auto* v : {&h.y, &h.r_p, &h.dy, &h.dy_b, &h.Dir_q, &h.Dir_v, &h.Dir_RHS2, &h.SLE_RHS2, &h.LEBOT_RHS2})
        v->assign(m, 0.0);
    double tb = now_s();
    int rc = be->construct(be->ctx, lp->m, lp->n, lp->col_ptr, lp->row_ind, lp->val);
    h.backend_s += now_s() - tb;
    if (rc != 0) return rc;
    const int rows = h.Solving();
    tb = now_s();
    be->destruct(be->ctx);
    h.backend_s += now_s() - tb;
    res->status = h.status;
    res->iterations = rows;
    res->solves = h.solves;
    res->renews = h.renews;
    res->primal_obj = h.primal_obj;
    res->dual_obj = h.dual_obj;
    res->rel_gap = h.relative_gap;
    res->primal_infeas = h.primal_infeas;
    res->dual_infeas = h.dual_infeas;
    res->tau = h.tau;
    res->kappa = h.kappa;
    res->backend_s = h.backend_s;
    res->wall_s = now_s() - t0;
    if (x_out)
        for (size_t j = 0; j < n; ++j) x_out[j] = h.x[j] / h.tau;
    if (y_out)
        for (size_t i = 0; i < m; ++i) y_out[i] = h.y[i] / h.tau;
    return h.be_error ? -2 : 0;
}

// With presolve_lindep: the dependent rows removed first, the reduced LP
// solved, y scattered back with 0 on the dropped rows (a dropped row is a
// combination of kept ones, so A^T y and b^T y are unchanged).
static int hsd_solve_presolved(const help_lp* lp, const help_ne_backend* be, const help_hsd_options* opt,
                               help_hsd_result* res, double* x_out, double* y_out) {
    if (!lp || !be || !res || lp->m <= 0 || lp->n <= 0) return hsd_solve(lp, be, opt, res, x_out, y_out);
    help_lp red;
    std::vector<int32_t> removed((size_t)lp->m, 0);
    const int rc = help_lp_remove_dependent_rows(lp, 1e-8, &red, removed.data());
    if (rc == -3) {  // b disagrees with a dependency: primal infeasible, no HSD run
        std::memset(res, 0, sizeof(*res));
        res->lp_status = 1;
        return 0;
    }
    if (rc <= 0) {  // nothing removed, or the presolve does not apply
        help_lp_free(&red);
        if (rc == -2) return -3;
        return hsd_solve(lp, be, opt, res, x_out, y_out);
    }
    std::vector<double> y_red(y_out ? (size_t)red.m : 0);
    const int r = hsd_solve(&red, be, opt, res, x_out, y_out ? y_red.data() : nullptr);
    help_lp_free(&red);
    if (y_out) {
        size_t k = 0;
        for (int32_t i = 0; i < lp->m; ++i) y_out[i] = removed[(size_t)i] ? 0.0 : y_red[k++];
    }
    res->rows_removed = rc;
    return r;
}

int help_hsd_solve(const help_lp* lp, const help_ne_backend* be, const help_hsd_options* opt_in,
                   help_hsd_result* res, double* x_out, double* y_out) {
    return c_guard(-3, [&] {
        if (opt_in && opt_in->presolve_lindep) return hsd_solve_presolved(lp, be, opt_in, res, x_out, y_out);
        return hsd_solve(lp, be, opt_in, res, x_out, y_out);
    });
}

}  // extern "C"
