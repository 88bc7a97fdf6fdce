// Impec2D CPU oracle -- TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Linear solvers standing in for HYPRE 2.8.0b (PCG + SMG, src/MGSolver.cpp:594-629), which
// is not available: a banded LU with iterative refinement (small grids, machine precision)
// and a CPU geometric multigrid (large grids, the timed CPU baseline).  Both solve exactly
// the discrete system the reference assembles; only the iteration differs.  Also the
// IMPES driver loop and the reference's two convergence tests.
#include "oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {
const int OFF[9][2] = {{0, 0}, {-1, 0}, {-1, -1}, {0, -1}, {1, -1}, {1, 0}, {1, 1}, {0, 1}, {-1, 1}};

// ---------------------------------------------------------------- banded LU
// Unknown ordering l = i*N2 + j; the 9-point stencil has half bandwidth N2+1.
struct Banded {
    int n, b;               // size, half bandwidth
    std::vector<double> a;  // row-major (n) x (2b+1), a[r*(2b+1) + (c - r + b)]
    double& at(int r, int c) { return a[(size_t)r * (2 * b + 1) + (c - r + b)]; }
};

bool factor(Banded& M) {  // Doolittle LU without pivoting, in place
    const int n = M.n, b = M.b;
    for (int k = 0; k < n; ++k) {
        double piv = M.at(k, k);
        if (piv == 0 || !std::isfinite(piv)) return false;
        int rmax = std::min(n - 1, k + b);
        int cmax = std::min(n - 1, k + b);
        for (int r = k + 1; r <= rmax; ++r) {
            double& lrk = M.at(r, k);
            if (lrk == 0) continue;
            lrk /= piv;
            const double l = lrk;
            double* rowr = &M.at(r, k + 1);
            const double* rowk = &M.at(k, k + 1);
            for (int c = 0; c < cmax - k; ++c) rowr[c] -= l * rowk[c];
        }
    }
    return true;
}

void lu_solve(Banded& M, std::vector<double>& x) {
    const int n = M.n, b = M.b;
    for (int r = 0; r < n; ++r) {
        double s = x[r];
        for (int c = std::max(0, r - b); c < r; ++c) s -= M.at(r, c) * x[c];
        x[r] = s;
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = x[r];
        for (int c = r + 1; c <= std::min(n - 1, r + b); ++c) s -= M.at(r, c) * x[c];
        x[r] = s / M.at(r, r);
    }
}

// ---------------------------------------------------------------- CPU multigrid
// Levels hold explicit (folded) 9-point stencils.  Coarse operators: Galerkin product with
// piecewise-constant 2x2 aggregation, scaled by 1/2 (equal to rediscretisation with averaged
// face coefficients for the 5-point operator).  Smoother: 4-colour Gauss-Seidel.  Transfer:
// summed restriction, bilinear (cell-centred 9/16,3/16,3/16,1/16) prolongation.
struct Level {
    int n1, n2;
    std::vector<double> A, x, b, r;
};

void build_coarse(const Level& f, Level& c) {
    c.n1 = (f.n1 + 1) / 2;
    c.n2 = (f.n2 + 1) / 2;
    size_t M = (size_t)c.n1 * c.n2;
    c.A.assign(M * 9, 0.0);
    c.x.assign(M, 0.0);
    c.b.assign(M, 0.0);
    c.r.assign(M, 0.0);
    for (int i = 0; i < f.n1; ++i)
        for (int j = 0; j < f.n2; ++j) {
            const double* a = &f.A[((size_t)i * f.n2 + j) * 9];
            const int I = i / 2, J = j / 2;
            double* ac = &c.A[((size_t)I * c.n2 + J) * 9];
            for (int e = 0; e < 9; ++e) {
                if (a[e] == 0) continue;
                int ii = i + OFF[e][0], jj = j + OFF[e][1];
                if (ii < 0 || ii >= f.n1 || jj < 0 || jj >= f.n2) continue;
                int dI = ii / 2 - I, dJ = jj / 2 - J;
                int ec = -1;
                for (int q = 0; q < 9; ++q)
                    if (OFF[q][0] == dI && OFF[q][1] == dJ) ec = q;
                ac[ec] += 0.5 * a[e];
            }
        }
}

void smooth4(Level& L, int sweeps, bool reverse) {
    const int n1 = L.n1, n2 = L.n2;
    for (int s = 0; s < sweeps; ++s)
        for (int cc = 0; cc < 4; ++cc) {
            int col = reverse ? 3 - cc : cc;
            int ci = col >> 1, cj = col & 1;
#pragma omp parallel for schedule(static)
            for (int i = ci; i < n1; i += 2)
                for (int j = cj; j < n2; j += 2) {
                    const double* a = &L.A[((size_t)i * n2 + j) * 9];
                    double sum = L.b[(size_t)i * n2 + j];
                    for (int e = 1; e < 9; ++e) {
                        int ii = i + OFF[e][0], jj = j + OFF[e][1];
                        if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
                        sum -= a[e] * L.x[(size_t)ii * n2 + jj];
                    }
                    L.x[(size_t)i * n2 + j] = sum / a[0];
                }
        }
}

void residual(Level& L) {
    const int n1 = L.n1, n2 = L.n2;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n1; ++i)
        for (int j = 0; j < n2; ++j) {
            const double* a = &L.A[((size_t)i * n2 + j) * 9];
            double s = L.b[(size_t)i * n2 + j];
            for (int e = 0; e < 9; ++e) {
                int ii = i + OFF[e][0], jj = j + OFF[e][1];
                if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
                s -= a[e] * L.x[(size_t)ii * n2 + jj];
            }
            L.r[(size_t)i * n2 + j] = s;
        }
}

void restrict_sum(const Level& f, Level& c) {
    std::fill(c.b.begin(), c.b.end(), 0.0);
    for (int i = 0; i < f.n1; ++i)
        for (int j = 0; j < f.n2; ++j) c.b[(size_t)(i / 2) * c.n2 + j / 2] += f.r[(size_t)i * f.n2 + j];
}

void prolong_add(Level& f, const Level& c) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < f.n1; ++i)
        for (int j = 0; j < f.n2; ++j) {
            int I = i / 2, J = j / 2;
            int I2 = (i & 1) ? I + 1 : I - 1, J2 = (j & 1) ? J + 1 : J - 1;
            if (I2 < 0 || I2 >= c.n1) I2 = I;
            if (J2 < 0 || J2 >= c.n2) J2 = J;
            double e = 0.5625 * c.x[(size_t)I * c.n2 + J] + 0.1875 * c.x[(size_t)I2 * c.n2 + J] +
                       0.1875 * c.x[(size_t)I * c.n2 + J2] + 0.0625 * c.x[(size_t)I2 * c.n2 + J2];
            f.x[(size_t)i * f.n2 + j] += e;
        }
}

struct MG {
    std::vector<Level> L;
    Banded coarse;
    bool singular;
    void setup(int n1, int n2, const double* A9, bool sing) {
        singular = sing;
        L.clear();
        L.emplace_back();
        L[0].n1 = n1;
        L[0].n2 = n2;
        L[0].A.assign(A9, A9 + (size_t)n1 * n2 * 9);
        L[0].x.assign((size_t)n1 * n2, 0);
        L[0].b.assign((size_t)n1 * n2, 0);
        L[0].r.assign((size_t)n1 * n2, 0);
        while (L.back().n1 > 8 || L.back().n2 > 8) {
            Level c;
            build_coarse(L.back(), c);
            L.push_back(std::move(c));
        }
        Level& C = L.back();
        coarse.n = C.n1 * C.n2;
        coarse.b = C.n2 + 1;
        coarse.a.assign((size_t)coarse.n * (2 * coarse.b + 1), 0.0);
        for (int i = 0; i < C.n1; ++i)
            for (int j = 0; j < C.n2; ++j) {
                int r = i * C.n2 + j;
                for (int e = 0; e < 9; ++e) {
                    int ii = i + OFF[e][0], jj = j + OFF[e][1];
                    if (ii < 0 || ii >= C.n1 || jj < 0 || jj >= C.n2) continue;
                    coarse.at(r, ii * C.n2 + jj) = C.A[(size_t)r * 9 + e];
                }
            }
        if (singular) {  // fix the constant null space at the coarsest level: pin unknown 0
            for (int c = 0; c <= std::min(coarse.n - 1, coarse.b); ++c) coarse.at(0, c) = 0;
            for (int r = 1; r <= std::min(coarse.n - 1, coarse.b); ++r) coarse.at(r, 0) = 0;
            coarse.at(0, 0) = 1;
        }
        factor(coarse);
    }
    void cycle(int l) {
        Level& F = L[l];
        if (l == (int)L.size() - 1) {
            std::vector<double> x(F.b);
            if (singular) x[0] = 0;
            lu_solve(coarse, x);
            if (singular) {
                double m = 0;
                for (double v : x) m += v;
                m /= x.size();
                for (double& v : x) v -= m;
            }
            F.x = x;
            return;
        }
        smooth4(F, 2, false);
        residual(F);
        Level& C = L[l + 1];
        restrict_sum(F, C);
        std::fill(C.x.begin(), C.x.end(), 0.0);
        cycle(l + 1);
        prolong_add(F, C);
        smooth4(F, 2, true);
    }
};

double norm2(const std::vector<double>& v) {
    long double s = 0;
    for (double x : v) s += (long double)x * x;
    return (double)sqrtl(s);
}

}  // namespace

extern "C" {

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// Threads of the oracle's OpenMP loops from now on (the CPU baseline's 1-thread and all-core
// runs in one process); returns the previous count.
int or_set_num_threads(int n) {
#ifdef _OPENMP
    const int prev = omp_get_max_threads();
    if (n > 0) omp_set_num_threads(n);
    return prev;
#else
    (void)n;
    return 1;
#endif
}

int or_solve_banded(const or_params* P, const double* A9, const double* b, double* x) {
    const int N1 = P->N1, N2 = P->N2, n = N1 * N2;
    Banded M;
    M.n = n;
    M.b = N2 + 1;
    M.a.assign((size_t)n * (2 * M.b + 1), 0.0);
    for (int i = 0; i < N1; ++i)
        for (int j = 0; j < N2; ++j) {
            int r = i * N2 + j;
            for (int e = 0; e < 9; ++e) {
                int ii = i + OFF[e][0], jj = j + OFF[e][1];
                if (ii < 0 || ii >= N1 || jj < 0 || jj >= N2) continue;
                M.at(r, ii * N2 + jj) = A9[(size_t)r * 9 + e];
            }
        }
    if (!factor(M)) return 1;
    std::vector<double> sol(b, b + n), res((size_t)n);
    lu_solve(M, sol);
    for (int it = 0; it < 3; ++it) {  // iterative refinement with long-double residuals
        for (int i = 0; i < N1; ++i)
            for (int j = 0; j < N2; ++j) {
                long double s = b[(size_t)i * N2 + j];
                const double* a = A9 + ((size_t)i * N2 + j) * 9;
                for (int e = 0; e < 9; ++e) {
                    int ii = i + OFF[e][0], jj = j + OFF[e][1];
                    if (ii < 0 || ii >= N1 || jj < 0 || jj >= N2) continue;
                    s -= (long double)a[e] * sol[(size_t)ii * N2 + jj];
                }
                res[(size_t)i * N2 + j] = (double)s;
            }
        lu_solve(M, res);
        for (int k = 0; k < n; ++k) sol[k] += res[k];
    }
    std::copy(sol.begin(), sol.end(), x);
    return 0;
}

// Multigrid on a folded 9-point system.  With pin_i >= 0 the matrix is the Neumann operator
// (zero row sums) and the reference's pinned system is solved as: compatible singular
// Neumann solve, then a constant shift so that x(pin) = pin_value.  The relative residual is
// measured on the reference's pinned system: the pinned row has residual zero after the shift.
int or_mg_solve(const or_params* P, const double* A9, const double* b, double* x, double tol,
                int max_cycles, int* cycles, double* relres, int pin_i, int pin_j, double pin_value) {
    const int N1 = P->N1, N2 = P->N2;
    const size_t n = (size_t)N1 * N2;
    const bool singular = pin_i >= 0;
    const size_t pin = singular ? (size_t)pin_i * N2 + pin_j : 0;
    MG mg;
    mg.setup(N1, N2, A9, singular);
    Level& F = mg.L[0];
    std::copy(b, b + n, F.b.begin());
    double bnorm = norm2(F.b);
    if (singular) {  // compatible right-hand side: the pinned entry balances the others
        long double s = 0;
        for (size_t k = 0; k < n; ++k)
            if (k != pin) s += F.b[k];
        F.b[pin] = (double)(-s);
    }
    std::copy(x, x + n, F.x.begin());
    auto rel = [&]() {
        residual(F);
        if (singular) F.r[pin] = 0;
        double r = norm2(F.r);
        return bnorm > 0 ? r / bnorm : r;
    };
    double rr = rel();
    int k = 0;
    while (rr > tol && k < max_cycles) {
        mg.cycle(0);
        ++k;
        rr = rel();
    }
    if (singular) {
        double shift = pin_value - F.x[pin];
        for (size_t q = 0; q < n; ++q) F.x[q] += shift;
    }
    std::copy(F.x.begin(), F.x.end(), x);
    if (cycles) *cycles = k;
    if (relres) *relres = rr;
    return (rr <= tol) ? 0 : 2;
}

// Solve_Elliptic_cc_to_c (src/MGSolver.cpp:223-248).  method 0: banded LU, 1: multigrid.
int or_pressure_solve(const or_params* P, const double* c, const double* q, double* p, int method,
                      double tol, int* its, double* relres) {
    const int N1 = P->N1, N2 = P->N2, g = P->g, w = N2 + 2 * g;
    const size_t n = (size_t)N1 * N2;
    std::vector<double> A(n * 9), b(n), x(n, 0.0);
    or_pressure_rhs(P, q, b.data());
    int rc = 0;
    if (method == 0 || P->stype == OR_HORIZONTAL) {
        or_pressure_matrix(P, c, A.data());
        rc = or_solve_banded(P, A.data(), b.data(), x.data());
        if (its) *its = 1;
        if (relres) *relres = or_relres9(P, A.data(), x.data(), b.data());
    } else {
        or_pressure_matrix(P, c, A.data());
        const double kappa_over_dA = A[((size_t)1 * N2 + 1) * 9];
        const double pin_value = b[(size_t)1 * N2 + 1] / kappa_over_dA;
        or_pressure_matrix_neumann(P, c, A.data());
        rc = or_mg_solve(P, A.data(), b.data(), x.data(), tol, 200, its, nullptr, 1, 1, pin_value);
        or_pressure_matrix(P, c, A.data());
        if (relres) *relres = or_relres9(P, A.data(), x.data(), b.data());
    }
    for (int i = 0; i < N1; ++i)
        for (int j = 0; j < N2; ++j) p[(size_t)(i + g) * w + (j + g)] = x[(size_t)i * N2 + j];
    return rc;
}

// Solve_Parabolic_cc_to_c (src/MGSolver.cpp:952-976): c interior <- (CN matrix)^-1 rhs.
int or_cn_solve(const or_params* P, double* c, const double* v, double dt, int method, double tol,
                int* its, double* relres) {
    const int N1 = P->N1, N2 = P->N2, g = P->g, w = N2 + 2 * g;
    const size_t n = (size_t)N1 * N2;
    std::vector<double> A(n * 9), b(n), x(n, 0.0);
    or_cn_matrix(P, v, dt, A.data());
    or_cn_rhs(P, c, v, dt, b.data());
    int rc;
    if (method == 0) {
        rc = or_solve_banded(P, A.data(), b.data(), x.data());
        if (its) *its = 1;
    } else {
        for (int i = 0; i < N1; ++i)
            for (int j = 0; j < N2; ++j) x[(size_t)i * N2 + j] = c[(size_t)(i + g) * w + (j + g)];
        rc = or_mg_solve(P, A.data(), b.data(), x.data(), tol, 200, its, nullptr, -1, -1, 0.0);
    }
    if (relres) *relres = or_relres9(P, A.data(), x.data(), b.data());
    for (int i = 0; i < N1; ++i)
        for (int j = 0; j < N2; ++j) c[(size_t)(i + g) * w + (j + g)] = x[(size_t)i * N2 + j];
    return rc;
}

static void fill_boundaries(const or_params* P, double* c) {
    if (P->is_test)
        or_fill_scalar_periodic(P, c);
    else
        or_fill_scalar_neumann(P, c);
}

// HyperbolicSplitSolver::Solve with SPLIT2ND (src/HyperbolicSplitSolver.cpp:162-198).
// solver: 0 banded LU, 1 multigrid for the Crank-Nicolson systems.
int or_hyperbolic_solve(const or_params* P, double* c, const double* v, const double* q, double dt,
                        int* prev_first_sweep, double* outflux, int solver) {
    int rc = 0;
    *outflux += fabs(or_tr_integrate(P, c, q, 0.5 * dt));
    fill_boundaries(P, c);
    if (P->diffusion) rc |= or_cn_solve(P, c, v, 0.5 * dt, solver, P->para_eps, nullptr, nullptr);
    or_advect_split(P, c, v, dt, prev_first_sweep);
    *outflux += fabs(or_tr_integrate(P, c, q, 0.5 * dt));
    fill_boundaries(P, c);
    if (P->diffusion) rc |= or_cn_solve(P, c, v, 0.5 * dt, solver, P->para_eps, nullptr, nullptr);
    return rc;
}

// One pass of the loop body in Impec2DSolver::Solve (src/Impec2DSolver.cpp:339-415).
int or_impes_step(const or_params* P, or_state* S, double* c, double* p, double* v, const double* q,
                  const double* times, int ntimes, int* tidx, int solver, double tol) {
    S->counter++;
    fill_boundaries(P, c);
    int its = 0;
    double rr = 0;
    int rc = or_pressure_solve(P, c, q, p, solver, tol, &its, &rr);
    S->its = its;
    S->relres = rr;
    or_calc_velocities(P, p, v, c);
    double dt = or_max_stable_dt(P, v);
    if (times && *tidx < ntimes && S->t + dt >= times[*tidx]) {
        dt = times[*tidx] - S->t;
        (*tidx)++;
    }
    rc |= or_hyperbolic_solve(P, c, v, q, dt, &S->prev_first_sweep, &S->total_outflux, solver);
    S->t += dt;
    S->dt = dt;
    S->mass_err = or_mass_error(P, c, S->t, S->total_outflux);
    S->vel_err = or_velocity_boundary_error(P, v);
    S->div_err = or_divergence_error(P, v, q);
    return rc;
}

// EllipticSolver::TestNeumann, one level (src/EllipticSolver.cpp:183-291): L1 errors of p, u, v.
int or_elliptic_test(const or_params* P, double* errs3) {
    const int N1 = P->N1, N2 = P->N2, g = P->g;
    const double dx = (P->x_ub - P->x_lb) / N1, dy = (P->y_ub - P->y_lb) / N2;
    const size_t ns = (size_t)(N1 + 2 * g) * (N2 + 2 * g), nv = (size_t)(N1 + 1 + 2 * g) * (N2 + 1 + 2 * g) * 2;
    std::vector<double> c(ns, 0.0), p(ns, 0.0), pex(ns, 0.0), v(nv, 0.0), vex(nv, 0.0), q((size_t)N1 * N2);
    const int w = N2 + 2 * g, wv = N2 + 1 + 2 * g;
    auto S = [&](std::vector<double>& a, int i, int j) -> double& { return a[(size_t)(i + g) * w + (j + g)]; };
    auto V = [&](std::vector<double>& a, int i, int j, int k) -> double& {
        return a[((size_t)(i + g) * wv + (j + g)) * 2 + k];
    };
    auto K11 = [&](double x, double y) {
        switch (P->testno) { case 2: return exp(-0.3 * x); case 3: case 4: return 2. + sin(2. * x) * sin(y); default: return 1.; }
    };
    auto K22 = [&](double x, double y) {
        switch (P->testno) { case 2: return exp(-0.3 * y); case 3: return 2. + sin(2. * x) * sin(y); case 4: return 2. + sin(x) * sin(2. * y); default: return 1.; }
    };
    auto qT = [&](double x, double y) {
        double mr = P->mu_res;
        switch (P->testno) {
            case 1: return 2. / mr * cos(x) * cos(y);
            case 2: { double a1 = exp(-0.3 * x), a2 = exp(-0.3 * y), a1x = -0.3 * exp(-0.3 * x), a2y = -0.3 * exp(-0.3 * y);
                      return 1. / mr * ((a1 + a2) * cos(x) * cos(y) + a1x * sin(x) * cos(y) + a2y * cos(x) * sin(y)); }
            case 3: { double a1 = 2. + sin(2. * x) * sin(y), a2 = 2. + sin(2. * x) * sin(y), a1x = 2. * cos(2. * x) * sin(y), a2y = cos(y) * sin(2. * x);
                      return 1. / mr * ((a1 + a2) * cos(x) * cos(y) + a1x * sin(x) * cos(y) + a2y * cos(x) * sin(y)); }
            default: { double a1 = 2. + sin(2. * x) * sin(y), a2 = 2. + sin(x) * sin(2. * y), a1x = 2. * cos(2. * x) * sin(y), a2y = 2. * cos(2. * y) * sin(x);
                       return 1. / mr * ((a1 + a2) * cos(x) * cos(y) + a1x * sin(x) * cos(y) + a2y * cos(x) * sin(y)); }
        }
    };
    // InitializeEllipticNeumannTest (src/EllipticSolver.cpp:357-410)
    for (int i = 0; i <= N1; i++)
        for (int j = 0; j < N2; j++) {
            double x = P->x_lb + i * dx, y = P->y_lb + (j + 0.5) * dy;
            V(vex, i, j, 0) = K11(x, y) / P->mu_res * sin(x) * cos(y);
        }
    for (int i = 0; i < N1; i++)
        for (int j = 0; j <= N2; j++) {
            double x = P->x_lb + (i + 0.5) * dx, y = P->y_lb + j * dy;
            V(vex, i, j, 1) = K22(x, y) / P->mu_res * cos(x) * sin(y);
        }
    for (int i = 0; i < N1; i++)
        for (int j = 0; j < N2; j++) {
            double x = P->x_lb + (i + 0.5) * dx, y = P->y_lb + (j + 0.5) * dy;
            S(pex, i, j) = cos(x) * cos(y);
            q[(size_t)i * N2 + j] = qT(x, y);
        }
    or_fill_scalar_neumann(P, c.data());
    int its;
    double rr;
    int rc = or_pressure_solve(P, c.data(), q.data(), p.data(), 0, 1e-14, &its, &rr);
    or_calc_velocities(P, p.data(), v.data(), c.data());
    double ps = 0, us = 0, vs = 0;
    for (int i = 0; i < N1; i++)
        for (int j = 0; j < N2; j++) ps += fabs(S(p, i, j) - S(pex, i, j));
    for (int i = 0; i <= N1; i++)
        for (int j = 0; j < N2; j++) us += fabs(V(vex, i, j, 0) - V(v, i, j, 0));
    for (int i = 0; i < N1; i++)
        for (int j = 0; j <= N2; j++) vs += fabs(V(vex, i, j, 1) - V(v, i, j, 1));
    errs3[0] = ps * dx * dy;
    errs3[1] = us * dx * dy;
    errs3[2] = vs * dx * dy;
    return rc;
}

}  // extern "C"
