/*
 * C entry points into the reference Impec2D build (oracle/_ref) -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference's own sources (src/*.cpp of pw359/Impec2D) are compiled unchanged against
 * the stand-in headers in oracle/refshim (a Blitz++ subset, libconfig++, one-rank MPI, and a
 * HYPRE whose solvers are one direct solve of the recorded system).  This file is the only
 * code of ours in that library besides the stand-ins: it opens a reference solver from a
 * .cfg, copies flat arrays in and out of the reference's Blitz arrays, and calls the
 * reference's own methods.  Layouts are the oracle's (oracle/oracle.h): scalar fields
 * (N1+2g) x (N2+2g), velocity (N1+1+2g) x (N2+1+2g) x 2, sources N1*N2, 9-point systems
 * N1*N2*9 in the HYPRE entry order C,W,SW,S,SE,E,NE,N,NW.
 *
 * The tests use it to check the oracle against the reference bit for bit, and the script
 * under tests/golden uses it to write fixtures; nothing in the engine loads it.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "HYPRE_struct_ls.h"
#include "blitz/array.h"
#include "libconfig.h++"
#include "mpi.h"

// The driver reads and calls members the reference keeps private or protected (including
// members of classes whose default access is private, hence class -> struct).  The
// reference headers use no templates, so the substitution is safe there.
#define class struct
#define private public
#define protected public
#include "EllipticSolver.h"
#include "HyperbolicSolver.h"
#include "HyperbolicSplitSolver.h"
#include "Impec2DSolver.h"
#include "MGSolver.h"
#include "MUSCLSplitSolver.h"
#include "ParallelProjector.h"
#include "SimParams.h"
#include "TRIntegrator.h"
#include "UpwindSplitSolver.h"
#include "Util.h"
#undef class
#undef private
#undef protected

// The reference leaves some SimParams members unset: ls_flagged_diff and ls_mod_diff belong to
// a section whose parsing is commented out (src/SimParams.cpp:294-309), yet the constructor
// tests them (src/SimParams.cpp:463-466).  Its own runs saw the zeros of fresh heap memory; this
// library gives every allocation made from its code zero-filled memory so that those runs are
// reproduced deterministically (the recipe links with -Bsymbolic-functions, so only this
// library's allocations come here).
void* operator new(std::size_t n) {
    void* p = std::calloc(1, n ? n : 1);
    if (!p) throw std::bad_alloc();
    return p;
}
void* operator new[](std::size_t n) {
    void* p = std::calloc(1, n ? n : 1);
    if (!p) throw std::bad_alloc();
    return p;
}
void operator delete(void* p) noexcept { std::free(p); }
void operator delete[](void* p) noexcept { std::free(p); }
void operator delete(void* p, std::size_t) noexcept { std::free(p); }
void operator delete[](void* p, std::size_t) noexcept { std::free(p); }

namespace {

struct RefCase {
    Impec2DSolver* solver = nullptr;  // owns sp, es (MGSolver), hs (MUSCL), c, p, v, q
    UpwindSplitSolver* upwind = nullptr;
    SimParams* sp() const { return solver->sp; }
    MGSolver* mg() const { return static_cast<MGSolver*>(solver->es); }
    HyperbolicSplitSolver* split(int scheme) const {
        // scheme: 0 upwind split, 4 MUSCL (the SimParams enum values)
        return scheme == 0 ? static_cast<HyperbolicSplitSolver*>(upwind)
                           : static_cast<HyperbolicSplitSolver*>(solver->hs);
    }
};

int G(const RefCase* h) { return h->sp()->c_bounds; }
int N1(const RefCase* h) { return h->sp()->N1; }
int N2(const RefCase* h) { return h->sp()->N2; }

Array2d scalar_in(const RefCase* h, const double* a) {
    const int g = G(h), n1 = N1(h) + 2 * g, n2 = N2(h) + 2 * g;
    Array2d A(n1, n2);
    A.reindexSelf(Idx2d(-g, -g));
    if (a)
        for (int i = -g; i < n1 - g; ++i)
            for (int j = -g; j < n2 - g; ++j) A(i, j) = a[(size_t)(i + g) * n2 + (j + g)];
    return A;
}
void scalar_out(const RefCase* h, const Array2d& A, double* a) {
    const int g = G(h), n1 = N1(h) + 2 * g, n2 = N2(h) + 2 * g;
    for (int i = -g; i < n1 - g; ++i)
        for (int j = -g; j < n2 - g; ++j) a[(size_t)(i + g) * n2 + (j + g)] = A(i, j);
}
Array3d vel_in(const RefCase* h, const double* v) {
    const int g = h->sp()->v_bounds, n1 = N1(h) + 1 + 2 * g, n2 = N2(h) + 1 + 2 * g;
    Array3d V(n1, n2, 2);
    V.reindexSelf(Idx3d(-g, -g, 0));
    if (v)
        for (int i = -g; i < n1 - g; ++i)
            for (int j = -g; j < n2 - g; ++j)
                for (int k = 0; k < 2; ++k) V(i, j, k) = v[((size_t)(i + g) * n2 + (j + g)) * 2 + k];
    return V;
}
void vel_out(const RefCase* h, const Array3d& V, double* v) {
    const int g = h->sp()->v_bounds, n1 = N1(h) + 1 + 2 * g, n2 = N2(h) + 1 + 2 * g;
    for (int i = -g; i < n1 - g; ++i)
        for (int j = -g; j < n2 - g; ++j)
            for (int k = 0; k < 2; ++k) v[((size_t)(i + g) * n2 + (j + g)) * 2 + k] = V(i, j, k);
}
void matrix_out(HYPRE_StructMatrix A, double* A9) {
    int lo[2], hi[2];
    const double* coef = nullptr;
    const int ne = impec_hypre_shim_matrix(A, lo, hi, &coef);
    const size_t n = (size_t)(hi[0] - lo[0] + 1) * (size_t)(hi[1] - lo[1] + 1);
    std::memcpy(A9, coef, n * ne * sizeof(double));
}
void vector_out(HYPRE_StructVector v, double* out) {
    const double* val = nullptr;
    const int n = impec_hypre_shim_vector(v, &val);
    std::memcpy(out, val, (size_t)n * sizeof(double));
}

}  // namespace

extern "C" {

/* Opens a reference solver on a .cfg: Impec2DSolver(cfg, 0, 1) (src/Impec2DSolver.cpp:67-110),
 * which parses the file, builds the MG and MUSCL solvers, sizes c, p, v and sets q. */
void* ref_open(const char* cfg) {
    RefCase* h = new RefCase();
    h->solver = new Impec2DSolver(std::string(cfg), 0, 1);
    h->upwind = new UpwindSplitSolver(h->solver->sp);
    h->upwind->AssignMGSolver(h->mg());
    return h;
}
void ref_close(void* hp) {
    RefCase* h = static_cast<RefCase*>(hp);
    delete h->upwind;
    delete h->solver;
    delete h;
}
/* N1, N2, ghost layers, and the grid spacings of the parsed parameters. */
void ref_dims(void* hp, int* n1, int* n2, int* g, double* dx, double* dy) {
    RefCase* h = static_cast<RefCase*>(hp);
    *n1 = N1(h);
    *n2 = N2(h);
    *g = G(h);
    *dx = h->sp()->dx;
    *dy = h->sp()->dy;
}
/* The source field q the constructor set (InitializeSource, src/Impec2DSolver.cpp:241-280). */
void ref_source(void* hp, double* q) {
    RefCase* h = static_cast<RefCase*>(hp);
    std::memcpy(q, h->solver->q, sizeof(double) * (size_t)h->sp()->M);
}
/* InitHorizontalFront at time t (src/Util.cpp:607-639). */
void ref_horizontal_source(void* hp, double* q, double t) {
    RefCase* h = static_cast<RefCase*>(hp);
    InitHorizontalFront(h->sp(), q, t);
}
double ref_exact_vol_frac_circle(double x1, double y1, double r, double dx, double dy) {
    return ExactVolFracCircle(x1, y1, r, dx, dy);
}

/* ---- ghost fills (src/Util.cpp:215-438) ---- */
void ref_fill_scalar_neumann(void* hp, double* a) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d A = scalar_in(h, a);
    FillGhostCellsNeumannScalar(A, G(h));
    scalar_out(h, A, a);
}
void ref_fill_scalar_periodic(void* hp, double* a) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d A = scalar_in(h, a);
    FillGhostCellsPeriodicScalar(A, G(h));
    scalar_out(h, A, a);
}
void ref_fill_velocity_neumann(void* hp, double* v) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array3d V = vel_in(h, v);
    FillGhostCellsNeumannVelocity(V, h->sp()->v_bounds);
    vel_out(h, V, v);
}

/* ---- elliptic part ---- */
double ref_mu(void* hp, double c) { return static_cast<RefCase*>(hp)->mg()->mu(c); }
/* Face values K/mu of KoverMu_11_im12j for i in [0,N1], j in [0,N2) and KoverMu_22_ijm12 for
 * i in [0,N1), j in [0,N2] (src/EllipticSolver.cpp:478-524); c with filled ghosts. */
void ref_face_mobility(void* hp, const double* c, double* lamx, double* lamy) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d C = scalar_in(h, c);
    MGSolver* mg = h->mg();
    const int n1 = N1(h), n2 = N2(h);
    for (int i = 0; i <= n1; ++i)
        for (int j = 0; j < n2; ++j) lamx[(size_t)i * n2 + j] = mg->KoverMu_11_im12j(C(i - 1, j), C(i, j), i, j);
    for (int i = 0; i < n1; ++i)
        for (int j = 0; j <= n2; ++j) lamy[(size_t)i * (n2 + 1) + j] = mg->KoverMu_22_ijm12(C(i, j - 1), C(i, j), i, j);
}
/* The assembled pressure matrix (SetMatrixCoefficients_Elliptic, src/MGSolver.cpp:268-570). */
void ref_pressure_matrix(void* hp, const double* c, double* A9) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d C = scalar_in(h, c);
    MGSolver* mg = h->mg();
    mg->InitializeComponents();
    mg->SetMatrixCoefficients_Elliptic(C);
    matrix_out(mg->A, A9);
    mg->DestroyComponents();
}
/* b = -q (SetRHS_Elliptic, src/MGSolver.cpp:573-590). */
void ref_pressure_rhs(void* hp, const double* q, double* b) {
    RefCase* h = static_cast<RefCase*>(hp);
    MGSolver* mg = h->mg();
    mg->InitializeComponents();
    mg->SetRHS_Elliptic(q);
    vector_out(mg->b, b);
    mg->DestroyComponents();
}
/* EllipticSolver::Solve (src/EllipticSolver.cpp:133-141): assemble, solve (direct), map to p.
 * c and p in the scalar ghost layout; p's interior is written. */
int ref_pressure_solve(void* hp, double* c, const double* q, double* p) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d C = scalar_in(h, c), Pa = scalar_in(h, p);
    std::vector<double> qq(q, q + h->sp()->M);
    bool ok = h->mg()->Solve(Pa, C, qq.data());
    scalar_out(h, Pa, p);
    return ok ? 0 : 1;
}
/* CalcVelocities (src/EllipticSolver.cpp:660-683): fills p's ghosts, writes v with ghosts. */
void ref_calc_velocities(void* hp, double* p, double* v, const double* c) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d Pa = scalar_in(h, p), C = scalar_in(h, c);
    Array3d V = vel_in(h, v);
    h->mg()->CalcVelocities(Pa, V, C);
    scalar_out(h, Pa, p);
    vel_out(h, V, v);
}

/* ---- hyperbolic part ---- */
double ref_max_stable_dt(void* hp, const double* c, const double* v) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d C = scalar_in(h, c);
    Array3d V = vel_in(h, v);
    return h->solver->hs->MaxStableTimestep(C, V);
}
/* TRIntegrator::Integrate (src/TRIntegrator.cpp:49-71); returns the outflux it records. */
double ref_tr_integrate(void* hp, double* c, const double* q, double dt) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d C = scalar_in(h, c);
    TimeIntegrator* ti = h->solver->hs->ti;
    ti->Integrate(C, q, dt);
    scalar_out(h, C, c);
    return ti->GetTotalMassOutflux();
}
/* Intercell fluxes F ((N1+1) x (N2+2g), j from -g) and G ((N1+2g) x (N2+1), i from -g),
 * with F, G zeroed first as Advect_X/Y do (src/HyperbolicSplitSolver.cpp:113-159). */
void ref_flux_F(void* hp, int scheme, double* F, const double* c, const double* v, double dt) {
    RefCase* h = static_cast<RefCase*>(hp);
    const int g = G(h), n1 = N1(h), n2 = N2(h);
    Array2d Fa(n1 + 1, n2 + 2 * g);
    Fa.reindexSelf(Idx2d(0, -g));
    Fa = 0;
    Array2d C = scalar_in(h, c);
    Array3d V = vel_in(h, v);
    h->split(scheme)->CalculateIntercellFlux_F(Fa, C, V, dt);
    for (int i = 0; i <= n1; ++i)
        for (int j = -g; j < n2 + g; ++j) F[(size_t)i * (n2 + 2 * g) + (j + g)] = Fa(i, j);
}
void ref_flux_G(void* hp, int scheme, double* Gf, const double* c, const double* v, double dt) {
    RefCase* h = static_cast<RefCase*>(hp);
    const int g = G(h), n1 = N1(h), n2 = N2(h);
    Array2d Ga(n1 + 2 * g, n2 + 1);
    Ga.reindexSelf(Idx2d(-g, 0));
    Ga = 0;
    Array2d C = scalar_in(h, c);
    Array3d V = vel_in(h, v);
    h->split(scheme)->CalculateIntercellFlux_G(Ga, C, V, dt);
    for (int i = -g; i < n1 + g; ++i)
        for (int j = 0; j <= n2; ++j) Gf[(size_t)(i + g) * (n2 + 1) + j] = Ga(i, j);
}
void ref_advect_x(void* hp, int scheme, double* c, const double* v, double dt) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d C = scalar_in(h, c);
    Array3d V = vel_in(h, v);
    h->split(scheme)->Advect_X(C, V, dt);
    scalar_out(h, C, c);
}
void ref_advect_y(void* hp, int scheme, double* c, const double* v, double dt) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d C = scalar_in(h, c);
    Array3d V = vel_in(h, v);
    h->split(scheme)->Advect_Y(C, V, dt);
    scalar_out(h, C, c);
}
/* AdvectSplit (src/HyperbolicSplitSolver.cpp:51-106) in the cfg's splitting mode;
 * *prev_first_sweep (0 X_SWEEP, 1 Y_SWEEP) is the alternating mode's state, in and out. */
void ref_advect_split(void* hp, int scheme, double* c, const double* v, double dt, int* prev_first_sweep) {
    RefCase* h = static_cast<RefCase*>(hp);
    HyperbolicSplitSolver* s = h->split(scheme);
    Array2d C = scalar_in(h, c);
    Array3d V = vel_in(h, v);
    s->prev_first_sweep = *prev_first_sweep ? Y_SWEEP : X_SWEEP;
    s->AdvectSplit(C, V, nullptr, dt);
    *prev_first_sweep = s->prev_first_sweep == Y_SWEEP ? 1 : 0;
    scalar_out(h, C, c);
}
/* HyperbolicSplitSolver::Solve (src/HyperbolicSplitSolver.cpp:162-198): half source, half CN
 * dispersion, advection, half source, half CN.  *outflux is total_mass_outflux, in and out. */
int ref_hyperbolic_solve(void* hp, int scheme, double* c, const double* v, const double* q, double dt,
                         int* prev_first_sweep, double* outflux) {
    RefCase* h = static_cast<RefCase*>(hp);
    HyperbolicSplitSolver* s = h->split(scheme);
    Array2d C = scalar_in(h, c);
    Array3d V = vel_in(h, v);
    s->prev_first_sweep = *prev_first_sweep ? Y_SWEEP : X_SWEEP;
    s->total_mass_outflux = *outflux;
    bool ok = s->Solve(C, V, q, dt);
    *prev_first_sweep = s->prev_first_sweep == Y_SWEEP ? 1 : 0;
    *outflux = s->total_mass_outflux;
    scalar_out(h, C, c);
    return ok ? 0 : 1;
}

/* ---- Peaceman dispersion and Crank-Nicolson (src/MGSolver.cpp:846-1392) ---- */
void ref_peaceman_F(void* hp, const double* v, int i, int j, double* d11, double* d12) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array3d V = vel_in(h, v);
    h->mg()->SetupDiffusionTensorF(h->sp()->dx, h->sp()->dy, V, i, j, *d11, *d12);
}
void ref_peaceman_G(void* hp, const double* v, int i, int j, double* d22, double* d21) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array3d V = vel_in(h, v);
    h->mg()->SetupDiffusionTensorG(h->sp()->dx, h->sp()->dy, V, i, j, *d22, *d21);
}
void ref_cn_matrix(void* hp, const double* v, double dt, double* A9) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array3d V = vel_in(h, v);
    MGSolver* mg = h->mg();
    mg->InitializeComponents();
    mg->SetMatrixCoefficients_Parabolic(V, nullptr, dt);
    matrix_out(mg->A, A9);
    mg->DestroyComponents();
}
void ref_cn_rhs(void* hp, const double* c, const double* v, double dt, double* b) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d C = scalar_in(h, c);
    Array3d V = vel_in(h, v);
    MGSolver* mg = h->mg();
    mg->InitializeComponents();
    mg->SetRHS_Parabolic(C, V, dt, nullptr);
    vector_out(mg->b, b);
    mg->DestroyComponents();
}
/* Solve_Parabolic_cc_to_c (src/MGSolver.cpp:952-976); c's interior is replaced. */
int ref_cn_solve(void* hp, double* c, const double* v, double dt) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d C = scalar_in(h, c);
    Array3d V = vel_in(h, v);
    bool ok = h->mg()->Solve_Parabolic_cc_to_c(C, G(h), V, h->sp()->v_bounds, nullptr, 0, dt);
    scalar_out(h, C, c);
    return ok ? 0 : 1;
}

/* ---- the reference's run loop and diagnostics ---- */
/* Impec2DSolver::Solve (src/Impec2DSolver.cpp:293-466) from the constructor's state to the
 * cfg's endtime, writing what the cfg asks for; then c, p, v (ghost layouts) and the number of
 * steps taken.  c0, when not NULL, replaces the initial concentration (interior and ghosts). */
int ref_run(void* hp, const double* c0, double* c, double* p, double* v, int* steps) {
    RefCase* h = static_cast<RefCase*>(hp);
    if (c0) {
        Array2d C0 = scalar_in(h, c0);
        h->solver->c = C0;
    }
    const int before = impec_hypre_shim_solves();
    bool ok = h->solver->Solve();
    if (steps) *steps = impec_hypre_shim_solves() - before;  // one pressure solve per step without CN
    if (c) scalar_out(h, h->solver->c, c);
    if (p) scalar_out(h, h->solver->p, p);
    if (v) vel_out(h, h->solver->v, v);
    return ok ? 0 : 1;
}
/* Impec2DSolver::Run (src/Impec2DSolver.cpp:747-760): the test component for is_test cfgs. */
int ref_run_component(void* hp) { return static_cast<RefCase*>(hp)->solver->Run() ? 0 : 1; }
double ref_total_mass(void* hp, const double* c) {
    RefCase* h = static_cast<RefCase*>(hp);
    h->solver->c = scalar_in(h, c);
    return h->solver->GetTotalMass();
}
double ref_mass_error(void* hp, const double* c, double t, double outflux) {
    RefCase* h = static_cast<RefCase*>(hp);
    h->solver->c = scalar_in(h, c);
    h->solver->hs->total_mass_outflux = outflux;
    return h->solver->CalculateMassError(t);
}
double ref_divergence_error(void* hp, const double* v) {
    RefCase* h = static_cast<RefCase*>(hp);
    h->solver->v = vel_in(h, v);
    return h->solver->CalculateDivergenceError();
}
double ref_velocity_boundary_error(void* hp, const double* v) {
    RefCase* h = static_cast<RefCase*>(hp);
    h->solver->v = vel_in(h, v);
    return h->solver->CalculateVelocityBoundaryError();
}
namespace {
// The advection test's profile as Impec2DSolver::Advection picks it (src/Impec2DSolver.cpp:854-870).
double (*profile_fn(const SimParams* sp))(SimParams const* const, double, double) {
    switch (sp->hyp_test) {
        case SINE: return Sinewave;
        case TOPHAT: return Tophat;
        case GAUSS: return Gaussbell;
        case HSINE: return VerticalSine;
    }
    return Sinewave;
}
}  // namespace

/* L1 (norm 1) or L2 (norm 2) error of c against the cfg's advection profile at time t
 * (src/Util.cpp:119-147). */
double ref_advection_norm(void* hp, const double* c, double t, int norm) {
    RefCase* h = static_cast<RefCase*>(hp);
    Array2d C = scalar_in(h, c);
    return norm == 1 ? CalcAdvectionL1Norm(h->sp(), C, t, profile_fn(h->sp()))
                     : CalcAdvectionL2Norm(h->sp(), C, t, profile_fn(h->sp()));
}

/* The reference's advection convergence test (Impec2DSolver::TestAdvection and Advection,
 * src/Impec2DSolver.cpp:773-990) on an is_test cfg, with the constant velocity (vx, vy) in
 * place of the shipped diagonal one, (-(x_ub-x_lb), y_ub-y_lb) (src/Impec2DSolver.cpp:
 * 1003-1015).  The profile, the grids (initial cells doubled `levels` times), the time step,
 * the output-time matching and the norm are the reference's; log(dx) and log(norm) of each
 * level go to logdx[k], lognorm[k].  Only the velocity is the caller's: the published
 * convergence rates are labelled "y-advection" (examples/hyperbolic_test.cfg:131). */
int ref_advection_test(const char* cfg, double vx, double vy, double* logdx, double* lognorm) {
    Impec2DSolver* s = new Impec2DSolver(std::string(cfg), 0, 1);
    SimParams* sp = s->sp;
    sp->N1 = sp->init_x_cells;
    sp->N2 = sp->init_y_cells;
    delete[] s->q;
    for (int k = 0; k < sp->levels; ++k) {
        sp->dx = (sp->x_ub - sp->x_lb) / sp->N1;
        sp->dy = (sp->y_ub - sp->y_lb) / sp->N2;
        sp->M = sp->N1 * sp->N2;
        s->c.resize(sp->N1 + 2 * sp->p_bounds, sp->N2 + 2 * sp->p_bounds);
        s->c.reindexSelf(Idx2d(-sp->p_bounds, -sp->p_bounds));
        s->v.resize(sp->N1 + 1 + 2 * sp->v_bounds, sp->N2 + 1 + 2 * sp->v_bounds, 2);
        s->v.reindexSelf(Idx3d(-sp->v_bounds, -sp->v_bounds, 0));
        s->v = 0;
        s->c = 0;
        s->q = (double*)calloc(sp->M, sizeof(double));
        double (*f)(SimParams const* const, double, double) = profile_fn(sp);
        s->InitAdvection(f);
        for (int i = -sp->v_bounds; i <= sp->N1 + sp->v_bounds; i++)
            for (int j = -sp->v_bounds; j <= sp->N2 + sp->v_bounds; j++) {
                s->v(i, j, 0) = vx;
                s->v(i, j, 1) = vy;
            }
        const double dt_max = s->hs->MaxStableAdvectionTimestep(s->c, s->v);
        std::vector<double> times = sp->times;
        if (std::find(times.begin(), times.end(), sp->tfinal) == times.end()) times.push_back(sp->tfinal);
        std::sort(times.begin(), times.end());
        size_t tidx = 0;
        double t = sp->tstart, dt = dt_max;
        bool ok = true;
        while (ok && t < sp->tfinal) {
            if (tidx < times.size() && t + dt >= times[tidx]) {
                dt = times[tidx] - t;
                tidx++;
            } else {
                dt = dt_max;
            }
            ok = s->hs->Solve(s->c, s->v, s->q, dt);
            t += dt;
        }
        const double norm = sp->hyp_norm == L1 ? CalcAdvectionL1Norm(sp, s->c, t, f) : CalcAdvectionL2Norm(sp, s->c, t, f);
        logdx[k] = std::log(sp->dx);
        lognorm[k] = std::log(norm);
        free(s->q);
        s->q = nullptr;
        if (!ok) {
            delete s;
            return 1;
        }
        sp->N1 *= 2;
        sp->N2 *= 2;
    }
    delete s;
    return 0;
}

}  // extern "C"
