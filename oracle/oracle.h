/*
 * Impec2D CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++ (FP64, IEEE, no FMA contraction) restatement of the reference
 * Impec2D discretisation (pw359/Impec2D, the src directory).  It exists to check the
 * CUDA implementation: only the tests, the smoke check and the CPU-baseline leg
 * of bench.py may load it.  The product never links or calls it.
 *
 * Parity status: PINNED to the reference itself.  The reference's own sources compile
 * unchanged against the stand-ins in oracle/refshim (a Blitz++ subset, libconfig++, one-rank
 * MPI, and HYPRE reduced to a recorded system with a direct solve) into oracle/_ref
 * (recipe oracle/Makefile.ref, entry points oracle/ref_driver.cpp).  Every operation of this
 * oracle that is reference code -- assembly with its Neumann folds and Dirichlet rows, face
 * and corner mobilities, velocities, the CFL step, TR, MUSCL and upwind fluxes, the five
 * split modes, Peaceman tensors, the Crank-Nicolson matrix and right-hand side, sources,
 * ghost fills and diagnostics -- equals the reference's output bit for bit
 * (tests/test_ref_pin.py; fixtures the reference wrote, tests/golden/ref_*, checked in
 * tests/test_oracle_golden.py).  At the HYPRE boundary only the discrete system A x = b is
 * reference code; HYPRE's iterates are not (its sources are not part of the reference), so
 * solves are compared by residual under the reference's own assembled system.
 *
 * Array layouts follow the reference's Blitz arrays (src/Impec2DSolver.cpp:151-182):
 *   scalar fields c, p: (N1+2g) x (N2+2g), row-major, j fastest, ghost width g;
 *                       element (i,j) at (i+g)*(N2+2g) + (j+g), i,j in [-g, N+g)
 *   velocity v:         (N1+1+2g) x (N2+1+2g) x 2, k innermost (0: u, 1: v)
 *   source q:           N1*N2, element (i,j) at i*N2 + j
 *   9-point stencils:   N1*N2*9 in HYPRE entry order C,W,SW,S,SE,E,NE,N,NW
 *                       (src/MGSolver.cpp:164-166, 286-294)
 */
#ifndef IMPEC_ORACLE_H
#define IMPEC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Enum values match src/SimParams.h:14-27. */
enum { OR_MEANCONC = 0, OR_HARMONIC = 1 };
enum { OR_EXPLICIT = 0, OR_CRANKNICOLSON = 1 };
enum { OR_ALTERNATING = 0, OR_X_FIRST = 1, OR_Y_FIRST = 2, OR_STRANG = 3, OR_SYMMETRIC_PARALLEL = 4 };
enum { OR_UPWINDSPLIT = 0, OR_WAFSPLIT = 1, OR_WAF = 2, OR_CTU = 3, OR_MUSCL = 4 };
enum { OR_PARALLEL = 0, OR_DIAGONAL = 1, OR_HORIZONTAL = 2 };
enum { OR_CIRCULAR = 0, OR_GAUSSIAN = 1, OR_ONECELL = 2 };
enum { OR_PULSING = 0, OR_LINEAR = 1, OR_CONSTANT = 2 };

typedef struct {
    int N1, N2, g;                 /* interior cells, ghost layers (num_ghostcells) */
    double x_lb, x_ub, y_lb, y_ub;
    double mu_res, mu_inj;
    int avgproc;                   /* OR_MEANCONC | OR_HARMONIC */
    double nu;                     /* parallel/diagonal stencil weight */
    double porosity, cfl, inj_fluid_conc, I;
    int diffusion;                 /* Peaceman dispersion on/off */
    double alpha_l, alpha_t;       /* in cell units: multiplied by max(dx,dy) */
    double Dm;                     /* extension: molecular diffusion (0 = reference) */
    int ptype;                     /* OR_EXPLICIT | OR_CRANKNICOLSON (dt rule only) */
    double dt_diff_limit;
    int dim_splitting;
    int hmtype;                    /* OR_MUSCL | OR_UPWINDSPLIT | OR_WAFSPLIT | OR_WAF | OR_CTU */
    int stype;                     /* OR_PARALLEL | OR_DIAGONAL | OR_HORIZONTAL */
    int is_test, testno;
    double eps, para_eps;
    int well_profile;
    double well_rc;
    double well_width, q_high_multiple, q_freq, tstart, tfinal;
    int inj_mode;
    const double* K11;             /* extension: per-cell permeability (N1*N2) or NULL (K = 1) */
    const double* K22;
    int peaceman_guard;            /* 1: Peaceman term := 0 where |u| = 0 (reference gives NaN) */
} or_params;

/* ---- ghost fills (src/Util.cpp:215-438) ---- */
void or_fill_scalar_neumann(const or_params* P, double* a);
void or_fill_scalar_periodic(const or_params* P, double* a);
void or_fill_velocity_neumann(const or_params* P, double* v);

/* ---- elliptic (src/EllipticSolver.cpp, src/MGSolver.cpp) ---- */
double or_mu(const or_params* P, double c);
/* Reference pressure matrix incl. Neumann folding and Dirichlet pin; A9: N1*N2*9. */
void or_pressure_matrix(const or_params* P, const double* c, double* A9);
/* Same matrix but the pinned rows keep their folded Neumann coefficients. */
void or_pressure_matrix_neumann(const or_params* P, const double* c, double* A9);
void or_pressure_rhs(const or_params* P, const double* q, double* b);
/* Face mobilities KoverMu_11_im12j ((N1+1)*N2) and KoverMu_22_ijm12 (N1*(N2+1)). */
void or_face_mobility(const or_params* P, const double* c, double* lamx, double* lamy);
void or_matvec9(const or_params* P, const double* A9, const double* x, double* y);
double or_relres9(const or_params* P, const double* A9, const double* x, const double* b);
/* Direct banded LU (+ iterative refinement).  Returns 0 on success. */
int or_solve_banded(const or_params* P, const double* A9, const double* b, double* x);
/* Full reference pressure solve: matrix + rhs + solve; p in ghost layout (interior written). */
int or_pressure_solve(const or_params* P, const double* c, const double* q, double* p,
                      int method, double tol, int* its, double* relres);
void or_calc_velocities(const or_params* P, double* p, double* v, const double* c);
double or_max_stable_dt(const or_params* P, const double* v);
double or_max_stable_advection_dt(const or_params* P, const double* v);

/* ---- hyperbolic (src/TRIntegrator.cpp and the split solvers) ---- */
double or_tr_integrate(const or_params* P, double* c, const double* q, double dt);
void or_flux_F(const or_params* P, double* F, const double* c, const double* v, double dt);
void or_flux_G(const or_params* P, double* G, const double* c, const double* v, double dt);
void or_advect_x(const or_params* P, double* c, const double* v, double dt);
void or_advect_y(const or_params* P, double* c, const double* v, double dt);
/* hyper_method "ctu": Colella's unsplit corner transport upwind update of the interior
 * (ghosts of c and v filled). */
void or_ctu_advect(const or_params* P, double* c, const double* v, double dt);
/* prev_first_sweep: 0 = X_SWEEP, 1 = Y_SWEEP (state of the ALTERNATING mode).  hmtype OR_CTU
 * advects unsplit (or_ctu_advect); OR_WAFSPLIT and OR_WAF use the WAF flux in the sweeps. */
void or_advect_split(const or_params* P, double* c, const double* v, double dt, int* prev_first_sweep);
void or_peaceman_F(const or_params* P, const double* v, int i, int j, double* d11, double* d12);
void or_peaceman_G(const or_params* P, const double* v, int i, int j, double* d22, double* d21);
void or_cn_matrix(const or_params* P, const double* v, double dt, double* A9);
void or_cn_rhs(const or_params* P, const double* c, const double* v, double dt, double* b);
int or_cn_solve(const or_params* P, double* c, const double* v, double dt, int method,
                double tol, int* its, double* relres);
/* HyperbolicSplitSolver::Solve; *outflux accumulates like total_mass_outflux. */
int or_hyperbolic_solve(const or_params* P, double* c, const double* v, const double* q,
                        double dt, int* prev_first_sweep, double* outflux, int solver);

/* ---- whole IMPES step (src/Impec2DSolver.cpp:339-415) ---- */
typedef struct {
    double t, dt, total_outflux;
    int counter, prev_first_sweep, its, para_its;
    double mass_err, vel_err, div_err, relres;
} or_state;
int or_impes_step(const or_params* P, or_state* S, double* c, double* p, double* v,
                  const double* q, const double* times, int ntimes, int* tidx,
                  int solver, double tol);

/* ---- diagnostics (src/Impec2DSolver.cpp:530-620) ---- */
double or_total_mass(const or_params* P, const double* c);
double or_mass_error(const or_params* P, const double* c, double t, double outflux);
double or_divergence_error(const or_params* P, const double* v, const double* q);
double or_velocity_boundary_error(const or_params* P, const double* v);

/* ---- wells and test profiles (src/Util.cpp, src/Impec2DSolver.cpp:241-280) ---- */
void or_init_source(const or_params* P, double* q, double t);
double or_exact_vol_frac_circle(double x1, double y1, double r, double dx, double dy);
/* profile: 0 sine, 1 tophat, 2 gaussbell, 3 vertical sine, 4 diagonal sine */
double or_profile(const or_params* P, int profile, double x, double y);
double or_advection_norm(const or_params* P, const double* c, int profile, int norm);
/* ParallelProjector (src/ParallelProjector.cpp:51-199, src/Impec2DSolver.cpp:690-716):
 * bilinear projection of a parallel-orientation field f (Blitz layout with ghosts, ghost ring
 * already filled) onto the dN1 x dN2 diagonal grid; out is dN1*dN2, row-major. */
void or_project_diagonal(const or_params* P, const double* f, int dN1, int dN2, double* out);
/* Elliptic manufactured test (src/EllipticSolver.cpp:155-311) at the grid in P. */
int or_elliptic_test(const or_params* P, double* errs3);

/* ---- CPU multigrid used as the timed CPU baseline ---- */
int or_mg_solve(const or_params* P, const double* A9_neumann, const double* b, double* x,
                double tol, int max_cycles, int* cycles, double* relres, int pin_i, int pin_j,
                double pin_value);
int or_num_threads(void);
int or_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
