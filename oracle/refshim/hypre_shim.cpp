/*
 * Stand-in for HYPRE's struct solvers -- TEST INFRASTRUCTURE ONLY.  What it keeps and what
 * it replaces is described in HYPRE_struct_ls.h beside it.
 *
 * The solve is a banded LU factorisation without pivoting of the recorded 9-point system
 * (cells ordered with the second index fastest, so the bandwidth is ny + 1), followed by two
 * steps of iterative refinement.  The reference's systems are M-matrix-like (positive
 * diagonal, non-positive neighbours for the pressure; identity plus a small dispersion
 * operator for Crank-Nicolson), for which elimination without pivoting is stable.
 */
#include "HYPRE_struct_ls.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

struct impec_hypre_grid {
    int lo[2] = {0, 0}, hi[2] = {-1, -1};
    int nx() const { return hi[0] - lo[0] + 1; }
    int ny() const { return hi[1] - lo[1] + 1; }
    size_t n() const { return (size_t)nx() * (size_t)ny(); }
    bool inside(int k, int l) const { return k >= lo[0] && k <= hi[0] && l >= lo[1] && l <= hi[1]; }
    size_t at(int k, int l) const { return (size_t)(k - lo[0]) * ny() + (size_t)(l - lo[1]); }
};
struct impec_hypre_stencil {
    std::vector<int> off;  // 2 per entry
};
struct impec_hypre_matrix {
    impec_hypre_grid grid;
    std::vector<int> off;
    std::vector<double> coef;  // n x entries
};
struct impec_hypre_vector {
    impec_hypre_grid grid;
    std::vector<double> val;
};
struct impec_hypre_solver {
    int its = 0;
    double relres = 0;
};

static int g_solves = 0;

HYPRE_Int HYPRE_StructGridCreate(MPI_Comm, HYPRE_Int, HYPRE_StructGrid* grid) {
    *grid = new impec_hypre_grid();
    return 0;
}
HYPRE_Int HYPRE_StructGridSetExtents(HYPRE_StructGrid g, HYPRE_Int* lo, HYPRE_Int* hi) {
    g->lo[0] = lo[0];
    g->lo[1] = lo[1];
    g->hi[0] = hi[0];
    g->hi[1] = hi[1];
    return 0;
}
HYPRE_Int HYPRE_StructGridAssemble(HYPRE_StructGrid) { return 0; }
HYPRE_Int HYPRE_StructGridDestroy(HYPRE_StructGrid g) {
    delete g;
    return 0;
}

HYPRE_Int HYPRE_StructStencilCreate(HYPRE_Int, HYPRE_Int size, HYPRE_StructStencil* s) {
    *s = new impec_hypre_stencil();
    (*s)->off.assign(2 * size, 0);
    return 0;
}
HYPRE_Int HYPRE_StructStencilSetElement(HYPRE_StructStencil s, HYPRE_Int e, HYPRE_Int* off) {
    s->off[2 * e] = off[0];
    s->off[2 * e + 1] = off[1];
    return 0;
}
HYPRE_Int HYPRE_StructStencilDestroy(HYPRE_StructStencil s) {
    delete s;
    return 0;
}

HYPRE_Int HYPRE_StructMatrixCreate(MPI_Comm, HYPRE_StructGrid g, HYPRE_StructStencil s, HYPRE_StructMatrix* A) {
    *A = new impec_hypre_matrix();
    (*A)->grid = *g;
    (*A)->off = s->off;
    return 0;
}
HYPRE_Int HYPRE_StructMatrixInitialize(HYPRE_StructMatrix A) {
    A->coef.assign(A->grid.n() * (A->off.size() / 2), 0.0);
    return 0;
}
HYPRE_Int HYPRE_StructMatrixSetValues(HYPRE_StructMatrix A, HYPRE_Int* idx, HYPRE_Int n, HYPRE_Int* entries,
                                      HYPRE_Real* values) {
    if (!A->grid.inside(idx[0], idx[1])) return 1;
    const size_t ne = A->off.size() / 2;
    const size_t row = A->grid.at(idx[0], idx[1]);
    for (int e = 0; e < n; ++e) A->coef[row * ne + entries[e]] = values[e];
    return 0;
}
HYPRE_Int HYPRE_StructMatrixAssemble(HYPRE_StructMatrix) { return 0; }
HYPRE_Int HYPRE_StructMatrixDestroy(HYPRE_StructMatrix A) {
    delete A;
    return 0;
}

HYPRE_Int HYPRE_StructVectorCreate(MPI_Comm, HYPRE_StructGrid g, HYPRE_StructVector* v) {
    *v = new impec_hypre_vector();
    (*v)->grid = *g;
    return 0;
}
HYPRE_Int HYPRE_StructVectorInitialize(HYPRE_StructVector v) {
    v->val.assign(v->grid.n(), 0.0);
    return 0;
}
HYPRE_Int HYPRE_StructVectorSetValues(HYPRE_StructVector v, HYPRE_Int* idx, HYPRE_Real value) {
    if (!v->grid.inside(idx[0], idx[1])) return 1;
    v->val[v->grid.at(idx[0], idx[1])] = value;
    return 0;
}
HYPRE_Int HYPRE_StructVectorSetBoxValues(HYPRE_StructVector v, HYPRE_Int* lo, HYPRE_Int* hi, HYPRE_Real* values) {
    size_t m = 0;
    for (int k = lo[0]; k <= hi[0]; ++k)
        for (int l = lo[1]; l <= hi[1]; ++l, ++m)
            if (v->grid.inside(k, l)) v->val[v->grid.at(k, l)] = values[m];
    return 0;
}
HYPRE_Int HYPRE_StructVectorGetValues(HYPRE_StructVector v, HYPRE_Int* idx, HYPRE_Real* value) {
    if (!v->grid.inside(idx[0], idx[1])) return 1;
    *value = v->val[v->grid.at(idx[0], idx[1])];
    return 0;
}
HYPRE_Int HYPRE_StructVectorAssemble(HYPRE_StructVector) { return 0; }
HYPRE_Int HYPRE_StructVectorDestroy(HYPRE_StructVector v) {
    delete v;
    return 0;
}

// y = A x over the grid box; couplings that leave the box count as zero.
static void matvec(const impec_hypre_matrix& A, const std::vector<double>& x, std::vector<double>& y) {
    const impec_hypre_grid& g = A.grid;
    const size_t ne = A.off.size() / 2;
    y.assign(g.n(), 0.0);
    for (int k = g.lo[0]; k <= g.hi[0]; ++k)
        for (int l = g.lo[1]; l <= g.hi[1]; ++l) {
            const size_t r = g.at(k, l);
            double s = 0;
            for (size_t e = 0; e < ne; ++e) {
                const int kk = k + A.off[2 * e], ll = l + A.off[2 * e + 1];
                if (g.inside(kk, ll)) s += A.coef[r * ne + e] * x[g.at(kk, ll)];
            }
            y[r] = s;
        }
}

static int direct_solve(const impec_hypre_matrix& A, const impec_hypre_vector& b, impec_hypre_vector& x,
                        impec_hypre_solver* S) {
    const impec_hypre_grid& g = A.grid;
    const long n = (long)g.n(), w = g.ny() + 1;  // lower = upper bandwidth
    const double work = (double)n * (double)w * (double)w;
    if (work > 6e10) {
        std::fprintf(stderr, "hypre shim: system of %ld cells too large for the direct solve\n", n);
        std::abort();
    }
    const long W = 2 * w + 1;
    std::vector<double> band((size_t)n * W, 0.0);  // row r, column c at band[r*W + (c - r + w)]
    const size_t ne = A.off.size() / 2;
    for (int k = g.lo[0]; k <= g.hi[0]; ++k)
        for (int l = g.lo[1]; l <= g.hi[1]; ++l) {
            const long r = (long)g.at(k, l);
            for (size_t e = 0; e < ne; ++e) {
                const int kk = k + A.off[2 * e], ll = l + A.off[2 * e + 1];
                if (!g.inside(kk, ll)) continue;
                const long c = (long)g.at(kk, ll);
                band[(size_t)r * W + (c - r + w)] += A.coef[(size_t)r * ne + e];
            }
        }
    for (long p = 0; p < n; ++p) {  // elimination without pivoting
        const double piv = band[(size_t)p * W + w];
        if (piv == 0.0 || !std::isfinite(piv)) {
            std::fprintf(stderr, "hypre shim: zero pivot at row %ld\n", p);
            std::abort();
        }
        const long rmax = std::min(n - 1, p + w);
        for (long r = p + 1; r <= rmax; ++r) {
            double& lrp = band[(size_t)r * W + (p - r + w)];
            if (lrp == 0.0) continue;
            lrp /= piv;
            const long cmax = std::min(n - 1, p + w);
            for (long c = p + 1; c <= cmax; ++c) band[(size_t)r * W + (c - r + w)] -= lrp * band[(size_t)p * W + (c - p + w)];
        }
    }
    auto lu_solve = [&](std::vector<double>& v) {
        for (long r = 0; r < n; ++r) {
            double s = v[r];
            for (long c = std::max(0L, r - w); c < r; ++c) s -= band[(size_t)r * W + (c - r + w)] * v[c];
            v[r] = s;
        }
        for (long r = n - 1; r >= 0; --r) {
            double s = v[r];
            for (long c = r + 1; c <= std::min(n - 1, r + w); ++c) s -= band[(size_t)r * W + (c - r + w)] * v[c];
            v[r] = s / band[(size_t)r * W + w];
        }
    };
    std::vector<double> sol = b.val;
    lu_solve(sol);
    std::vector<double> ax, res((size_t)n);
    for (int it = 0; it < 2; ++it) {  // iterative refinement
        matvec(A, sol, ax);
        for (long r = 0; r < n; ++r) res[r] = b.val[r] - ax[r];
        lu_solve(res);
        for (long r = 0; r < n; ++r) sol[r] += res[r];
    }
    matvec(A, sol, ax);
    double rn = 0, bn = 0;
    for (long r = 0; r < n; ++r) {
        rn += (b.val[r] - ax[r]) * (b.val[r] - ax[r]);
        bn += b.val[r] * b.val[r];
    }
    x.val = sol;
    ++g_solves;
    if (S) {
        S->its = 1;
        S->relres = bn > 0 ? std::sqrt(rn / bn) : std::sqrt(rn);
    }
    return 0;
}

#define IMPEC_SHIM_SOLVER(NAME)                                                                                     \
    HYPRE_Int HYPRE_Struct##NAME##Create(MPI_Comm, HYPRE_StructSolver* s) {                                          \
        *s = new impec_hypre_solver();                                                                               \
        return 0;                                                                                                    \
    }                                                                                                                \
    HYPRE_Int HYPRE_Struct##NAME##Destroy(HYPRE_StructSolver s) {                                                    \
        delete s;                                                                                                    \
        return 0;                                                                                                    \
    }                                                                                                                \
    HYPRE_Int HYPRE_Struct##NAME##SetMaxIter(HYPRE_StructSolver, HYPRE_Int) { return 0; }                            \
    HYPRE_Int HYPRE_Struct##NAME##SetTol(HYPRE_StructSolver, HYPRE_Real) { return 0; }                               \
    HYPRE_Int HYPRE_Struct##NAME##Setup(HYPRE_StructSolver, HYPRE_StructMatrix, HYPRE_StructVector, HYPRE_StructVector) { \
        return 0;                                                                                                    \
    }                                                                                                                \
    HYPRE_Int HYPRE_Struct##NAME##Solve(HYPRE_StructSolver s, HYPRE_StructMatrix A, HYPRE_StructVector b,           \
                                        HYPRE_StructVector x) {                                                      \
        return direct_solve(*A, *b, *x, s);                                                                          \
    }                                                                                                                \
    HYPRE_Int HYPRE_Struct##NAME##GetNumIterations(HYPRE_StructSolver s, HYPRE_Int* n) {                             \
        *n = s->its;                                                                                                 \
        return 0;                                                                                                    \
    }                                                                                                                \
    HYPRE_Int HYPRE_Struct##NAME##GetFinalRelativeResidualNorm(HYPRE_StructSolver s, HYPRE_Real* r) {                \
        *r = s->relres;                                                                                              \
        return 0;                                                                                                    \
    }
IMPEC_SHIM_SOLVER(PCG)
IMPEC_SHIM_SOLVER(SMG)
IMPEC_SHIM_SOLVER(Jacobi)
#undef IMPEC_SHIM_SOLVER

HYPRE_Int HYPRE_StructPCGSetTwoNorm(HYPRE_StructSolver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_StructPCGSetRelChange(HYPRE_StructSolver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_StructPCGSetPrintLevel(HYPRE_StructSolver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_StructPCGSetLogging(HYPRE_StructSolver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_StructPCGSetPrecond(HYPRE_StructSolver, HYPRE_PtrToStructSolverFcn, HYPRE_PtrToStructSolverFcn,
                                    HYPRE_StructSolver) {
    return 0;
}
HYPRE_Int HYPRE_StructSMGSetMemoryUse(HYPRE_StructSolver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_StructSMGSetZeroGuess(HYPRE_StructSolver) { return 0; }
HYPRE_Int HYPRE_StructSMGSetRelChange(HYPRE_StructSolver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_StructSMGSetNumPreRelax(HYPRE_StructSolver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_StructSMGSetNumPostRelax(HYPRE_StructSolver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_StructSMGSetLogging(HYPRE_StructSolver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_StructJacobiSetNonZeroGuess(HYPRE_StructSolver) { return 0; }

HYPRE_Int impec_hypre_shim_matrix(HYPRE_StructMatrix A, HYPRE_Int* lo, HYPRE_Int* hi, const HYPRE_Real** coef) {
    lo[0] = A->grid.lo[0];
    lo[1] = A->grid.lo[1];
    hi[0] = A->grid.hi[0];
    hi[1] = A->grid.hi[1];
    *coef = A->coef.data();
    return (HYPRE_Int)(A->off.size() / 2);
}
HYPRE_Int impec_hypre_shim_vector(HYPRE_StructVector v, const HYPRE_Real** values) {
    *values = v->val.data();
    return (HYPRE_Int)v->val.size();
}
HYPRE_Int impec_hypre_shim_solves(void) { return g_solves; }
