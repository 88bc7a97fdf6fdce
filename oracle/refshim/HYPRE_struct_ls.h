/*
 * Stand-in for HYPRE 2.8.0b's struct interface -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference solves its pressure and Crank-Nicolson systems with HYPRE (PCG + SMG,
 * src/MGSolver.cpp:594-667).  HYPRE is not part of the reference's sources, so the reference
 * build under oracle/_ref links this stand-in instead.  It keeps what the reference defines:
 * the grid box, the 9-entry stencil and every coefficient and right-hand-side value the
 * reference sets, which the reference build reads back to compare the assembled systems with
 * the oracle's.  The solvers (PCG, SMG, Jacobi) all become one direct banded-LU solve of the
 * recorded system; the reported iteration count is 1 and the final relative residual is the
 * true ||b - A x|| / ||b|| of that solve.  Couplings to cells outside the grid box count as
 * zero, as in HYPRE.
 */
#ifndef IMPEC_REFSHIM_HYPRE_STRUCT_LS_H
#define IMPEC_REFSHIM_HYPRE_STRUCT_LS_H

#include "_hypre_utilities.h"
#include "mpi.h"

typedef struct impec_hypre_grid* HYPRE_StructGrid;
typedef struct impec_hypre_stencil* HYPRE_StructStencil;
typedef struct impec_hypre_matrix* HYPRE_StructMatrix;
typedef struct impec_hypre_vector* HYPRE_StructVector;
typedef struct impec_hypre_solver* HYPRE_StructSolver;
typedef HYPRE_Int (*HYPRE_PtrToStructSolverFcn)(HYPRE_StructSolver, HYPRE_StructMatrix, HYPRE_StructVector,
                                                HYPRE_StructVector);

HYPRE_Int HYPRE_StructGridCreate(MPI_Comm, HYPRE_Int ndim, HYPRE_StructGrid* grid);
HYPRE_Int HYPRE_StructGridSetExtents(HYPRE_StructGrid grid, HYPRE_Int* ilower, HYPRE_Int* iupper);
HYPRE_Int HYPRE_StructGridAssemble(HYPRE_StructGrid grid);
HYPRE_Int HYPRE_StructGridDestroy(HYPRE_StructGrid grid);

HYPRE_Int HYPRE_StructStencilCreate(HYPRE_Int ndim, HYPRE_Int size, HYPRE_StructStencil* stencil);
HYPRE_Int HYPRE_StructStencilSetElement(HYPRE_StructStencil stencil, HYPRE_Int entry, HYPRE_Int* offset);
HYPRE_Int HYPRE_StructStencilDestroy(HYPRE_StructStencil stencil);

HYPRE_Int HYPRE_StructMatrixCreate(MPI_Comm, HYPRE_StructGrid grid, HYPRE_StructStencil stencil, HYPRE_StructMatrix* A);
HYPRE_Int HYPRE_StructMatrixInitialize(HYPRE_StructMatrix A);
HYPRE_Int HYPRE_StructMatrixSetValues(HYPRE_StructMatrix A, HYPRE_Int* index, HYPRE_Int nentries, HYPRE_Int* entries,
                                      HYPRE_Real* values);
HYPRE_Int HYPRE_StructMatrixAssemble(HYPRE_StructMatrix A);
HYPRE_Int HYPRE_StructMatrixDestroy(HYPRE_StructMatrix A);

HYPRE_Int HYPRE_StructVectorCreate(MPI_Comm, HYPRE_StructGrid grid, HYPRE_StructVector* v);
HYPRE_Int HYPRE_StructVectorInitialize(HYPRE_StructVector v);
HYPRE_Int HYPRE_StructVectorSetValues(HYPRE_StructVector v, HYPRE_Int* index, HYPRE_Real value);
HYPRE_Int HYPRE_StructVectorSetBoxValues(HYPRE_StructVector v, HYPRE_Int* ilower, HYPRE_Int* iupper, HYPRE_Real* values);
HYPRE_Int HYPRE_StructVectorGetValues(HYPRE_StructVector v, HYPRE_Int* index, HYPRE_Real* value);
HYPRE_Int HYPRE_StructVectorAssemble(HYPRE_StructVector v);
HYPRE_Int HYPRE_StructVectorDestroy(HYPRE_StructVector v);

HYPRE_Int HYPRE_StructPCGCreate(MPI_Comm, HYPRE_StructSolver* s);
HYPRE_Int HYPRE_StructPCGDestroy(HYPRE_StructSolver s);
HYPRE_Int HYPRE_StructPCGSetMaxIter(HYPRE_StructSolver s, HYPRE_Int n);
HYPRE_Int HYPRE_StructPCGSetTol(HYPRE_StructSolver s, HYPRE_Real tol);
HYPRE_Int HYPRE_StructPCGSetTwoNorm(HYPRE_StructSolver s, HYPRE_Int on);
HYPRE_Int HYPRE_StructPCGSetRelChange(HYPRE_StructSolver s, HYPRE_Int on);
HYPRE_Int HYPRE_StructPCGSetPrintLevel(HYPRE_StructSolver s, HYPRE_Int level);
HYPRE_Int HYPRE_StructPCGSetLogging(HYPRE_StructSolver s, HYPRE_Int level);
HYPRE_Int HYPRE_StructPCGSetPrecond(HYPRE_StructSolver s, HYPRE_PtrToStructSolverFcn solve,
                                    HYPRE_PtrToStructSolverFcn setup, HYPRE_StructSolver precond);
HYPRE_Int HYPRE_StructPCGSetup(HYPRE_StructSolver s, HYPRE_StructMatrix A, HYPRE_StructVector b, HYPRE_StructVector x);
HYPRE_Int HYPRE_StructPCGSolve(HYPRE_StructSolver s, HYPRE_StructMatrix A, HYPRE_StructVector b, HYPRE_StructVector x);
HYPRE_Int HYPRE_StructPCGGetNumIterations(HYPRE_StructSolver s, HYPRE_Int* n);
HYPRE_Int HYPRE_StructPCGGetFinalRelativeResidualNorm(HYPRE_StructSolver s, HYPRE_Real* r);

HYPRE_Int HYPRE_StructSMGCreate(MPI_Comm, HYPRE_StructSolver* s);
HYPRE_Int HYPRE_StructSMGDestroy(HYPRE_StructSolver s);
HYPRE_Int HYPRE_StructSMGSetMemoryUse(HYPRE_StructSolver s, HYPRE_Int m);
HYPRE_Int HYPRE_StructSMGSetMaxIter(HYPRE_StructSolver s, HYPRE_Int n);
HYPRE_Int HYPRE_StructSMGSetTol(HYPRE_StructSolver s, HYPRE_Real tol);
HYPRE_Int HYPRE_StructSMGSetZeroGuess(HYPRE_StructSolver s);
HYPRE_Int HYPRE_StructSMGSetRelChange(HYPRE_StructSolver s, HYPRE_Int on);
HYPRE_Int HYPRE_StructSMGSetNumPreRelax(HYPRE_StructSolver s, HYPRE_Int n);
HYPRE_Int HYPRE_StructSMGSetNumPostRelax(HYPRE_StructSolver s, HYPRE_Int n);
HYPRE_Int HYPRE_StructSMGSetLogging(HYPRE_StructSolver s, HYPRE_Int level);
HYPRE_Int HYPRE_StructSMGSetup(HYPRE_StructSolver s, HYPRE_StructMatrix A, HYPRE_StructVector b, HYPRE_StructVector x);
HYPRE_Int HYPRE_StructSMGSolve(HYPRE_StructSolver s, HYPRE_StructMatrix A, HYPRE_StructVector b, HYPRE_StructVector x);
HYPRE_Int HYPRE_StructSMGGetNumIterations(HYPRE_StructSolver s, HYPRE_Int* n);
HYPRE_Int HYPRE_StructSMGGetFinalRelativeResidualNorm(HYPRE_StructSolver s, HYPRE_Real* r);

HYPRE_Int HYPRE_StructJacobiCreate(MPI_Comm, HYPRE_StructSolver* s);
HYPRE_Int HYPRE_StructJacobiDestroy(HYPRE_StructSolver s);
HYPRE_Int HYPRE_StructJacobiSetTol(HYPRE_StructSolver s, HYPRE_Real tol);
HYPRE_Int HYPRE_StructJacobiSetMaxIter(HYPRE_StructSolver s, HYPRE_Int n);
HYPRE_Int HYPRE_StructJacobiSetNonZeroGuess(HYPRE_StructSolver s);
HYPRE_Int HYPRE_StructJacobiSetup(HYPRE_StructSolver s, HYPRE_StructMatrix A, HYPRE_StructVector b, HYPRE_StructVector x);
HYPRE_Int HYPRE_StructJacobiSolve(HYPRE_StructSolver s, HYPRE_StructMatrix A, HYPRE_StructVector b, HYPRE_StructVector x);
HYPRE_Int HYPRE_StructJacobiGetNumIterations(HYPRE_StructSolver s, HYPRE_Int* n);
HYPRE_Int HYPRE_StructJacobiGetFinalRelativeResidualNorm(HYPRE_StructSolver s, HYPRE_Real* r);

/* ---- read-back for the reference build's driver (not HYPRE API) ---- */
/* Grid box of A and its coefficients: ncells x 9, cell (k,l) at (k-ilower0)*ny + (l-ilower1),
 * entries in the stencil's entry order. */
HYPRE_Int impec_hypre_shim_matrix(HYPRE_StructMatrix A, HYPRE_Int* ilower, HYPRE_Int* iupper, const HYPRE_Real** coef);
/* Values of v over its grid box, in the same cell order. */
HYPRE_Int impec_hypre_shim_vector(HYPRE_StructVector v, const HYPRE_Real** values);
/* Number of direct solves performed so far (all solvers). */
HYPRE_Int impec_hypre_shim_solves(void);

#endif
