// Pressure equation: mobility, operator assembly, multigrid solve, Darcy velocities.
//
// The reference assembles the nu-weighted 9-point (nu < 1) or 5-point (nu = 1) operator with
// Neumann folding and one Dirichlet pin at cell (1,1) (src/MGSolver.cpp:268-570) and solves
// it with HYPRE PCG + SMG (:594-629).  Here the same pinned system is solved as follows:
// every non-pinned row has zero row sum, so with b~ = b except b~(pin) = -sum_{k != pin} b(k)
// the singular Neumann system A_N x = b~ is consistent; any solution shifted by
// (p_pin - x_pin) satisfies all rows of the pinned system.  The consistent singular system is
// solved by geometric multigrid (cell-centred, Galerkin coarse operators from 2x2
// aggregation scaled by 1/2, red-black / four-colour Gauss-Seidel, summed restriction,
// bilinear prolongation, dense coarsest solve with one unknown fixed).
//
// Internally the operator is stored in integrated form with positive diagonal:
// A_int = -dA * A_ref, f = dA * q, so that ||f - A_int x|| / ||f|| equals the reference's
// relative residual ||b - A x|| / ||b||.
#include <cooperative_groups.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "internal.cuh"
#include "reduce.cuh"

namespace impec {

constexpr int BX = 32, BY = 8;
static inline dim3 grid2(int n1, int n2) { return dim3((n2 + BX - 1) / BX, (n1 + BY - 1) / BY); }
#define IX(i, j, n2) ((size_t)(i) * (n2) + (j))

// Tuning switches read from the environment (defaults are the measured best on GB300).
static long env_long(const char* name, long dflt) {
    const char* e = getenv(name);
    return e && *e ? strtol(e, nullptr, 10) : dflt;
}

// ---------------------------------------------------------------- mobility
// Cell value w = mu/K (harmonic averaging) or K/mu (arithmetic averaging), where
// mu(c) = 1/(x^4) * mu_res, x = 1 - c + M^(1/4) c   (src/EllipticSolver.cpp:692-695).
__global__ void k_cell_w(int n1, int n2, const double* __restrict__ c, const double* __restrict__ K1,
                         const double* __restrict__ K2, double m14, double mu_res, int harmonic,
                         double* __restrict__ w1, double* __restrict__ w2) {
    pdl_enter();
    int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    if (i >= n1 || j >= n2) return;
    size_t k = IX(i, j, n2);
    double cc = c[k];
    double x = __dadd_rn(1. - cc, __dmul_rn(m14, cc));  // no FMA: same rounding as the reference
    double mu = 1. / (x * x * x * x) * mu_res;
    double a = K1 ? K1[k] : 1.0;
    w1[k] = harmonic ? (K1 ? mu / a : mu) : (K1 ? a / mu : 1.0 / mu);
    if (w2) {
        double b = K2[k];
        w2[k] = harmonic ? mu / b : b / mu;
    }
}

// Face mobilities KoverMu_11_im12j / KoverMu_22_ijm12 (src/EllipticSolver.cpp:478-524),
// neighbours outside the grid mirrored (FillGhostCellsNeumannScalar).
__global__ void k_face_lam(int n1, int n2, const double* __restrict__ w1, const double* __restrict__ w2,
                           int harmonic, double* __restrict__ lamx, double* __restrict__ lamy) {
    pdl_enter();
    int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    if (i <= n1 && j < n2) {  // x-face between cells (i-1,j) and (i,j)
        double a = w1[IX(refl_cell(i - 1, n1), j, n2)], b = w1[IX(refl_cell(i, n1), j, n2)];
        lamx[IX(i, j, n2)] = harmonic ? 2. / (a + b) : 1. / 2 * (a + b);
    }
    if (i < n1 && j <= n2) {  // y-face between cells (i,j-1) and (i,j)
        double a = w2[IX(i, refl_cell(j - 1, n2), n2)], b = w2[IX(i, refl_cell(j, n2), n2)];
        lamy[IX(i, j, n2 + 1)] = harmonic ? 2. / (a + b) : 1. / 2 * (a + b);
    }
}

// Corner tensors of the rotated stencil.  Corner (ci,cj), ci in [0,n1], cj in [0,n2], sits at
// (ci-1/2, cj-1/2); its four cells are (ci-1..ci, cj-1..cj), mirrored at the boundary.
// KoverMu_*_ip12jp12 (src/EllipticSolver.cpp:697-754), GetTransformedMobilityTensor
// (src/MGSolver.cpp:807-841) and M_im12j (src/EllipticSolver.cpp:554-562).
__global__ void k_corner(int n1, int n2, const double* __restrict__ w1, const double* __restrict__ w2,
                         int harmonic, Geo G, double* __restrict__ m11, double* __restrict__ m22,
                         double* __restrict__ m12) {
    pdl_enter();
    int cj = blockIdx.x * BX + threadIdx.x, ci = blockIdx.y * BY + threadIdx.y;
    if (ci > n1 || cj > n2) return;
    const int i = ci - 1, j = cj - 1;  // reference corner (i+1/2, j+1/2)
    const int a0 = refl_cell(i, n1), a1 = refl_cell(i + 1, n1), b0 = refl_cell(j, n2), b1 = refl_cell(j + 1, n2);
    // order of the reference sum: (ip1j + ij) + ijp1 + ip1jp1
    double s1 = w1[IX(a1, b0, n2)] + w1[IX(a0, b0, n2)] + w1[IX(a0, b1, n2)] + w1[IX(a1, b1, n2)];
    double s2 = w2[IX(a1, b0, n2)] + w2[IX(a0, b0, n2)] + w2[IX(a0, b1, n2)] + w2[IX(a1, b1, n2)];
    double K11 = harmonic ? 4. / s1 : 1. / 4 * s1;
    double K22 = harmonic ? 4. / s2 : 1. / 4 * s2;
    size_t k = IX(ci, cj, n2 + 1);
    m11[k] = G.secamt2 * (K11 * G.cosa2 + K22 * G.sina2);
    m22[k] = G.secamt2 * (K22 * G.cost2 + K11 * G.sint2);
    m12[k] = G.secamt2 * (K22 * G.costsina - K11 * G.cosasint);
}

// ---------------------------------------------------------------- fine operators
// nu = 1: face transmissibilities dA/dx^2 * lambda with zero flux through the boundary.
// tx32 / ty32 (or nullptr): their FP32 copies for the mixed-precision cycle.
// Diagonal of a five-point cell from its four faces, in k_idiag's order, and its reciprocal
// (with the FP32 copies of the mixed-precision cycle when asked).
__device__ __forceinline__ void store_diag5(size_t k, double tw, double te, double ts, double tn,
                                            double* __restrict__ diag, double* __restrict__ idiag,
                                            float* __restrict__ diag32, float* __restrict__ idiag32) {
    const double d = tw + te + ts + tn;
    const double id = d != 0.0 ? 1.0 / d : 0.0;
    diag[k] = d;
    idiag[k] = id;
    if (diag32) diag32[k] = (float)d;
    if (idiag32) idiag32[k] = (float)id;
}

// Finest five-point faces t = lambda * dA / h^2 (boundary faces 0).  With diag != null (no
// Dirichlet row, which changes the faces afterwards) the kernel also writes the diagonal and its
// reciprocal, recomputing the east and north faces of its cell: the separate k_idiag launch of
// this level is then not needed, and the values are the same bit for bit.
__global__ void k_face5_fine(int n1, int n2, const double* __restrict__ lamx, const double* __restrict__ lamy,
                             double sx, double sy, double* __restrict__ tx, double* __restrict__ ty,
                             float* __restrict__ tx32, float* __restrict__ ty32, double* __restrict__ diag,
                             double* __restrict__ idiag, float* __restrict__ diag32, float* __restrict__ idiag32) {
    pdl_enter();
    int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    auto fx = [&](int a, int b) { return (a == 0 || a == n1) ? 0.0 : lamx[IX(a, b, n2)] * sx; };
    auto fy = [&](int a, int b) { return (b == 0 || b == n2) ? 0.0 : lamy[IX(a, b, n2 + 1)] * sy; };
    if (i <= n1 && j < n2) {
        const double t = fx(i, j);
        tx[IX(i, j, n2)] = t;
        if (tx32) tx32[IX(i, j, n2)] = (float)t;
    }
    if (i < n1 && j <= n2) {
        const double t = fy(i, j);
        ty[IX(i, j, n2 + 1)] = t;
        if (ty32) ty32[IX(i, j, n2 + 1)] = (float)t;
    }
    if (diag && i < n1 && j < n2)
        store_diag5(IX(i, j, n2), fx(i, j), fx(i + 1, j), fy(i, j), fy(i, j + 1), diag, idiag, diag32, idiag32);
}

// Reference row (C,W,SW,S,SE,E,NE,N,NW) of GetWeightedMatrixCoefficientsForCell
// (src/MGSolver.cpp:710-804) with the Neumann folding of :304-515.
__device__ void ref_row(int i, int j, int n1, int n2, const double* __restrict__ lamx,
                        const double* __restrict__ lamy, const double* __restrict__ m11,
                        const double* __restrict__ m22, const double* __restrict__ m12, double nu, const Geo& G,
                        double* o) {
    const double dx = G.dx, dy = G.dy, dxi = G.dxi, deta = G.deta;
    // parallel (five-point) part
    double K11_im = lamx[IX(i, j, n2)], K11_ip = lamx[IX(i + 1, j, n2)];
    double K22_jm = lamy[IX(i, j, n2 + 1)], K22_jp = lamy[IX(i, j + 1, n2 + 1)];
    double Wp = 1. / (dx * dx) * K11_im, Ep = 1. / (dx * dx) * K11_ip;
    double Sp = 1. / (dy * dy) * K22_jm, Np = 1. / (dy * dy) * K22_jp;
    double Cp = -1. / (dy * dy) * (K22_jm + K22_jp) - 1. / (dx * dx) * (K11_im + K11_ip);
    // diagonal (rotated nine-point) part; corners (i+1/2,j+1/2) -> (i+1,j+1) etc.
    const int w = n2 + 1;
    double M11_ip12j = m11[IX(i + 1, j + 1, w)], M11_im12j = m11[IX(i, j, w)];
    double M22_ijp12 = m22[IX(i, j + 1, w)], M22_ijm12 = m22[IX(i + 1, j, w)];
    double M12_ip12j = m12[IX(i + 1, j + 1, w)], M21_ijp12 = m12[IX(i, j + 1, w)];
    double M12_im12j = m12[IX(i, j, w)], M21_ijm12 = m12[IX(i + 1, j, w)];
    double NEd = M11_ip12j / (dxi * dxi), SWd = M11_im12j / (dxi * dxi);
    double NWd = M22_ijp12 / (deta * deta), SEd = M22_ijm12 / (deta * deta);
    double Cd = -1. / (dxi * dxi) * (M11_ip12j + M11_im12j) - 1. / (deta * deta) * (M22_ijp12 + M22_ijm12);
    double Nd = 1. / (deta * dxi) * (M12_ip12j + M21_ijp12);
    double Wd = -1. / (deta * dxi) * (M21_ijp12 + M12_im12j);
    double Ed = -1. / (deta * dxi) * (M12_ip12j + M21_ijm12);
    double Sd = 1. / (deta * dxi) * (M12_im12j + M21_ijm12);
    double C = nu * Cp + (1 - nu) * Cd, W = nu * Wp + (1 - nu) * Wd, SW = nu * 0.0 + (1 - nu) * SWd;
    double S = nu * Sp + (1 - nu) * Sd, SE = nu * 0.0 + (1 - nu) * SEd, E = nu * Ep + (1 - nu) * Ed;
    double NE = nu * 0.0 + (1 - nu) * NEd, N = nu * Np + (1 - nu) * Nd, NW = nu * 0.0 + (1 - nu) * NWd;
    double s[9] = {C, W, SW, S, SE, E, NE, N, NW};
    for (int e = 0; e < 9; ++e) o[e] = s[e];
    const int k = i, l = j;
    auto set = [&](double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7, double a8) {
        o[0] = a0; o[1] = a1; o[2] = a2; o[3] = a3; o[4] = a4; o[5] = a5; o[6] = a6; o[7] = a7; o[8] = a8;
    };
    if (l == 0) set(C + S, W + SW, 0, 0, 0, E + SE, NE, N, NW);
    if (l == n2 - 1) set(C + N, W + NW, SW, S, SE, E + NE, 0, 0, 0);
    if (k == 0) set(C + W, 0, 0, S + SW, SE, E, NE, N + NW, 0);
    if (k == n1 - 1) set(C + E, W, SW, S + SE, 0, 0, 0, N + NE, NW);
    if (k == 0 && l == 0) set(C + W + S + SW, 0, 0, 0, 0, E + SE, NE, N + NW, 0);
    if (k == 0 && l == n2 - 1) set(C + W + N + NW, 0, 0, S + SW, SE, E + NE, 0, 0, 0);
    if (k == n1 - 1 && l == n2 - 1) set(C + N + NE + E, W + NW, SW, S + SE, 0, 0, 0, 0, 0);
    if (k == n1 - 1 && l == 0) set(C + S + E + SE, W + SW, 0, 0, 0, 0, 0, N + NE, NW);
}

__global__ void k_exp9_fine(int n1, int n2, const double* __restrict__ lamx, const double* __restrict__ lamy,
                            const double* __restrict__ m11, const double* __restrict__ m22,
                            const double* __restrict__ m12, double nu, Geo G, double* __restrict__ a9) {
    pdl_enter();
    int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    if (i >= n1 || j >= n2) return;
    double o[9];
    ref_row(i, j, n1, n2, lamx, lamy, m11, m22, m12, nu, G, o);
    const size_t n = (size_t)n1 * n2, k = IX(i, j, n2);
    for (int e = 0; e < 9; ++e) a9[e * n + k] = -G.dA * o[e];
}

// Stencil offsets in HYPRE entry order (src/MGSolver.cpp:164-166).
__constant__ int c_off[9][2] = {{0, 0}, {-1, 0}, {-1, -1}, {0, -1}, {1, -1}, {1, 0}, {1, 1}, {0, 1}, {-1, 1}};

// ---------------------------------------------------------------- coarse operators
// Coarse five-point faces (half the sum of the two fine faces they cover).  With diag != null
// (no extra diagonal from a Dirichlet row) the kernel also writes the coarse diagonal and its
// reciprocal from recomputed faces, in place of the level's k_idiag launch (same values).
__global__ void k_face5_coarsen(int n1f, int n2f, const double* __restrict__ txf, const double* __restrict__ tyf,
                                int n1c, int n2c, double* __restrict__ txc, double* __restrict__ tyc,
                                float* __restrict__ txc32, float* __restrict__ tyc32, double* __restrict__ diag,
                                double* __restrict__ idiag, float* __restrict__ diag32, float* __restrict__ idiag32) {
    pdl_enter();
    int J = blockIdx.x * BX + threadIdx.x, I = blockIdx.y * BY + threadIdx.y;
    auto cx = [&](int a, int b) {  // coarse x-face (a, b)
        int fi = 2 * a;
        double s = 0.0;
        if (fi <= n1f) {
            s = txf[IX(fi, 2 * b, n2f)];
            if (2 * b + 1 < n2f) s += txf[IX(fi, 2 * b + 1, n2f)];
        }
        return 0.5 * s;
    };
    auto cy = [&](int a, int b) {  // coarse y-face (a, b)
        int fj = 2 * b;
        double s = 0.0;
        if (fj <= n2f) {
            s = tyf[IX(2 * a, fj, n2f + 1)];
            if (2 * a + 1 < n1f) s += tyf[IX(2 * a + 1, fj, n2f + 1)];
        }
        return 0.5 * s;
    };
    if (I <= n1c && J < n2c) {
        const double t = cx(I, J);
        txc[IX(I, J, n2c)] = t;
        if (txc32) txc32[IX(I, J, n2c)] = (float)t;
    }
    if (I < n1c && J <= n2c) {
        const double t = cy(I, J);
        tyc[IX(I, J, n2c + 1)] = t;
        if (tyc32) tyc32[IX(I, J, n2c + 1)] = (float)t;
    }
    if (diag && I < n1c && J < n2c)
        store_diag5(IX(I, J, n2c), cx(I, J), cx(I + 1, J), cy(I, J), cy(I, J + 1), diag, idiag, diag32, idiag32);
}

__global__ void k_exp9_coarsen(int n1f, int n2f, const double* __restrict__ af, const unsigned char* __restrict__ maskf,
                               int n1c, int n2c, double* __restrict__ ac) {
    pdl_enter();
    int J = blockIdx.x * BX + threadIdx.x, I = blockIdx.y * BY + threadIdx.y;
    if (I >= n1c || J >= n2c) return;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const size_t nf = (size_t)n1f * n2f;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) {
            int i = 2 * I + a, j = 2 * J + b;
            if (i >= n1f || j >= n2f) continue;
            if (maskf && maskf[IX(i, j, n2f)]) continue;  // known cells are not unknowns of the coarse problem
            for (int e = 0; e < 9; ++e) {
                int ii = i + c_off[e][0], jj = j + c_off[e][1];
                if (ii < 0 || ii >= n1f || jj < 0 || jj >= n2f) continue;
                double val = af[e * nf + IX(i, j, n2f)];
                int dI = (ii >> 1) - I, dJ = (jj >> 1) - J;
                int ec = 0;
                for (int q = 0; q < 9; ++q)
                    if (c_off[q][0] == dI && c_off[q][1] == dJ) ec = q;
                acc[ec] += val;
            }
        }
    const size_t nc = (size_t)n1c * n2c;
    for (int e = 0; e < 9; ++e) ac[e * nc + IX(I, J, n2c)] = 0.5 * acc[e];
}

// Coarse extra diagonal: half the sum over the 2x2 children (Galerkin product with piecewise
// constant transfer, scaled by 1/2, of the couplings moved to the diagonal).
__global__ void k_ed_coarsen(int n1f, int n2f, const double* __restrict__ edf, int n1c, int n2c,
                             double* __restrict__ edc) {
    pdl_enter();
    int J = blockIdx.x * BX + threadIdx.x, I = blockIdx.y * BY + threadIdx.y;
    if (I >= n1c || J >= n2c) return;
    double s = 0.0;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) {
            const int i = 2 * I + a, j = 2 * J + b;
            if (i < n1f && j < n2f) s += edf[IX(i, j, n2f)];
        }
    edc[IX(I, J, n2c)] = 0.5 * s;
}

// Dirichlet row of the horizontal source (cells (dr, j), row kappa/dA p = -q,
// src/MGSolver.cpp:119-140, 518-567): the known values x_d = -q_d dA / kappa are moved to the
// right-hand sides of their neighbours and the couplings to them removed, which leaves an SPD
// system in the unknowns.  Five-point operator: each removed face joins the neighbour's
// diagonal (ed); one thread per column j.
__global__ void k_dirichlet_face5(int n1, int n2, int dr, const double* __restrict__ q, double dA, double kappa,
                                  double* __restrict__ tx, double* __restrict__ ty, double* __restrict__ ed,
                                  double* __restrict__ fd, unsigned char* __restrict__ mask) {
    pdl_enter();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n2) return;
    const size_t kd = IX(dr, j, n2);
    const double xd = -q[kd] * dA / kappa;
    mask[kd] = 1;
    fd[kd] = xd;
    if (dr > 0) {
        const double t = tx[IX(dr, j, n2)];
        ed[IX(dr - 1, j, n2)] += t;
        fd[IX(dr - 1, j, n2)] += t * xd;
        tx[IX(dr, j, n2)] = 0.0;
    }
    if (dr < n1 - 1) {
        const double t = tx[IX(dr + 1, j, n2)];
        ed[IX(dr + 1, j, n2)] += t;
        fd[IX(dr + 1, j, n2)] += t * xd;
        tx[IX(dr + 1, j, n2)] = 0.0;
    }
    ty[IX(dr, j, n2 + 1)] = 0.0;
    if (j == n2 - 1) ty[IX(dr, n2, n2 + 1)] = 0.0;
}

// Nine-point operator: rows dr-1 and dr+1 drop their entries towards row dr (the value moves to
// fd); the known row becomes x = fd.  One thread per cell of rows dr-1 .. dr+1.
__global__ void k_dirichlet_exp9(int n1, int n2, int dr, const double* __restrict__ q, double dA, double kappa,
                                 double* __restrict__ a9, double* __restrict__ fd, unsigned char* __restrict__ mask) {
    pdl_enter();
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = dr - 1 + (int)blockIdx.y;
    if (j >= n2 || i < 0 || i >= n1) return;
    const size_t n = (size_t)n1 * n2, k = IX(i, j, n2);
    if (i == dr) {
        mask[k] = 1;
        fd[k] = -q[k] * dA / kappa;
        a9[k] = 1.0;
        for (int e = 1; e < 9; ++e) a9[e * n + k] = 0.0;
        return;
    }
    double add = 0.0;
    for (int e = 1; e < 9; ++e) {
        const int ii = i + c_off[e][0], jj = j + c_off[e][1];
        if (ii != dr || jj < 0 || jj >= n2) continue;
        add -= a9[e * n + k] * (-q[IX(dr, jj, n2)] * dA / kappa);
        a9[e * n + k] = 0.0;
    }
    fd[k] = add;
}

// f := f + fd on unknown cells, f := the known value on known cells; x := the known value there.
__global__ void k_dirichlet_rhs(size_t n, double* __restrict__ f, double* __restrict__ x,
                                const double* __restrict__ fd, const unsigned char* __restrict__ mask) {
    pdl_enter();
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        if (mask[k]) {
            f[k] = fd[k];
            x[k] = fd[k];
        } else {
            f[k] += fd[k];
        }
    }
}

__global__ void k_idiag(int n1, int n2, int kind, const double* __restrict__ tx, const double* __restrict__ ty,
                        const double* __restrict__ a9, const double* __restrict__ ed,
                        const unsigned char* __restrict__ mask, double* __restrict__ diag, double* __restrict__ idiag,
                        float* __restrict__ diag32, float* __restrict__ idiag32) {
    pdl_enter();
    int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    if (i >= n1 || j >= n2) return;
    double d;
    if (kind == FACE5) {
        d = tx[IX(i, j, n2)] + tx[IX(i + 1, j, n2)] + ty[IX(i, j, n2 + 1)] + ty[IX(i, j + 1, n2 + 1)];
        if (ed) d += ed[IX(i, j, n2)];
    } else {
        d = a9[IX(i, j, n2)];
    }
    if (mask && mask[IX(i, j, n2)]) d = 1.0;  // known cell: x = rhs
    const double id = d != 0.0 ? 1.0 / d : 0.0;
    diag[IX(i, j, n2)] = d;
    idiag[IX(i, j, n2)] = id;
    if (diag32) diag32[IX(i, j, n2)] = (float)d;  // FP32 copies for the mixed-precision cycle
    if (idiag32) idiag32[IX(i, j, n2)] = (float)id;
}

__global__ void k_to_float(size_t n, const double* __restrict__ a, float* __restrict__ b) {
    pdl_enter();
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        b[k] = (float)a[k];
}

// ---------------------------------------------------------------- operator application
template <class T>
__device__ __forceinline__ T apply_face5(int i, int j, int n1, int n2, const T* __restrict__ tx,
                                         const T* __restrict__ ty, const T* __restrict__ x, T& diag, T& offsum) {
    T tw = tx[IX(i, j, n2)], te = tx[IX(i + 1, j, n2)], ts = ty[IX(i, j, n2 + 1)], tn = ty[IX(i, j + 1, n2 + 1)];
    T s = 0;
    if (i > 0) s += tw * x[IX(i - 1, j, n2)];
    if (i < n1 - 1) s += te * x[IX(i + 1, j, n2)];
    if (j > 0) s += ts * x[IX(i, j - 1, n2)];
    if (j < n2 - 1) s += tn * x[IX(i, j + 1, n2)];
    diag = tw + te + ts + tn;
    offsum = s;
    return diag * x[IX(i, j, n2)] - s;
}

template <class T>
__device__ __forceinline__ T offsum_exp9(int i, int j, int n1, int n2, const T* __restrict__ a9,
                                         const T* __restrict__ x) {
    const size_t n = (size_t)n1 * n2, k = IX(i, j, n2);
    T s = 0;
#pragma unroll
    for (int e = 1; e < 9; ++e) {
        int ii = i + c_off[e][0], jj = j + c_off[e][1];
        if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
        s += a9[e * n + k] * x[IX(ii, jj, n2)];
    }
    return s;
}

// ---------------------------------------------------------------- smoothers
// One colour of a red-black sweep.  Each thread updates two cells of the colour, RB_ROWS * BY /
// 2 rows apart, with all loads issued before either update: the FP64 pipe, not load latency,
// then sets the pace.  The arithmetic per cell is s = b + sum t * x_nb, x = s * idiag.
constexpr int RB_ROWS = 2;

template <class T>
__global__ void k_rb_face5(int n1, int n2, const T* __restrict__ tx, const T* __restrict__ ty,
                           const T* __restrict__ idiag, const T* __restrict__ b, T* __restrict__ x, int color) {
    pdl_enter();
    const int jj = blockIdx.x * BX + threadIdx.x, i0 = blockIdx.y * (RB_ROWS * BY) + threadIdx.y;
    T v[RB_ROWS];
#pragma unroll
    for (int r = 0; r < RB_ROWS; ++r) {
        const int i = i0 + r * BY, j = 2 * jj + ((i + color) & 1);
        if (i >= n1 || j >= n2) continue;
        T s = b[IX(i, j, n2)];
        if (i > 0) s += tx[IX(i, j, n2)] * x[IX(i - 1, j, n2)];
        if (i < n1 - 1) s += tx[IX(i + 1, j, n2)] * x[IX(i + 1, j, n2)];
        if (j > 0) s += ty[IX(i, j, n2 + 1)] * x[IX(i, j - 1, n2)];
        if (j < n2 - 1) s += ty[IX(i, j + 1, n2 + 1)] * x[IX(i, j + 1, n2)];
        v[r] = s * idiag[IX(i, j, n2)];
    }
#pragma unroll
    for (int r = 0; r < RB_ROWS; ++r) {
        const int i = i0 + r * BY, j = 2 * jj + ((i + color) & 1);
        if (i < n1 && j < n2) x[IX(i, j, n2)] = v[r];
    }
}

// The first colour of a sweep that starts from x = 0: every neighbour term of k_rb_face5 is
// zero, so s = b and x = b * idiag.  The second colour reads only this colour's cells, so the
// iterate needs no zero fill beforehand.
template <class T>
__global__ void k_rb_zero(int n1, int n2, const T* __restrict__ idiag, const T* __restrict__ b,
                          T* __restrict__ x, int color) {
    pdl_enter();
    const int jj = blockIdx.x * BX + threadIdx.x, i0 = blockIdx.y * (RB_ROWS * BY) + threadIdx.y;
#pragma unroll
    for (int r = 0; r < RB_ROWS; ++r) {
        const int i = i0 + r * BY, j = 2 * jj + ((i + color) & 1);
        if (i < n1 && j < n2) x[IX(i, j, n2)] = b[IX(i, j, n2)] * idiag[IX(i, j, n2)];
    }
}

// One whole red-black sweep in one launch (levels whose arrays stream from HBM).  A CTA owns a
// TILE_R x TILE_C tile.  Phase 1 updates the first colour F on the tile and a one-cell ring
// around it (the ring's values equal what the neighbouring tiles compute: same inputs, same
// arithmetic), from the other colour's old values in x_in; phase 2 updates the other colour
// on the tile from the phase-1 values in shared memory.  Both colours of the tile go to x_out.
// The other colour's old values of a tile's edge are read by its neighbours' phase 1, so the
// sweep cannot write in place: x_in and x_out are two buffers (ping-pong).  Each coefficient
// (b, 1/diag, tx, ty) is read once per sweep instead of once per colour, and x once, in whole
// sectors.  Per-cell arithmetic and its order equal k_rb_face5's, so the result is the same bit
// for bit.  ZERO: the sweep starts from x = 0 (as k_rb_zero), so phase 1 is x = b * idiag and
// x_in is not read.
// Asynchronous copy of one element, global -> this CTA's shared memory (cp.async of 4 or 8
// bytes: any element-aligned address qualifies).  A staging loop issues all of its copies
// before one cp.async.wait_all, instead of one global-load round trip per element.
template <class T>
__device__ __forceinline__ void stage_async(T* dst, const T* src) {
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "cp.async element");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src),
                 "n"(sizeof(T))
                 : "memory");
}
__device__ __forceinline__ void stage_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

constexpr int TILE_R = 32, TILE_C = 64, TILE_THREADS = 256;
constexpr int TILE_W = TILE_C + 4;  // shared row width: columns j0-2 .. j0+TILE_C+1

template <class T, bool ZERO>
__global__ void __launch_bounds__(TILE_THREADS) k_rb_tile(int n1, int n2, const T* __restrict__ tx,
                                                          const T* __restrict__ ty, const T* __restrict__ idiag,
                                                          const T* __restrict__ b, const T* __restrict__ x_in,
                                                          T* __restrict__ x_out, int first) {
    pdl_enter();
    // FP32 zero-start sweeps stage b (in place of x, which is not read, and overwritten colour
    // by colour) and 1/diag of the ring region; FP64 ones read them from global memory (staged,
    // the 4096^2 FP64 solve took 18.13 against 17.93 ms; FP32 13.99 against 14.28 ms)
    constexpr bool ZSTAGE = ZERO && sizeof(T) == 4;
    __shared__ T sx[(TILE_R + 4) * TILE_W];  // rows i0-2 .. i0+TILE_R+1
    __shared__ T sid[ZSTAGE ? (TILE_R + 4) * TILE_W : 1];  // 1/diag, indexed as sx
    const int i0 = blockIdx.y * TILE_R, j0 = blockIdx.x * TILE_C, t = threadIdx.x;
    auto S = [&](int i, int j) -> T& { return sx[(i - i0 + 2) * TILE_W + (j - j0 + 2)]; };
    auto SID = [&](int i, int j) -> T { return sid[ZSTAGE ? (i - i0 + 2) * TILE_W + (j - j0 + 2) : 0]; };
    if (!ZERO) {  // the iterate tile: every element copy in flight at once
        for (int k = t; k < (TILE_R + 4) * TILE_W; k += TILE_THREADS) {
            const int i = i0 - 2 + k / TILE_W, j = j0 - 2 + k % TILE_W;
            if (i >= 0 && i < n1 && j >= 0 && j < n2) stage_async(sx + k, x_in + IX(i, j, n2));
            else sx[k] = T(0);
        }
    } else if (ZSTAGE) {  // the ring region: rows i0-1 .. i0+TILE_R, columns j0-1 .. j0+TILE_C
        constexpr int RW = TILE_C + 2;
        for (int k = t; k < (TILE_R + 2) * RW; k += TILE_THREADS) {
            const int i = i0 - 1 + k / RW, j = j0 - 1 + k % RW;
            const int s = (i - i0 + 2) * TILE_W + (j - j0 + 2);
            if (i >= 0 && i < n1 && j >= 0 && j < n2) {
                stage_async(sx + s, b + IX(i, j, n2));
                stage_async(sid + (ZSTAGE ? s : 0), idiag + IX(i, j, n2));
            }
        }
    }
    if (!ZERO || ZSTAGE) {
        stage_wait();
        __syncthreads();
    }
    // phase 1: colour `first` on rows i0-1 .. i0+TILE_R, columns j0-1 .. j0+TILE_C
    constexpr int H1 = (TILE_C + 2) / 2;
    for (int k = t; k < (TILE_R + 2) * H1; k += TILE_THREADS) {
        const int i = i0 - 1 + k / H1;
        const int j = j0 - 1 + (((i + j0 - 1 + first) & 1)) + 2 * (k % H1);
        if (i < 0 || i >= n1 || j < 0 || j >= n2) continue;
        T v;
        if (ZERO) {
            v = ZSTAGE ? S(i, j) * SID(i, j) : b[IX(i, j, n2)] * idiag[IX(i, j, n2)];
        } else {
            T s = b[IX(i, j, n2)];
            if (i > 0) s += tx[IX(i, j, n2)] * S(i - 1, j);
            if (i < n1 - 1) s += tx[IX(i + 1, j, n2)] * S(i + 1, j);
            if (j > 0) s += ty[IX(i, j, n2 + 1)] * S(i, j - 1);
            if (j < n2 - 1) s += ty[IX(i, j + 1, n2 + 1)] * S(i, j + 1);
            v = s * idiag[IX(i, j, n2)];
        }
        S(i, j) = v;  // phase 1 reads only the other colour: no conflict
    }
    __syncthreads();
    // phase 2: the other colour on the tile, from the phase-1 values
    constexpr int H2 = TILE_C / 2;
    const int second = first ^ 1;
    for (int k = t; k < TILE_R * H2; k += TILE_THREADS) {
        const int i = i0 + k / H2;
        const int j = j0 + ((i + j0 + second) & 1) + 2 * (k % H2);
        if (i >= n1 || j >= n2) continue;
        T s = ZSTAGE ? S(i, j) : b[IX(i, j, n2)];  // staged: this colour's cells still hold b
        if (i > 0) s += tx[IX(i, j, n2)] * S(i - 1, j);
        if (i < n1 - 1) s += tx[IX(i + 1, j, n2)] * S(i + 1, j);
        if (j > 0) s += ty[IX(i, j, n2 + 1)] * S(i, j - 1);
        if (j < n2 - 1) s += ty[IX(i, j + 1, n2 + 1)] * S(i, j + 1);
        S(i, j) = s * (ZSTAGE ? SID(i, j) : idiag[IX(i, j, n2)]);  // phase 2 reads only colour `first`
    }
    __syncthreads();
    for (int k = t; k < TILE_R * TILE_C; k += TILE_THREADS) {
        const int i = i0 + k / TILE_C, j = j0 + k % TILE_C;
        if (i < n1 && j < n2) x_out[IX(i, j, n2)] = S(i, j);
    }
}

template <class T>
__global__ void k_gs4_exp9(int n1, int n2, const T* __restrict__ a9, const T* __restrict__ idiag,
                           const T* __restrict__ b, T* __restrict__ x, int ci, int cj) {
    pdl_enter();
    int j = 2 * (blockIdx.x * BX + threadIdx.x) + cj, i = 2 * (blockIdx.y * BY + threadIdx.y) + ci;
    if (i >= n1 || j >= n2) return;
    T s = b[IX(i, j, n2)] - offsum_exp9<T>(i, j, n1, n2, a9, x);
    x[IX(i, j, n2)] = s * idiag[IX(i, j, n2)];
}

// ---------------------------------------------------------------- transfers
// r = b - A x at (i, j) as one accumulation: s = b + sum t * x_nb (FACE5) or
// b - sum a_e * x_nb (EXP9), then r = s - diag * x.
template <class T>
__device__ __forceinline__ T resid(const Level& Lv, int i, int j, const T* __restrict__ tx, const T* __restrict__ ty,
                                   const T* __restrict__ a9, const T* __restrict__ dg, const T* __restrict__ b,
                                   const T* __restrict__ x) {
    const int n1 = Lv.n1, n2 = Lv.n2;
    const size_t k = IX(i, j, n2);
    T s = b[k];
    if (Lv.kind == FACE5) {
        if (i > 0) s += tx[k] * x[k - n2];
        if (i < n1 - 1) s += tx[k + n2] * x[k + n2];
        if (j > 0) s += ty[IX(i, j, n2 + 1)] * x[k - 1];
        if (j < n2 - 1) s += ty[IX(i, j + 1, n2 + 1)] * x[k + 1];
    } else {
        const size_t n = (size_t)n1 * n2;
#pragma unroll
        for (int e = 1; e < 9; ++e) {
            const int ii = i + c_off[e][0], jj = j + c_off[e][1];
            if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
            s -= a9[e * n + k] * x[IX(ii, jj, n2)];
        }
    }
    return s - dg[k] * x[k];
}

// Residual of the fine level summed over each 2x2 aggregate -> coarse rhs; coarse x := 0.
template <class T>
__global__ void k_restrict(Level F, const T* __restrict__ tx, const T* __restrict__ ty, const T* __restrict__ a9,
                           const T* __restrict__ dg, const T* __restrict__ b, const T* __restrict__ x, int n1c,
                           int n2c, T* __restrict__ bc, T* __restrict__ xc, int zero_color, const T* __restrict__ idc) {
    pdl_enter();
    int J = blockIdx.x * BX + threadIdx.x, I = blockIdx.y * BY + threadIdx.y;
    if (I >= n1c || J >= n2c) return;
    T s = 0;
    for (int a = 0; a < 2; ++a)
        for (int bb = 0; bb < 2; ++bb) {
            int i = 2 * I + a, j = 2 * J + bb;
            // zero_color >= 0: the red-black sweep just updated that colour, whose residual
            // s - diag (s / diag) is zero up to one rounding (resid() recomputes the same s)
            if (((i + j) & 1) == zero_color) continue;
            if (i < F.n1 && j < F.n2) s += resid<T>(F, i, j, tx, ty, a9, dg, b, x);
        }
    bc[IX(I, J, n2c)] = s;
    // The coarse cycle starts from x = 0.  Without idc that zero is written.  With idc (the
    // coarse 1/diag), the coarse pre-smoothing's first colour (red, as k_rb_zero:
    // x = b * idiag) is done here, and the black cells are left for its black pass to overwrite.
    if (!idc) xc[IX(I, J, n2c)] = 0;
    else if (((I + J) & 1) == 0) xc[IX(I, J, n2c)] = s * idc[IX(I, J, n2c)];
}

// Bilinear cell-centred prolongation (weights 9/16, 3/16, 3/16, 1/16; the outside
// neighbour is replaced by the cell itself), added to the fine iterate.
template <class T>
__device__ __forceinline__ T prolong_cell(int i, int j, int n2, const T* __restrict__ x, int n1c, int n2c,
                                          const T* __restrict__ xc) {
    int I = i >> 1, J = j >> 1;
    int I2 = (i & 1) ? I + 1 : I - 1, J2 = (j & 1) ? J + 1 : J - 1;
    if (I2 < 0 || I2 >= n1c) I2 = I;
    if (J2 < 0 || J2 >= n2c) J2 = J;
    T v = x[IX(i, j, n2)];
    v += T(0.5625) * xc[IX(I, J, n2c)];
    v += T(0.1875) * xc[IX(I2, J, n2c)];
    v += T(0.1875) * xc[IX(I, J2, n2c)];
    v += T(0.0625) * xc[IX(I2, J2, n2c)];
    return v;
}

template <class T>
__global__ void k_prolong(int n1, int n2, T* __restrict__ x, int n1c, int n2c, const T* __restrict__ xc,
                          const unsigned char* __restrict__ mask) {
    pdl_enter();
    int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    if (i >= n1 || j >= n2) return;
    if (mask && mask[IX(i, j, n2)]) return;  // known cells take no correction
    x[IX(i, j, n2)] = prolong_cell(i, j, n2, x, n1c, n2c, xc);
}

// The same correction on the cells of one colour only (threads mapped as k_rb_face5).  When a
// red-black sweep that starts with the other colour follows, that sweep overwrites the other
// colour's cells without reading them, so their correction would be dead work.
template <class T>
__global__ void k_prolong_rb(int n1, int n2, T* __restrict__ x, int n1c, int n2c, const T* __restrict__ xc,
                             const unsigned char* __restrict__ mask, int color) {
    pdl_enter();
    const int jj = blockIdx.x * BX + threadIdx.x, i0 = blockIdx.y * (RB_ROWS * BY) + threadIdx.y;
#pragma unroll
    for (int r = 0; r < RB_ROWS; ++r) {
        const int i = i0 + r * BY, j = 2 * jj + ((i + color) & 1);
        if (i >= n1 || j >= n2) continue;
        if (mask && mask[IX(i, j, n2)]) continue;
        x[IX(i, j, n2)] = prolong_cell(i, j, n2, x, n1c, n2c, xc);
    }
}

// ---------------------------------------------------------------- coarsest level (dense)
__global__ void k_dense_build(Level C, const double* __restrict__ tx, const double* __restrict__ ty,
                              const double* __restrict__ a9, int singular, double* __restrict__ D) {
    pdl_enter();
    const int n1 = C.n1, n2 = C.n2, n = n1 * n2;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        for (int cc = 0; cc < n; ++cc) D[(size_t)r * n + cc] = 0.0;
        int i = r / n2, j = r % n2;
        if (C.kind == FACE5) {
            double tw = tx[IX(i, j, n2)], te = tx[IX(i + 1, j, n2)], ts = ty[IX(i, j, n2 + 1)], tn = ty[IX(i, j + 1, n2 + 1)];
            D[(size_t)r * n + r] = C.diag[r];  // the faces' sum (+ couplings moved to the diagonal)
            if (i > 0) D[(size_t)r * n + IX(i - 1, j, n2)] = -tw;
            if (i < n1 - 1) D[(size_t)r * n + IX(i + 1, j, n2)] = -te;
            if (j > 0) D[(size_t)r * n + IX(i, j - 1, n2)] = -ts;
            if (j < n2 - 1) D[(size_t)r * n + IX(i, j + 1, n2)] = -tn;
        } else {
            for (int e = 0; e < 9; ++e) {
                int ii = i + c_off[e][0], jj = j + c_off[e][1];
                if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
                D[(size_t)r * n + IX(ii, jj, n2)] = a9[(size_t)e * n + r];
            }
        }
    }
    __syncthreads();
    if (singular && threadIdx.x == 0) {  // fix the constant mode: row 0 := e_0
        for (int cc = 0; cc < n; ++cc) D[cc] = 0.0;
        D[0] = 1.0;
    }
}

// Gauss-Jordan inversion of an n x n (n <= 64) diagonally dominant matrix in shared memory.
// singular: D is the pinned singular system (row 0 = e_0), whose coarse solution has its mean
// removed; the mean removal is linear, so it is folded into the stored matrix, which becomes
// (I - 1 1^T / n) D^-1: every column less its mean.
__global__ void k_dense_invert(int n, const double* __restrict__ D, double* __restrict__ Dinv, int singular) {
    pdl_enter();
    extern __shared__ double sm[];
    double* A = sm;          // n x n
    double* B = sm + n * n;  // n x n
    for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
        A[k] = D[k];
        B[k] = (k / n == k % n) ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int piv = 0; piv < n; ++piv) {
        double inv = 1.0 / A[piv * n + piv];
        __syncthreads();
        for (int cc = threadIdx.x; cc < n; cc += blockDim.x) {
            A[piv * n + cc] *= inv;
            B[piv * n + cc] *= inv;
        }
        __syncthreads();
        for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
            int r = k / n, cc = k % n;
            if (r == piv) continue;
            double f = A[r * n + piv];
            if (cc != piv) A[r * n + cc] -= f * A[piv * n + cc];
            B[r * n + cc] -= f * B[piv * n + cc];
        }
        __syncthreads();
        for (int r = threadIdx.x; r < n; r += blockDim.x)
            if (r != piv) A[r * n + piv] = 0.0;
        __syncthreads();
    }
    if (singular) {
        for (int cc = threadIdx.x; cc < n; cc += blockDim.x) {
            double m = 0;
            for (int r = 0; r < n; ++r) m += B[r * n + cc];
            m /= n;
            for (int r = 0; r < n; ++r) B[r * n + cc] -= m;
        }
        __syncthreads();
    }
    for (int k = threadIdx.x; k < n * n; k += blockDim.x) Dinv[k] = B[k];
}

// ---------------------------------------------------------------- fine residual, norms, rhs
// r = f - A x on the fine level (FP64); accumulates ||r||^2 over all cells except the pinned
// one; optionally stores r as FP32 for the mixed-precision correction cycle.
__global__ void __launch_bounds__(RED_THREADS) k_fine_resid(Level F, const double* __restrict__ f,
                                                            const double* __restrict__ x, int pin,
                                                            float* __restrict__ r32, double* __restrict__ r64,
                                                            double* partials, int mb, unsigned* counter,
                                                            double* out) {
    pdl_enter();
    double acc[1] = {0.0};
    for_cells(F.n1, F.n2, [&](int i, int j, size_t k) {
        double r = resid<double>(F, i, j, F.tx, F.ty, F.a9, F.diag, f, x);
        if (r64) r64[k] = r;
        if (r32) r32[k] = (float)r;  // consistent rhs of the singular correction equation
        if ((int)k == pin) r = 0.0;  // the pinned row of the reference system has zero residual
        acc[0] += r * r;
    });
    grid_reduce<1>(acc, 0u, partials, mb, counter, out);
}

// f = dA*q with sum and sum of squares.
__global__ void __launch_bounds__(RED_THREADS) k_rhs(size_t n, const double* __restrict__ q, double dA,
                                                     double* __restrict__ f, double* partials, int mb,
                                                     unsigned* counter, double* out) {
    pdl_enter();
    double acc[2] = {0.0, 0.0};
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        double v = dA * q[k];
        f[k] = v;
        acc[0] += v;
        acc[1] += v * v;
    }
    grid_reduce<2>(acc, 0u, partials, mb, counter, out);
}

// Consistent right-hand side and pinned value: f(pin) := -(sum f - f(pin));
// p_pin = -q_pin dA / kappa  (pinned row kappa/dA p = -q, src/MGSolver.cpp:553-565).
__global__ void k_fix_pin(double* f, const double* q, int pin, double dA, double kappa, DevScalars* S) {
    pdl_enter();
    double fp = f[pin];
    S->pin_value = -q[pin] * dA / kappa;
    f[pin] = -(S->fsum - fp);
}

__global__ void k_add_f32(size_t n, double* __restrict__ x, const float* __restrict__ e) {
    pdl_enter();
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        x[k] += (double)e[k];
}

__global__ void k_shift(size_t n, double* __restrict__ x, int pin, const DevScalars* S) {
    pdl_enter();
    double s = S->pin_value - x[pin];
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        x[k] += s;
}

// y = A_ref x (reference pinned matrix) from the device operator.
__global__ void k_apply_ref(Level F, const double* __restrict__ x, int pin, int dir_row, double dA, double kappa,
                            double* __restrict__ y) {
    pdl_enter();
    int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    if (i >= F.n1 || j >= F.n2) return;
    size_t k = IX(i, j, F.n2);
    if ((int)k == pin || i == dir_row) { y[k] = kappa / dA * x[k]; return; }
    double v;
    if (F.kind == FACE5) {
        double d, o;
        v = apply_face5<double>(i, j, F.n1, F.n2, F.tx, F.ty, x, d, o);
    } else {
        v = F.a9[k] * x[k] + offsum_exp9<double>(i, j, F.n1, F.n2, F.a9, x);
    }
    y[k] = -v / dA;
}

#include "mgfused.cuh"
#include "mgcluster.cuh"

constexpr size_t MG_COARSE_SMEM = 160 * 1024;
constexpr size_t MG_CLUSTER_SMEM = 200 * 1024;

// CTAs per cluster for k_cluster_vcycle: 16 where the device can co-schedule such a cluster
// with the kernel's shared memory, else 8, else 0 (the per-level path is used).
template <class T>
static int cluster_size_for(int want) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(want);
    cfg.blockDim = dim3(CL_THREADS);
    cfg.dynamicSmemBytes = MG_CLUSTER_SMEM;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = want;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int num = 0;
    if (cudaOccupancyMaxActiveClusters(&num, k_cluster_vcycle<T>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return num > 0 ? want : 0;
}

// ---------------------------------------------------------------- host orchestration

impec_status pressure_alloc(impec_ctx* ctx) {
    const impec_params& P = ctx->P;
    int n1 = P.N1, n2 = P.N2;
    const bool nine = P.nu < 1.0;
    const size_t nc = (size_t)(n1 + 1) * (n2 + 1);
    if (nine) {
        IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->cm11, nc * 8));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->cm22, nc * 8));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->cm12, nc * 8));
    }
    ctx->L.clear();
    for (int l = 0;; ++l) {
        Level Lv;
        Lv.n1 = n1;
        Lv.n2 = n2;
        Lv.kind = nine ? EXP9 : FACE5;
        const size_t n = Lv.n();
        if (Lv.kind == FACE5) {
            IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.tx, (size_t)(n1 + 1) * n2 * 8));
            IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.ty, (size_t)n1 * (n2 + 1) * 8));
            IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.tx32, (size_t)(n1 + 1) * n2 * 4));
            IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.ty32, (size_t)n1 * (n2 + 1) * 4));
        } else {
            IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.a9, n * 9 * 8));
            IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.a932, n * 9 * 4));
        }
        IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.idiag, n * 8));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.idiag32, n * 4));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.diag, n * 8));
        if (ctx->dir_row >= 0 && Lv.kind == FACE5) IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.ed, n * 8));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.diag32, n * 4));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.x, n * 8));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.b, n * 8));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.x32, n * 4));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.b32, n * 4));
        if (Lv.kind == FACE5) {
            IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.xa, n * 8));
            IMPEC_CUDA_TRY(cudaMalloc((void**)&Lv.xa32, n * 4));
        }
        ctx->L.push_back(Lv);
        const int cmax = (int)env_long("IMPEC_MG_COARSEST", 4);  // coarsest level: both sides <= cmax
        if (n1 <= cmax && n2 <= cmax) break;
        n1 = (n1 + 1) / 2;
        n2 = (n2 + 1) / 2;
    }
    ctx->dense_n = ctx->L.back().n1 * ctx->L.back().n2;
    {
        const size_t nf = ctx->L[0].n();
        IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->cg_x, nf * 8));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->cg_p, nf * 8));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->cg_q, nf * 8));
        IMPEC_CUDA_TRY(cudaMemset(ctx->cg_q, 0, nf * 8));
        ctx->krylov = (int)env_long("IMPEC_MG_KRYLOV", 1) != 0;
        Tuning& T = ctx->tune;
        if (ctx->L[0].kind != FACE5) {
            // weighted nine-point operators (nu < 1): V(1,1) preconditions CG best (1024^2 step:
            // 6.97 ms against 8.55 ms with V(2,2); 16 instead of 14 iterations)
            T.pre = 1;
            T.post = 1;
        }
        T.pre = env_long("IMPEC_MG_PRE", T.pre);
        T.post = env_long("IMPEC_MG_POST", T.post);
        T.cluster = env_long("IMPEC_MG_CLUSTER", T.cluster);
        T.cl_cells = env_long("IMPEC_MG_CL_CELLS", T.cl_cells);
        T.cl_cta0 = env_long("IMPEC_MG_CL_CTA0", T.cl_cta0);
        T.coarse_cells64 = env_long("IMPEC_MG_COARSE_CELLS64", T.coarse_cells64);
        T.coarse_cells32 = env_long("IMPEC_MG_COARSE_CELLS32", T.coarse_cells32);
        T.rb_skip = env_long("IMPEC_MG_RB_SKIP", T.rb_skip);
        T.rb_resid = env_long("IMPEC_MG_RB_RESID", T.rb_resid);
        T.tile_cells = env_long("IMPEC_MG_TILE_CELLS", T.tile_cells);
        T.tile_cells32 = env_long("IMPEC_MG_TILE_CELLS32", T.tile_cells32);
        ctx->cn_predict = env_long("IMPEC_CN_PREDICT", 1) != 0;
        if (ctx->dir_row >= 0) {
            IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->dmask, nf));
            IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->dfd, nf * 8));
        }
    }
    IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->dense_inv, (size_t)ctx->dense_n * ctx->dense_n * 8 * 2));
    IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_dense_invert, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 64 * 64 * 8));
    const int cs = (int)MG_COARSE_SMEM;
    IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_coarse_vcycle<double, FACE5>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs));
    IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_coarse_vcycle<double, EXP9>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs));
    IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_coarse_vcycle<float, FACE5>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs));
    IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_coarse_vcycle<float, EXP9>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs));
    const int cls = (int)MG_CLUSTER_SMEM;
    IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_cluster_vcycle<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, cls));
    IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_cluster_vcycle<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, cls));
    ctx->cl_size = 0;
    if (cudaFuncSetAttribute(k_cluster_vcycle<double>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
        cudaFuncSetAttribute(k_cluster_vcycle<float>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
        const int want = (int)env_long("IMPEC_MG_CL_CTAS", CL_MAX_CTAS);
        for (int cs = want < CL_MAX_CTAS ? want : CL_MAX_CTAS; cs >= 2 && !ctx->cl_size; cs /= 2)
            if (cluster_size_for<double>(cs) && cluster_size_for<float>(cs)) ctx->cl_size = cs;
    }
    cudaGetLastError();
    return IMPEC_OK;
}

void pressure_free(impec_ctx* ctx) {
    for (Level& Lv : ctx->L) {
        void* ps[] = {Lv.tx,   Lv.ty,   Lv.a9,   Lv.idiag,   Lv.diag,   Lv.ed,  Lv.x,   Lv.b,
                      Lv.tx32, Lv.ty32, Lv.a932, Lv.idiag32, Lv.diag32, Lv.x32, Lv.b32, Lv.xa, Lv.xa32};
        for (void* p : ps)
            if (p) cudaFree(p);
    }
    ctx->L.clear();
    void* ps[] = {ctx->cm11, ctx->cm22, ctx->cm12, ctx->dense_inv, ctx->cg_x, ctx->cg_p, ctx->cg_q, ctx->dmask, ctx->dfd};
    for (void* p : ps)
        if (p) cudaFree(p);
}

impec_status face_mobility(impec_ctx* ctx, const double* c) {
    const impec_params& P = ctx->P;
    const int n1 = P.N1, n2 = P.N2;
    const int harm = P.avgproc == IMPEC_HARMONIC;
    double* w2 = ctx->K22 ? ctx->muK22 : nullptr;
    ++ctx->nlaunch, launch_k(ctx->stream, k_cell_w, grid2(n1, n2), dim3(BX, BY), 0, n1, n2, c, ctx->K11, ctx->K22, ctx->G.mob1over4,
                                                               P.mu_res, harm, ctx->muK11, w2);
    IMPEC_LAUNCH_CHECK();
    const double* W2 = w2 ? w2 : ctx->muK11;
    ++ctx->nlaunch, launch_k(ctx->stream, k_face_lam, grid2(n1 + 1, n2 + 1), dim3(BX, BY), 0, n1, n2, ctx->muK11, W2, harm, ctx->lamx,
                                                                          ctx->lamy);
    IMPEC_LAUNCH_CHECK();
    if (P.nu < 1.0) {
        ++ctx->nlaunch, launch_k(ctx->stream, k_corner, grid2(n1 + 1, n2 + 1), dim3(BX, BY), 0, n1, n2, ctx->muK11, W2, harm, ctx->G,
                                                                            ctx->cm11, ctx->cm22, ctx->cm12);
        IMPEC_LAUNCH_CHECK();
    }
    return IMPEC_OK;
}

impec_status pressure_setup(impec_ctx* ctx, const double* c) {
    const impec_params& P = ctx->P;
    IMPEC_TRY(face_mobility(ctx, c));
    Level& F = ctx->L[0];
    const Geo& G = ctx->G;
    const bool mixed = P.precision == IMPEC_PREC_MIXED;
    // Dirichlet row (horizontal source): known cells out of the operator, their values into fd
    const bool dir = ctx->dir_row >= 0 && ctx->eliminate;
    // FP32 copies of the five-point faces written with the FP64 ones, except the finest
    // level's faces when the Dirichlet elimination changes them afterwards
    const bool f32 = mixed && F.kind == FACE5;
    if (F.kind == FACE5) {
        double sx = G.dA * (1. / (G.dx * G.dx)), sy = G.dA * (1. / (G.dy * G.dy));
        ++ctx->nlaunch, launch_k(ctx->stream, k_face5_fine, grid2(F.n1 + 1, F.n2 + 1), dim3(BX, BY), 0, F.n1, F.n2, ctx->lamx, ctx->lamy,
                                 sx, sy, F.tx, F.ty, f32 && !dir ? F.tx32 : nullptr, f32 && !dir ? F.ty32 : nullptr,
                                 dir ? nullptr : F.diag, dir ? nullptr : F.idiag,
                                 mixed && !dir ? F.diag32 : nullptr, mixed && !dir ? F.idiag32 : nullptr);
    } else {
        ++ctx->nlaunch, launch_k(ctx->stream, k_exp9_fine, grid2(F.n1, F.n2), dim3(BX, BY), 0, F.n1, F.n2, ctx->lamx, ctx->lamy, ctx->cm11,
                                                                         ctx->cm22, ctx->cm12, P.nu, G, F.a9);
    }
    IMPEC_LAUNCH_CHECK();
    const unsigned char* mask0 = dir ? ctx->dmask : nullptr;
    if (dir) {
        const size_t n = F.n();
        IMPEC_CUDA_TRY(cudaMemsetAsync(ctx->dmask, 0, n, ctx->stream));
        IMPEC_CUDA_TRY(cudaMemsetAsync(ctx->dfd, 0, n * 8, ctx->stream));
        if (F.kind == FACE5) {
            IMPEC_CUDA_TRY(cudaMemsetAsync(F.ed, 0, n * 8, ctx->stream));
            ++ctx->nlaunch, launch_k(ctx->stream, k_dirichlet_face5, (F.n2 + 127) / 128, 128, 0, F.n1, F.n2, ctx->dir_row,
                                     ctx->q, G.dA, ctx->pin_kappa, F.tx, F.ty, F.ed, ctx->dfd, ctx->dmask);
        } else {
            ++ctx->nlaunch, launch_k(ctx->stream, k_dirichlet_exp9, dim3((F.n2 + 127) / 128, 3), 128, 0, F.n1, F.n2,
                                     ctx->dir_row, ctx->q, G.dA, ctx->pin_kappa, F.a9, ctx->dfd, ctx->dmask);
        }
        IMPEC_LAUNCH_CHECK();
    }
    for (size_t l = 0; l + 1 < ctx->L.size(); ++l) {
        Level &A = ctx->L[l], &B = ctx->L[l + 1];
        if (A.kind == FACE5) {
            ++ctx->nlaunch, launch_k(ctx->stream, k_face5_coarsen, grid2(B.n1 + 1, B.n2 + 1), dim3(BX, BY), 0, A.n1, A.n2, A.tx, A.ty, B.n1,
                                     B.n2, B.tx, B.ty, f32 ? B.tx32 : nullptr, f32 ? B.ty32 : nullptr,
                                     dir ? nullptr : B.diag, dir ? nullptr : B.idiag,
                                     mixed && !dir ? B.diag32 : nullptr, mixed && !dir ? B.idiag32 : nullptr);
            if (dir)
                ++ctx->nlaunch, launch_k(ctx->stream, k_ed_coarsen, grid2(B.n1, B.n2), dim3(BX, BY), 0, A.n1, A.n2, A.ed,
                                         B.n1, B.n2, B.ed);
        } else {
            ++ctx->nlaunch, launch_k(ctx->stream, k_exp9_coarsen, grid2(B.n1, B.n2), dim3(BX, BY), 0, A.n1, A.n2, A.a9,
                                     l == 0 ? mask0 : nullptr, B.n1, B.n2, B.a9);
        }
        IMPEC_LAUNCH_CHECK();
    }
    for (size_t l = 0; l < ctx->L.size(); ++l) {
        Level& Lv = ctx->L[l];
        if (Lv.kind != FACE5 || dir) {  // five-point levels without a Dirichlet row got theirs above
            ++ctx->nlaunch, launch_k(ctx->stream, k_idiag, grid2(Lv.n1, Lv.n2), dim3(BX, BY), 0, Lv.n1, Lv.n2, Lv.kind,
                                     Lv.tx, Lv.ty, Lv.a9, dir && Lv.kind == FACE5 ? Lv.ed : nullptr,
                                     l == 0 ? mask0 : nullptr, Lv.diag, Lv.idiag, mixed ? Lv.diag32 : nullptr,
                                     mixed ? Lv.idiag32 : nullptr);
            IMPEC_LAUNCH_CHECK();
        }
        if (mixed) {
            const size_t n = Lv.n();
            int nb = ctx->num_sms * 4;
            if (Lv.kind == FACE5) {
                if (l == 0 && dir) {  // the elimination changed the finest faces after k_face5_fine
                    ++ctx->nlaunch, launch_k(ctx->stream, k_to_float, nb, 256, 0, (size_t)(Lv.n1 + 1) * Lv.n2, Lv.tx, Lv.tx32);
                    ++ctx->nlaunch, launch_k(ctx->stream, k_to_float, nb, 256, 0, (size_t)Lv.n1 * (Lv.n2 + 1), Lv.ty, Lv.ty32);
                }
            } else {
                ++ctx->nlaunch, launch_k(ctx->stream, k_to_float, nb, 256, 0, n * 9, Lv.a9, Lv.a932);
            }
            IMPEC_LAUNCH_CHECK();
        }
    }
    Level& C = ctx->L.back();
    ++ctx->nlaunch, launch_k(ctx->stream, k_dense_build, 1, 256, 0, C, C.tx, C.ty, C.a9, ctx->singular,
                             ctx->dense_inv + (size_t)ctx->dense_n * ctx->dense_n);
    IMPEC_LAUNCH_CHECK();
    ++ctx->nlaunch, launch_k(ctx->stream, k_dense_invert, 1, 256, 2 * ctx->dense_n * ctx->dense_n * 8,
        ctx->dense_n, ctx->dense_inv + (size_t)ctx->dense_n * ctx->dense_n, ctx->dense_inv, ctx->singular);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

template <class T>
static void level_ptrs(Level& Lv, const T*& tx, const T*& ty, const T*& a9, const T*& id, T*& x, T*& b);
template <>
void level_ptrs<double>(Level& Lv, const double*& tx, const double*& ty, const double*& a9, const double*& id,
                        double*& x, double*& b) {
    tx = Lv.tx; ty = Lv.ty; a9 = Lv.a9; id = Lv.idiag; x = Lv.x; b = Lv.b;
}
template <>
void level_ptrs<float>(Level& Lv, const float*& tx, const float*& ty, const float*& a9, const float*& id,
                       float*& x, float*& b) {
    tx = Lv.tx32; ty = Lv.ty32; a9 = Lv.a932; id = Lv.idiag32; x = Lv.x32; b = Lv.b32;
}

template <class T>
static const T* level_diag(const Level& Lv);
template <>
const double* level_diag<double>(const Level& Lv) { return Lv.diag; }
template <>
const float* level_diag<float>(const Level& Lv) { return Lv.diag32; }

template <class T>
static T* level_alt(Level& Lv);
template <>
double* level_alt<double>(Level& Lv) { return Lv.xa; }
template <>
float* level_alt<float>(Level& Lv) { return Lv.xa32; }
template <class T>
static void swap_iterate(Level& Lv);
template <>
void swap_iterate<double>(Level& Lv) { std::swap(Lv.x, Lv.xa); }
template <>
void swap_iterate<float>(Level& Lv) { std::swap(Lv.x32, Lv.xa32); }

// Whether level l sweeps with k_rb_tile.  Each sweep writes the other iterate buffer and the
// level's pointers are swapped, so every kernel takes the iterate from the Level when it is
// launched.  A captured loop body replays the pointers of its capture, which is consistent only
// if each V-cycle starts the level from a write that reads no old iterate: true for the coarse
// levels and, with CG, for the finest level (its cycles start from x = 0); the stationary
// iteration's finest level, which corrects the solution in place, keeps the two-launch sweep.
// FP64 only: the FP32 sweeps of the mixed-precision cycle measured no faster in one launch
// (4096^2: 133 against 131 us cold).
template <class T>
static bool use_tile(impec_ctx* ctx, size_t l) {
    Level& Lv = ctx->L[l];
    const long cells = sizeof(T) == 8 ? ctx->tune.tile_cells : ctx->tune.tile_cells32;
    return cells > 0 && Lv.kind == FACE5 && Lv.n() >= (size_t)cells && (ctx->krylov || l > 0) &&
           level_alt<T>(Lv) != nullptr;
}

// Grid of the red-black kernels (k_rb_face5, k_rb_zero, k_prolong_rb): RB_ROWS rows and two
// columns per thread.
static dim3 rb_grid(const Level& Lv) {
    return dim3((Lv.n2 / 2 + 1 + BX - 1) / BX, (Lv.n1 + RB_ROWS * BY - 1) / (RB_ROWS * BY));
}

// zero: x holds no values yet and stands for x = 0 (five-point levels only, where the first
// colour's update then needs no neighbour).  first_done: that first colour was already done
// by the restriction that produced b (k_restrict with the coarse 1/diag).
template <class T>
static void smooth(impec_ctx* ctx, Level& Lv, int sweeps, bool reverse, bool zero = false, bool first_done = false) {
    const T *tx, *ty, *a9, *id;
    T *x, *b;
    level_ptrs<T>(Lv, tx, ty, a9, id, x, b);
    if (use_tile<T>(ctx, (size_t)(&Lv - ctx->L.data()))) {  // one launch per sweep, ping-pong
        const dim3 g((Lv.n2 + TILE_C - 1) / TILE_C, (Lv.n1 + TILE_R - 1) / TILE_R);
        for (int s = 0; s < sweeps; ++s) {
            level_ptrs<T>(Lv, tx, ty, a9, id, x, b);
            T* xo = level_alt<T>(Lv);
            const int first = reverse ? 1 : 0;
            ++ctx->nlaunch;
            if (zero && s == 0)  // x = 0: the first colour is b * idiag (first is red here)
                launch_k(ctx->stream, k_rb_tile<T, true>, g, TILE_THREADS, 0, Lv.n1, Lv.n2, tx, ty, id, b, (const T*)x,
                         xo, first);
            else
                launch_k(ctx->stream, k_rb_tile<T, false>, g, TILE_THREADS, 0, Lv.n1, Lv.n2, tx, ty, id, b,
                         (const T*)x, xo, first);
            swap_iterate<T>(Lv);
        }
        return;
    }
    for (int s = 0; s < sweeps; ++s) {
        if (Lv.kind == FACE5) {
            const dim3 g = rb_grid(Lv);
            for (int cc = 0; cc < 2; ++cc) {
                const int col = reverse ? 1 - cc : cc;
                if (zero && s == 0 && cc == 0) {
                    if (first_done) continue;
                    ++ctx->nlaunch;
                    launch_k(ctx->stream, k_rb_zero<T>, g, dim3(BX, BY), 0, Lv.n1, Lv.n2, id, b, x, col);
                } else {
                    ++ctx->nlaunch;
                    launch_k(ctx->stream, k_rb_face5<T>, g, dim3(BX, BY), 0, Lv.n1, Lv.n2, tx, ty, id, b, x, col);
                }
            }
        } else {
            dim3 g(((Lv.n2 + 1) / 2 + BX - 1) / BX, ((Lv.n1 + 1) / 2 + BY - 1) / BY);
            for (int cc = 0; cc < 4; ++cc) {
                int col = reverse ? 3 - cc : cc;
                ++ctx->nlaunch, launch_k(ctx->stream, k_gs4_exp9<T>, g, dim3(BX, BY), 0, Lv.n1, Lv.n2, a9, id, b, x, col >> 1, col & 1);
            }
        }
    }
}

// Shared-memory bytes the coarse CTA needs for levels l .. L-1.
template <class T>
static size_t coarse_bytes(const impec_ctx* ctx, size_t l) {
    size_t b = 0;
    for (size_t k = l; k < ctx->L.size(); ++k) {
        const Level& Lv = ctx->L[k];
        const size_t n = Lv.n();
        b += Lv.kind == FACE5 ? (size_t)(Lv.n1 + 1) * Lv.n2 + (size_t)Lv.n1 * (Lv.n2 + 1) + 4 * n : 12 * n;
    }
    return b * sizeof(T);
}

// First level handled by the single-CTA coarse V-cycle: the largest level whose cell count is
// within the precision's limit (FP64 work on one SM is slow, FP32 is 57x faster per SM).
template <class T>
static size_t coarse_start(const impec_ctx* ctx) {
    const size_t cells = (size_t)(sizeof(T) == 8 ? ctx->tune.coarse_cells64 : ctx->tune.coarse_cells32);
    // with a Dirichlet row the finest level keeps its own kernels (its prolongation is masked)
    const size_t l0 = ctx->dir_row >= 0 && ctx->L.size() > 1 ? 1 : 0;
    for (size_t l = l0; l < ctx->L.size(); ++l)
        if (ctx->L[l].n() <= cells && coarse_bytes<T>(ctx, l) <= MG_COARSE_SMEM) return l;
    return ctx->L.size() - 1;
}

// The colour whose residual the restriction skips: after a five-point pre-smoothing the colour
// updated last (black, 1) has a residual of zero up to one rounding.  -1: none.  Every V-cycle
// implementation (per-level, cluster, single-CTA) uses it, so they stay bit-identical.
static int restrict_zero_color(const impec_ctx* ctx, const Level& Lv) {
    return ctx->tune.rb_resid != 0 && Lv.kind == FACE5 && ctx->tune.pre >= 1 ? 1 : -1;
}

template <class T>
static void launch_coarse(impec_ctx* ctx, size_t lc) {
    CoarseArgs<T> A{};
    A.nl = (int)(ctx->L.size() - lc);
    A.singular = ctx->singular;
    A.pre = (int)ctx->tune.pre;
    A.post = (int)ctx->tune.post;
    A.zero_color = restrict_zero_color(ctx, ctx->L[lc]);
    A.dn = ctx->dense_n;
    A.dinv = ctx->dense_inv;
    for (int k = 0; k < A.nl; ++k) {
        Level& Lv = ctx->L[lc + k];
        const T *tx, *ty, *a9, *id;
        T *x, *b;
        level_ptrs<T>(Lv, tx, ty, a9, id, x, b);
        A.n1[k] = Lv.n1;
        A.n2[k] = Lv.n2;
        A.tx[k] = tx; A.ty[k] = ty; A.a9[k] = a9; A.id[k] = id; A.dg[k] = level_diag<T>(Lv);
        if (k == 0) { A.x0 = x; A.b0 = b; }
    }
    const size_t smem = coarse_bytes<T>(ctx, lc);
    ++ctx->nlaunch;
    if (ctx->L[lc].kind == FACE5)
        launch_k(ctx->stream, k_coarse_vcycle<T, FACE5>, 1, 1024, smem, A);
    else
        launch_k(ctx->stream, k_coarse_vcycle<T, EXP9>, 1, 1024, smem, A);
}

// Layout of the cluster V-cycle over levels ls .. L-1: which levels are spread over the cluster
// (a prefix of at least one level above the CTA-0 threshold), each CTA's band height and the
// shared-memory offsets.  False when the levels do not fit the kernel (operators of two kinds,
// too many levels, too much shared memory, a coarsest level above CL_THREADS cells).
template <class T>
static bool cluster_plan(impec_ctx* ctx, size_t ls, ClusterArgs<T>& A, size_t& smem) {
    const int CS = ctx->cl_size;
    const size_t nl = ctx->L.size() - ls;
    if (CS < 2 || nl < 2 || nl > (size_t)CL_MAXL || ctx->dense_n > CL_THREADS) return false;
    const long cta0 = ctx->tune.cl_cta0;
    A = ClusterArgs<T>{};
    A.kind = ctx->L[ls].kind;
    A.nl = (int)nl;
    A.singular = ctx->singular;
    A.pre = (int)ctx->tune.pre;
    A.post = (int)ctx->tune.post;
    A.zero_color = restrict_zero_color(ctx, ctx->L[ls]);
    A.rb_skip = A.kind == FACE5 && ctx->tune.rb_skip != 0 && ctx->tune.pre >= 1 && ctx->tune.post >= 1 ? 1 : 0;
    A.dn = ctx->dense_n;
    A.dinv = ctx->dense_inv;
    size_t off = 0;
    int nd = 0;
    for (size_t k = 0; k < nl; ++k) {
        Level& Lv = ctx->L[ls + k];
        if (Lv.kind != A.kind) return false;
        int R = Lv.n1;
        if (k + 1 < nl && nd == (int)k && (long)Lv.n() > cta0) {
            R = (Lv.n1 + CS - 1) / CS;
            R += R & 1;
            ++nd;
        }
        A.n1[k] = Lv.n1;
        A.n2[k] = Lv.n2;
        A.rows[k] = R;
        const size_t n2 = (size_t)Lv.n2, r = (size_t)R;
        const size_t ops = k + 1 < nl ? r * n2 : 0;  // nine-point: the dense level keeps x and b only
        const size_t sz[6] = {A.kind == FACE5 ? (r + 1) * n2 : 9 * ops, A.kind == FACE5 ? r * (n2 + 1) : 0,
                              A.kind == FACE5 ? r * n2 : ops, A.kind == FACE5 ? r * n2 : 0, r * n2, r * n2};
        for (int a = 0; a < 6; ++a) {
            A.off[k][a] = (unsigned)off;
            off += sz[a];
        }
        const T *tx, *ty, *a9, *id;
        T *x, *b;
        level_ptrs<T>(Lv, tx, ty, a9, id, x, b);
        A.tx[k] = tx;
        A.ty[k] = ty;
        A.id[k] = id;
        A.dg[k] = level_diag<T>(Lv);
        A.a9[k] = a9;
        if (k == 0) {
            A.x0 = x;
            A.b0 = b;
        }
    }
    A.nd = nd;
    A.dinv_off = (unsigned)((off * sizeof(T) + 15) / 16 * 16);
    smem = A.dinv_off + (size_t)A.dn * A.dn * sizeof(double);
    return nd > 0 && smem <= MG_CLUSTER_SMEM;
}

// First level handled by the cluster V-cycle (the largest level within IMPEC_MG_CL_CELLS cells
// whose plan fits), or SIZE_MAX for the per-level path.
template <class T>
static size_t cluster_start(impec_ctx* ctx) {
    if (ctx->cl_size < 2 || ctx->tune.cluster == 0) return SIZE_MAX;
    // FP32 nine-point cycles keep their per-level and single-CTA kernels: each level's four
    // colours are cheap launches there, and ten cluster-barrier phases per level cost more
    // (mixed solve at 1024^2, nu = 2/3: 5.10 ms with the cluster against 4.76 ms without)
    if (sizeof(T) == 4 && ctx->L[0].kind != FACE5) return SIZE_MAX;
    const long cells = ctx->tune.cl_cells;
    ClusterArgs<T> A;
    size_t smem;
    const size_t l0 = ctx->dir_row >= 0 ? 1 : 0;  // the finest level's prolongation is masked there
    for (size_t l = l0; l < ctx->L.size(); ++l)
        if ((long)ctx->L[l].n() <= cells && cluster_plan<T>(ctx, l, A, smem)) return l;
    return SIZE_MAX;
}

template <class T>
static void launch_cluster(impec_ctx* ctx, size_t ls) {
    ClusterArgs<T> A;
    size_t smem = 0;
    cluster_plan<T>(ctx, ls, A, smem);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctx->cl_size);
    cfg.blockDim = dim3(CL_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = ctx->cl_size;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 2 : 1;
    ++ctx->nlaunch;
    cudaLaunchKernelEx(&cfg, k_cluster_vcycle<T>, A);
}

// Whether the V-cycle at level l runs per-level red-black kernels, so that a cycle started
// from x = 0 needs no zero fill of the level's iterate (the first colour is k_rb_zero).
template <class T>
static bool zero_start_free(impec_ctx* ctx, size_t l) {
    const Level& F = ctx->L[l];
    return ctx->tune.rb_skip != 0 && F.kind == FACE5 && ctx->tune.pre >= 1 && l != cluster_start<T>(ctx) &&
           l != coarse_start<T>(ctx);
}

// One V-cycle from level l down.  zero: the level's iterate stands for x = 0; unless
// zero_start_free<T>(ctx, l), the caller has filled it with zeros.  first_done: the caller
// (the restriction from level l - 1) also did the pre-smoothing's first colour.
template <class T>
static void vcycle(impec_ctx* ctx, size_t l, bool zero, bool first_done = false) {
    Level& F = ctx->L[l];
    const T *tx, *ty, *a9, *id;
    T *x, *b;
    level_ptrs<T>(F, tx, ty, a9, id, x, b);
    if (l == cluster_start<T>(ctx)) {
        launch_cluster<T>(ctx, l);
        return;
    }
    const size_t lc = coarse_start<T>(ctx);
    if (l == lc) {
        launch_coarse<T>(ctx, lc);
        return;
    }
    Level& C = ctx->L[l + 1];
    const T *ctx_, *cty, *ca9, *cid;
    T *cx, *cb;
    level_ptrs<T>(C, ctx_, cty, ca9, cid, cx, cb);
    const bool zs = zero && zero_start_free<T>(ctx, l);
    smooth<T>(ctx, F, (int)ctx->tune.pre, false, zs, zs && first_done);
    level_ptrs<T>(F, tx, ty, a9, id, x, b);  // the sweep may have moved the iterate (ping-pong)
    ++ctx->nlaunch;
    const int zero_color = restrict_zero_color(ctx, F);
    // the coarse cycle's first colour is done here, unless that level sweeps in one launch
    // (its zero-start sweep computes the first colour itself)
    const bool cz = zero_start_free<T>(ctx, l + 1) && !use_tile<T>(ctx, l + 1);
    launch_k(ctx->stream, k_restrict<T>, grid2(C.n1, C.n2), dim3(BX, BY), 0, F, tx, ty, a9, level_diag<T>(F), b, x,
             C.n1, C.n2, cb, cx, zero_color, cz ? (const T*)cid : nullptr);
    vcycle<T>(ctx, l + 1, true, cz);
    level_ptrs<T>(C, ctx_, cty, ca9, cid, cx, cb);  // the coarse iterate may have moved too
    const unsigned char* mask = l == 0 && ctx->dir_row >= 0 ? ctx->dmask : nullptr;
    ++ctx->nlaunch;
    if (ctx->tune.rb_skip != 0 && F.kind == FACE5 && ctx->tune.post >= 1)  // the black cells are overwritten next
        launch_k(ctx->stream, k_prolong_rb<T>, rb_grid(F), dim3(BX, BY), 0, F.n1, F.n2, x, C.n1, C.n2, cx, mask, 0);
    else
        launch_k(ctx->stream, k_prolong<T>, grid2(F.n1, F.n2), dim3(BX, BY), 0, F.n1, F.n2, x, C.n1, C.n2, cx, mask);
    smooth<T>(ctx, F, (int)ctx->tune.post, true);
}

// Convergence check of the solve loop (one thread): relres = ||r||/||f||; decides whether
// another cycle runs and, inside a graph, sets the WHILE node's condition.  With CG
// (krylov) and after an iteration, it also keeps the iteration's alpha and (r, z) for the
// next search direction, and stops on a breakdown ((p, Ap) <= 0).
__device__ __forceinline__ void mg_check(DevScalars* S, double tol, int max_cycles, int inc,
                                         cudaGraphConditionalHandle h, int use_h, int krylov) {
    bool breakdown = false;
    if (inc) {
        S->mg_cycles++;
        if (krylov) {
            breakdown = !(S->pcg_pq > 0.0);
            S->pcg_alpha = breakdown ? 0.0 : S->pcg_rz / S->pcg_pq;
            S->pcg_rz_old = S->pcg_rz;
        }
    }
    double fn = S->fnorm2, rn = S->rnorm2;
    double rr = fn > 0 ? sqrt(rn / fn) : sqrt(rn);
    S->relres = rr;
    if (!inc && S->mg_cycles == 0) S->relres0 = rr;
    const bool bad = !(rr == rr) || isinf(rr);
    const bool go = !bad && !breakdown && rr > tol && S->mg_cycles < max_cycles;
    if (bad) S->flags |= FLAG_MG_NAN;
    else if (!go && rr > tol) S->flags |= FLAG_MG_NOT_CONVERGED;
    S->go = go ? 1 : 0;
    if (use_h) cudaGraphSetConditional(h, go ? 1u : 0u);
}

__global__ void k_mg_check(DevScalars* S, double tol, int max_cycles, int inc, cudaGraphConditionalHandle h,
                           int use_h, int krylov) {
    pdl_enter();
    mg_check(S, tol, max_cycles, inc, h, use_h, krylov);
}

// ---------------------------------------------------------------- V-cycle preconditioned CG
// The reference solves the pressure system with CG preconditioned by HYPRE's SMG
// (src/MGSolver.cpp:594-629); here the preconditioner is one V-cycle of the engine's own
// multigrid (V(1,2) for five-point, V(1,1) for nine-point operators by default), z = M^-1 r, in
// FP64 or (mixed precision) in FP32 on the FP32 copy of r.  CG runs in FP64 on the consistent
// singular system.  Because neither a cycle with unequal pre- and post-smoothing nor the FP32
// cycle is a symmetric operator, the direction uses the flexible (Polak-Ribiere) coefficient
//   beta = (z_k, r_k - r_{k-1}) / (z_{k-1}, r_{k-1}) = -alpha_{k-1} (z_k, A p_{k-1}) / (z_{k-1}, r_{k-1}),
// which needs only (z, r) and (z, q) with q = A p still holding the previous direction.

// z: the V-cycle's finest iterate, FP64 or FP32.
__device__ __forceinline__ double cg_z(const double* __restrict__ z, const float* __restrict__ z32, size_t k) {
    return z32 ? (double)z32[k] : z[k];
}

// (r, z) and (z, q) into out[0], out[1].  With S (CG, out = &S->pcg_rz), the last block also
// stores the direction's beta = -alpha_old (z, q) / (z, r)_old (0 on the first iteration).
__global__ void __launch_bounds__(RED_THREADS) k_cg_dots(int n1, int n2, const double* __restrict__ r,
                                                         const double* __restrict__ z, const float* __restrict__ z32,
                                                         const double* __restrict__ q, double* partials, int mb,
                                                         unsigned* counter, double* out, DevScalars* S) {
    pdl_enter();
    double acc[2] = {0.0, 0.0};
    for_cells(n1, n2, [&](int, int, size_t k) {
        const double zz = cg_z(z, z32, k);
        acc[0] += r[k] * zz;
        acc[1] += zz * q[k];
    });
    if (grid_reduce<2>(acc, 0u, partials, mb, counter, out) && threadIdx.x == 0 && S) {
        const bool first = S->mg_cycles == 0 || S->pcg_rz_old == 0.0;
        S->pcg_beta = first ? 0.0 : -S->pcg_alpha * S->pcg_zq / S->pcg_rz_old;
    }
}

// p = z + beta p (p = z on the first iteration, whatever p held).
__global__ void k_cg_direction(size_t n, const double* __restrict__ z, const float* __restrict__ z32,
                               double* __restrict__ p, const DevScalars* __restrict__ S) {
    pdl_enter();
    const bool first = S->mg_cycles == 0 || S->pcg_rz_old == 0.0;
    const double beta = S->pcg_beta;  // from k_cg_dots
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        p[k] = first ? cg_z(z, z32, k) : cg_z(z, z32, k) + beta * p[k];
}

// q = A p with the integrated operator (diag p - sum t p_nb) and (p, q) into out[0].  With S
// (CG, out = &S->pcg_pq), the last block also stores the update's alpha = (r, z) / (p, Ap)
// (0 unless (p, Ap) > 0).
__global__ void __launch_bounds__(RED_THREADS) k_cg_apply(Level F, const double* __restrict__ p,
                                                          double* __restrict__ q, double* partials, int mb,
                                                          unsigned* counter, double* out, DevScalars* S) {
    pdl_enter();
    double acc[1] = {0.0};
    for_cells(F.n1, F.n2, [&](int i, int j, size_t k) {
        const int n1 = F.n1, n2 = F.n2;
        double s = F.diag[k] * p[k];
        if (F.kind == FACE5) {
            if (i > 0) s -= F.tx[k] * p[k - n2];
            if (i < n1 - 1) s -= F.tx[k + n2] * p[k + n2];
            if (j > 0) s -= F.ty[IX(i, j, n2 + 1)] * p[k - 1];
            if (j < n2 - 1) s -= F.ty[IX(i, j + 1, n2 + 1)] * p[k + 1];
        } else {
            const size_t n = (size_t)n1 * n2;
            for (int e = 1; e < 9; ++e) {
                const int ii = i + c_off[e][0], jj = j + c_off[e][1];
                if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
                s += F.a9[e * n + k] * p[IX(ii, jj, n2)];
            }
        }
        q[k] = s;
        acc[0] += p[k] * s;
    });
    if (grid_reduce<1>(acc, 0u, partials, mb, counter, out) && threadIdx.x == 0 && S) {
        const double pq = S->pcg_pq;
        S->pcg_step = pq > 0.0 ? S->pcg_rz / pq : 0.0;
    }
}

// alpha = (r, z) / (p, Ap); x += alpha p; r -= alpha Ap (and its FP32 copy); ||r||^2 over the
// cells other than the pinned one.  The last block of the reduction then runs the iteration's
// convergence check (k_mg_check's work, one launch fewer per iteration).
__global__ void __launch_bounds__(RED_THREADS) k_cg_update(int n1, int n2, double* __restrict__ x,
                                                           double* __restrict__ r, float* __restrict__ r32,
                                                           const double* __restrict__ p, const double* __restrict__ q,
                                                           int pin, DevScalars* S, double* partials, int mb,
                                                           unsigned* counter, double* out, double tol, int max_cycles,
                                                           cudaGraphConditionalHandle h, int use_h) {
    pdl_enter();
    const double alpha = S->pcg_step;  // from k_cg_apply
    double acc[1] = {0.0};
    for_cells(n1, n2, [&](int, int, size_t k) {
        x[k] += alpha * p[k];
        const double rr = r[k] - alpha * q[k];
        r[k] = rr;
        if (r32) r32[k] = (float)rr;
        if ((int)k != pin) acc[0] += rr * rr;
    });
    if (grid_reduce<1>(acc, 0u, partials, mb, counter, out) && threadIdx.x == 0) {
        __threadfence();
        mg_check(S, tol, max_cycles, 1, h, use_h, 1);
    }
}

// Convergence decision on the true residual (one thread; S->rnorm2 = ||f - A x||^2 of the
// iterate).  It becomes the reported relres and alone sets or clears FLAG_MG_NOT_CONVERGED.
__device__ __forceinline__ void true_check(DevScalars* S, double tol, int max_cycles, cudaGraphConditionalHandle h,
                                           int use_h) {
    const double fn = S->fnorm2, rn = S->rnorm2;
    const double rr = fn > 0 ? sqrt(rn / fn) : sqrt(rn);
    S->relres = rr;
    const bool bad = !(rr == rr) || isinf(rr);
    const bool go = !bad && rr > tol && S->mg_cycles < max_cycles;
    if (bad) S->flags |= FLAG_MG_NAN;
    if (!bad && !go && rr > tol) S->flags |= FLAG_MG_NOT_CONVERGED;
    else S->flags &= ~FLAG_MG_NOT_CONVERGED;
    S->go = go ? 1 : 0;
    if (use_h) cudaGraphSetConditional(h, go ? 1u : 0u);
}

// End of a CG pass, after k_cg_update, whose check set S->go from the recurrence residual.
// That residual drifts from the true one by rounding, so a stop (converged, max_cycles or a
// breakdown) is verified here: the true residual f - A x of the final iterate replaces r (and
// its FP32 copy), its norm gives the reported relres, and CG continues from it while it is
// above tol and cycles remain.  On the other passes the kernel only hands S->go to the WHILE
// condition.  Every thread reads S->go before the last block (the only writer) can change it.
__global__ void __launch_bounds__(RED_THREADS) k_cg_verify(Level F, const double* __restrict__ f,
                                                           const double* __restrict__ x, int pin,
                                                           float* __restrict__ r32, double* __restrict__ r64,
                                                           DevScalars* S, double* partials, int mb, unsigned* counter,
                                                           double tol, int max_cycles, cudaGraphConditionalHandle h,
                                                           int use_h) {
    pdl_enter();
    const int go = S->go, nan = S->flags & FLAG_MG_NAN;
    if (go || nan) {
        if (use_h && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(h, go ? 1u : 0u);
        return;
    }
    double acc[1] = {0.0};
    for_cells(F.n1, F.n2, [&](int i, int j, size_t k) {
        double r = resid<double>(F, i, j, F.tx, F.ty, F.a9, F.diag, f, x);
        r64[k] = r;
        if (r32) r32[k] = (float)r;
        if ((int)k == pin) r = 0.0;  // as k_fine_resid
        acc[0] += r * r;
    });
    if (grid_reduce<1>(acc, 0u, partials, mb, counter, &S->rnorm2) && threadIdx.x == 0) {
        __threadfence();
        true_check(S, tol, max_cycles, h, use_h);
    }
}

// The pinned cell of the singular system (-1 with a Dirichlet row: nothing is pinned).
static int pin_index(impec_ctx* ctx) { return ctx->singular ? (int)IX(ctx->pin_i, ctx->pin_j, ctx->L[0].n2) : -1; }

// The iterate the loop updates: CG keeps it in its own buffer (the finest level's iterate is
// the preconditioner's output), stationary cycles update the finest iterate itself.
static double* solve_iterate(impec_ctx* ctx) { return ctx->krylov ? ctx->cg_x : ctx->L[0].x; }

// FP64 residual r = f - A x of the iterate and ||r||^2, optionally stored in FP32 (r32: the
// rhs of the mixed-precision cycle) and in FP64 (r64: the CG residual).
static impec_status fine_residual(impec_ctx* ctx, const double* x, float* r32, double* r64) {
    Level& F = ctx->L[0];
    ++ctx->nlaunch;
    // about seven cells per thread: the FP64 warp sums of the reduction stay small beside the residual
    const int blocks = seg_blocks(F.n1, F.n2, red_cap(ctx->num_sms, ctx->max_blocks));
    launch_k(ctx->stream, k_fine_resid, blocks, RED_THREADS, 0, F, ctx->f, x, pin_index(ctx), r32, r64,
             ctx->partials, ctx->max_blocks, ctx->counter, &ctx->dscal->rnorm2);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

// x += alpha d with alpha = (r0, d) / (d, A d) (from k_cg_dots: pcg_rz, pcg_zq), the step
// along the learned direction that minimises the A-norm error; 0 when (d, A d) is not
// positive or alpha is not finite.
__global__ void k_learn_step(size_t n, double* __restrict__ x, const double* __restrict__ d,
                             const DevScalars* __restrict__ S, double* alpha_out) {
    pdl_enter();
    const double dad = S->pcg_zq, rd = S->pcg_rz;
    double a = dad > 0.0 ? rd / dad : 0.0;
    if (!(a == a) || isinf(a)) a = 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) *alpha_out = a;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        x[k] += a * d[k];
}

// Learned initial guess (an attached network): r0 = f - A x, the network's direction d from
// the state and r0, then the A-norm-optimal step along d (launch only).
static impec_status learned_guess(impec_ctx* ctx, double* x) {
    Level& F = ctx->L[0];
    DevScalars* S = ctx->dscal;
    IMPEC_TRY(fine_residual(ctx, x, nullptr, ctx->lrn_r0));
    IMPEC_TRY(learned_predict(ctx, x, ctx->lrn_r0, ctx->lrn_d));
    if (!learned_predicts(ctx)) return IMPEC_OK;
    const int cap = red_cap(ctx->num_sms, ctx->max_blocks), blocks = seg_blocks(F.n1, F.n2, cap);
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_cg_apply, blocks, RED_THREADS, 0, F, (const double*)ctx->lrn_d, ctx->lrn_Ad, ctx->partials,
             ctx->max_blocks, ctx->counter, &S->pcg_pq, (DevScalars*)nullptr);
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_cg_dots, blocks, RED_THREADS, 0, F.n1, F.n2, (const double*)ctx->lrn_r0,
             (const double*)ctx->lrn_d, (const float*)nullptr, (const double*)ctx->lrn_Ad, ctx->partials,
             ctx->max_blocks, ctx->counter, &S->pcg_rz, (DevScalars*)nullptr);
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_learn_step, ctx->num_sms * 4, 256, 0, F.n(), x, (const double*)ctx->lrn_d,
             (const DevScalars*)S, ctx->lrn_alpha);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

// Operator, hierarchy, consistent rhs, initial iterate and initial residual (launch only).
impec_status pressure_prepare(impec_ctx* ctx, const double* c, const double* p) {
    const impec_params& P = ctx->P;
    IMPEC_TRY(pressure_setup(ctx, c));
    Level& F = ctx->L[0];
    const size_t n = F.n();
    const int pin = pin_index(ctx);
    DevScalars* S = ctx->dscal;
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_rhs, flat_blocks(n, red_cap(ctx->num_sms, ctx->max_blocks)), RED_THREADS, 0, n, ctx->q,
             ctx->G.dA, ctx->f, ctx->partials, ctx->max_blocks, ctx->counter, &S->fsum);
    if (ctx->singular) {
        ++ctx->nlaunch;
        launch_k(ctx->stream, k_fix_pin, 1, 1, 0, ctx->f, ctx->q, pin, ctx->G.dA, ctx->pin_kappa, S);
    }
    IMPEC_LAUNCH_CHECK();
    double* x = solve_iterate(ctx);
    if (P.warm_start)
        IMPEC_CUDA_TRY(cudaMemcpyAsync(x, p, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    else
        IMPEC_CUDA_TRY(cudaMemsetAsync(x, 0, n * 8, ctx->stream));
    if (!ctx->singular) {  // Dirichlet row: known values into f and x, their couplings into f
        ++ctx->nlaunch;
        launch_k(ctx->stream, k_dirichlet_rhs, ctx->num_sms * 4, 256, 0, n, ctx->f, x, ctx->dfd, ctx->dmask);
        IMPEC_LAUNCH_CHECK();
    }
    if (ctx->learned) IMPEC_TRY(learned_guess(ctx, x));
    if (!ctx->krylov) IMPEC_CUDA_TRY(cudaMemcpyAsync(F.b, ctx->f, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaMemsetAsync(&S->mg_cycles, 0, sizeof(int), ctx->stream));
    const bool mixed = P.precision == IMPEC_PREC_MIXED;
    if (ctx->krylov) return fine_residual(ctx, x, mixed ? F.b32 : nullptr, mixed ? ctx->r : F.b);
    return pressure_residual(ctx);
}

// FP64 fine residual and its norm of the stationary iteration (r32 for the mixed correction).
impec_status pressure_residual(impec_ctx* ctx) {
    Level& F = ctx->L[0];
    return fine_residual(ctx, F.x, ctx->P.precision == IMPEC_PREC_MIXED ? F.b32 : nullptr, nullptr);
}

impec_status pressure_check(impec_ctx* ctx, double tol, int inc, cudaGraphConditionalHandle h, int use_h) {
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_mg_check, 1, 1, 0, ctx->dscal, tol, ctx->P.max_cycles, inc, h, use_h, ctx->krylov);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

// One iteration on the current iterate, the new residual and the convergence check (launch
// only): a stationary V-cycle, or a CG step preconditioned by one V-cycle (whose residual
// kernel also runs the check).  h / use_h: the graph's WHILE condition, as pressure_check.
impec_status pressure_step(impec_ctx* ctx, double tol, cudaGraphConditionalHandle h, int use_h) {
    if (!ctx->krylov) {
        IMPEC_TRY(pressure_iteration(ctx, tol, h, use_h));
        return pressure_check(ctx, tol, 1, h, use_h);
    }
    return pressure_iteration(ctx, tol, h, use_h);
}

impec_status pressure_iteration(impec_ctx* ctx, double tol, cudaGraphConditionalHandle h, int use_h) {
    Level& F = ctx->L[0];
    const size_t n = F.n();
    const bool mixed = ctx->P.precision == IMPEC_PREC_MIXED;
    if (!ctx->krylov) {
        if (mixed) {
            if (!zero_start_free<float>(ctx, 0)) IMPEC_CUDA_TRY(cudaMemsetAsync(F.x32, 0, n * 4, ctx->stream));
            vcycle<float>(ctx, 0, true);
            ++ctx->nlaunch;
            launch_k(ctx->stream, k_add_f32, ctx->num_sms * 4, 256, 0, n, F.x, F.x32);
            IMPEC_LAUNCH_CHECK();
            return pressure_residual(ctx);
        }
        vcycle<double>(ctx, 0, false);  // corrects the iterate itself
        IMPEC_LAUNCH_CHECK();
        return pressure_residual(ctx);
    }
    DevScalars* S = ctx->dscal;
    double* r = mixed ? ctx->r : F.b;
    if (mixed) {
        if (!zero_start_free<float>(ctx, 0)) IMPEC_CUDA_TRY(cudaMemsetAsync(F.x32, 0, n * 4, ctx->stream));
        vcycle<float>(ctx, 0, true);
    } else {
        if (!zero_start_free<double>(ctx, 0)) IMPEC_CUDA_TRY(cudaMemsetAsync(F.x, 0, n * 8, ctx->stream));
        vcycle<double>(ctx, 0, true);
    }
    // the preconditioned residual z, where the cycle left it (the sweeps may swap buffers)
    const double* z = mixed ? nullptr : F.x;
    const float* z32 = mixed ? F.x32 : nullptr;
    const int cap = red_cap(ctx->num_sms, ctx->max_blocks), blocks = seg_blocks(F.n1, F.n2, cap);
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_cg_dots, blocks, RED_THREADS, 0, F.n1, F.n2, r, z, z32, ctx->cg_q, ctx->partials,
             ctx->max_blocks, ctx->counter, &S->pcg_rz, S);
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_cg_direction, ctx->num_sms * 4, 256, 0, n, z, z32, ctx->cg_p, S);
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_cg_apply, blocks, RED_THREADS, 0, F, ctx->cg_p, ctx->cg_q, ctx->partials,
             ctx->max_blocks, ctx->counter, &S->pcg_pq, S);
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_cg_update, blocks, RED_THREADS, 0, F.n1, F.n2, ctx->cg_x, r, mixed ? F.b32 : nullptr,
             (const double*)ctx->cg_p, (const double*)ctx->cg_q, pin_index(ctx), S, ctx->partials, ctx->max_blocks,
             ctx->counter, &S->rnorm2, tol, ctx->P.max_cycles, h, 0);
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_cg_verify, blocks, RED_THREADS, 0, F, (const double*)ctx->f, (const double*)ctx->cg_x,
             pin_index(ctx), mixed ? F.b32 : nullptr, r, S, ctx->partials, ctx->max_blocks, ctx->counter, tol,
             ctx->P.max_cycles, h, use_h);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

// Constant shift to the pinned value and copy to p (launch only).  With CG the reported relres
// is the true one, from the k_cg_verify that ended the loop.
impec_status pressure_finish(impec_ctx* ctx, double* p) {
    Level& F = ctx->L[0];
    const size_t n = F.n();
    double* x = solve_iterate(ctx);
    if (ctx->singular) {  // the constant that puts the pinned cell at its value
        ++ctx->nlaunch;
        launch_k(ctx->stream, k_shift, ctx->num_sms * 4, 256, 0, n, x, pin_index(ctx), ctx->dscal);
    }
    IMPEC_LAUNCH_CHECK();
    IMPEC_CUDA_TRY(cudaMemcpyAsync(p, x, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    return IMPEC_OK;
}

// Host-driven solve (per-operation entry point): one host round trip per cycle.
impec_status pressure_solve(impec_ctx* ctx, const double* c, double* p, double tol, int* cycles, double* relres) {
    IMPEC_CUDA_TRY(cudaMemsetAsync(&ctx->dscal->flags, 0, sizeof(int), ctx->stream));
    IMPEC_TRY(pressure_prepare(ctx, c, p));
    IMPEC_TRY(pressure_check(ctx, tol, 0, 0, 0));
    for (;;) {
        IMPEC_TRY(sync_scalars(ctx));
        if (!ctx->hscal->go) break;
        IMPEC_TRY(pressure_step(ctx, tol, 0, 0));
    }
    IMPEC_TRY(pressure_finish(ctx, p));
    IMPEC_TRY(sync_scalars(ctx));
    const int k = ctx->hscal->mg_cycles;
    const double rr = ctx->hscal->relres;
    if (cycles) *cycles = k;
    if (relres) *relres = rr;
    ctx->last_its = k;
    ctx->last_relres = rr;
    if (ctx->hscal->flags & FLAG_MG_NAN) return IMPEC_ERR_NAN;
    if (ctx->hscal->flags & FLAG_MG_NOT_CONVERGED) return IMPEC_ERR_NOT_CONVERGED;
    return IMPEC_OK;
}

impec_status pressure_apply_ref(impec_ctx* ctx, const double* x, double* y) {
    Level& F = ctx->L[0];
    const int pin = ctx->singular ? (int)IX(ctx->pin_i, ctx->pin_j, F.n2) : -1;
    ++ctx->nlaunch, launch_k(ctx->stream, k_apply_ref, grid2(F.n1, F.n2), dim3(BX, BY), 0, F, x, pin, ctx->dir_row,
                             ctx->G.dA, ctx->pin_kappa, y);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

// ---------------------------------------------------------------- Darcy velocities
// CalcVelocities (src/EllipticSolver.cpp:541-683): u = nu * parallel + (1-nu) * diagonal.
struct VelArgs {
    int n1, n2;
    double nu, inv_dx, inv_dy, inv_dxi, inv_deta, cost, sina, sint, cosa;
};

// (xi,eta) Darcy velocity at corner (ci,cj) = reference corner (ci-1/2, cj-1/2), rotated back
// to (x,y): GetDiagonalW_im12j + XYFromXiEta.
__device__ __forceinline__ void corner_vel(const VelArgs& A, const double* __restrict__ p,
                                           const double* __restrict__ m11, const double* __restrict__ m22,
                                           const double* __restrict__ m12, int ci, int cj, double& u1, double& u2) {
    const int n1 = A.n1, n2 = A.n2;
    int i0 = refl_cell(ci - 1, n1), i1 = refl_cell(ci, n1), j0 = refl_cell(cj - 1, n2), j1 = refl_cell(cj, n2);
    double d1dp = A.inv_dxi * (p[IX(i1, j1, n2)] - p[IX(i0, j0, n2)]);
    double d2dp = A.inv_deta * (p[IX(i0, j1, n2)] - p[IX(i1, j0, n2)]);
    size_t k = IX(ci, cj, n2 + 1);
    double M11 = m11[k], M12 = m12[k], M22 = m22[k];
    double w1 = -d1dp * M11 - d2dp * M12;
    double w2 = -d1dp * M12 - d2dp * M22;
    u1 = A.cost * w1 - A.sina * w2;
    u2 = A.sint * w1 + A.cosa * w2;
}

__global__ void k_velocity(VelArgs A, const double* __restrict__ p, const double* __restrict__ lamx,
                           const double* __restrict__ lamy, const double* __restrict__ m11,
                           const double* __restrict__ m22, const double* __restrict__ m12, double* __restrict__ u,
                           double* __restrict__ v) {
    pdl_enter();
    int j = blockIdx.x * BX + threadIdx.x, i = blockIdx.y * BY + threadIdx.y;
    const int n1 = A.n1, n2 = A.n2;
    const bool diag = A.nu < 1.0;
    if (i <= n1 && j < n2) {
        double dp = p[IX(refl_cell(i, n1), j, n2)] - p[IX(refl_cell(i - 1, n1), j, n2)];
        double par = (-lamx[IX(i, j, n2)] * dp) * A.inv_dx;
        double val = par;
        if (diag) {
            double a1, a2, b1, b2;
            corner_vel(A, p, m11, m22, m12, i, j, a1, a2);
            corner_vel(A, p, m11, m22, m12, i, j + 1, b1, b2);
            val = A.nu * par + (1. - A.nu) * (0.5 * (b1 + a1));
        }
        u[IX(i, j, n2)] = val;
    }
    if (i < n1 && j <= n2) {
        double dp = p[IX(i, refl_cell(j, n2), n2)] - p[IX(i, refl_cell(j - 1, n2), n2)];
        double par = (-lamy[IX(i, j, n2 + 1)] * dp) * A.inv_dy;
        double val = par;
        if (diag) {
            double a1, a2, b1, b2;
            corner_vel(A, p, m11, m22, m12, i, j, a1, a2);
            corner_vel(A, p, m11, m22, m12, i + 1, j, b1, b2);
            val = A.nu * par + (1. - A.nu) * (0.5 * (a2 + b2));
        }
        v[IX(i, j, n2 + 1)] = val;
    }
}

impec_status velocity(impec_ctx* ctx, const double* p, const double* c, double* u, double* v) {
    (void)c;  // mobilities were computed from c by the preceding pressure setup
    const impec_params& P = ctx->P;
    const Geo& G = ctx->G;
    VelArgs A{P.N1, P.N2, P.nu, 1.0 / G.dx, 1.0 / G.dy, 1.0 / G.dxi, 1.0 / G.deta, G.cost, G.sina, G.sint, G.cosa};
    ++ctx->nlaunch, launch_k(ctx->stream, k_velocity, grid2(P.N1 + 1, P.N2 + 1), dim3(BX, BY), 0, A, p, ctx->lamx, ctx->lamy, ctx->cm11,
                                                                            ctx->cm22, ctx->cm12, u, v);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

// MaxStableTimestepCombined (src/HyperbolicSolver.cpp:123-198); dt written to S->dt.
__global__ void __launch_bounds__(RED_THREADS) k_maxvel(int n1, int n2, const double* __restrict__ u,
                                                        const double* __restrict__ v, int diffusion, double al,
                                                        double at, double dx, double* partials, int mb,
                                                        unsigned* counter, double* out) {
    pdl_enter();
    // acc[0]: the largest |u_i + u_i+1| or |v_j + v_j+1| of a cell.  The reference's cell speed is
    // half of it, floored at the smallest normal double; both are applied once, to the maximum,
    // by k_finish_dt (halving is exact, and a maximum commutes with both).
    double acc[2] = {0.0, -1.0e10};  // max |face velocity sum|, max of -dt_diff
    for_cells(n1, n2, [&](int i, int j, size_t) {
        const double su = u[IX(i, j, n2)] + u[IX(i + 1, j, n2)];
        const double sv = v[IX(i, j, n2 + 1)] + v[IX(i, j + 1, n2 + 1)];
        acc[0] = fmax(acc[0], fmax(fabs(su), fabs(sv)));
        if (diffusion) {
            const double uij = 0.5 * su, vij = 0.5 * sv;
            double vij2 = vij * vij, uij2 = uij * uij;
            double absu = sqrt(vij2 + uij2);
            double d11 = dx / absu * (al * uij2 + at * vij2);
            double d22 = dx / absu * (al * vij2 + at * uij2);
            double dt = 1. / 2 * dx * dx / (d11 + d22);
            acc[1] = fmax(acc[1], -dt);
        }
    });
    grid_reduce<2>(acc, 3u, partials, mb, counter, out);
}

__global__ void k_finish_dt(DevScalars* S, double dx, double dy, double cfl, int use_diff, double limit) {
    pdl_enter();
    double mv = fmax(0.5 * S->red[0], 2.2250738585072014e-308);  // see k_maxvel
    S->maxvel = mv;
    double dt = fmin(dx / mv, dy / mv) * cfl;
    if (use_diff) {
        double dd = fmin(-S->red[1], 1.e10) * limit;
        dt = fmin(dd, dt);
    }
    S->dt = dt;
}

impec_status max_stable_dt_dev(impec_ctx* ctx, const double* u, const double* v) {
    const impec_params& P = ctx->P;
    const Geo& G = ctx->G;
    // the diffusive limit (sqrt and two FP64 divisions per cell) only when it enters dt
    const int use_diff = P.diffusion && P.ptype != IMPEC_CRANKNICOLSON;
    ++ctx->nlaunch, launch_k(ctx->stream, k_maxvel, seg_blocks(P.N1, P.N2, red_cap(ctx->num_sms, ctx->max_blocks)), RED_THREADS, 0,
        P.N1, P.N2, u, v, use_diff, P.alpha_l, P.alpha_t, G.dx, ctx->partials, ctx->max_blocks, ctx->counter,
        ctx->dscal->red);
    double cfl = P.cfl_porosity ? P.cfl * P.porosity : P.cfl;
    ++ctx->nlaunch, launch_k(ctx->stream, k_finish_dt, 1, 1, 0, ctx->dscal, G.dx, G.dy, cfl, use_diff, P.dt_diff_limit);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

}  // namespace impec

using namespace impec;

// Cold timing of one probed kernel: before each repetition `flush_bytes` of `flush` are
// overwritten on the context's stream (evicting the kernel's data from L2), then the kernel
// runs between two events on that stream.  *ms: mean over the repetitions, *ms_min: the fastest.
extern "C" impec_status impec_time_kernel_cold(impec_ctx* ctx, int which, int reps, void* flush, size_t flush_bytes,
                                               double* ms, double* ms_min, double* bytes) {
    if (!ctx || reps <= 0 || which < 0 || which > 1 || !flush || !flush_bytes) return IMPEC_ERR_ARG;
    Level& F = ctx->L[0];
    if (F.kind != FACE5) return IMPEC_ERR_ARG;
    const double n = (double)F.n();
    if (which == 1 && ctx->P.precision != IMPEC_PREC_MIXED) {  // FP32 copies of the fine level
        const int nb = ctx->num_sms * 4;
        launch_k(ctx->stream, k_to_float, nb, 256, 0, (size_t)(F.n1 + 1) * F.n2, F.tx, F.tx32);
        launch_k(ctx->stream, k_to_float, nb, 256, 0, (size_t)F.n1 * (F.n2 + 1), F.ty, F.ty32);
        launch_k(ctx->stream, k_to_float, nb, 256, 0, F.n(), F.idiag, F.idiag32);
        launch_k(ctx->stream, k_to_float, nb, 256, 0, F.n(), F.b, F.b32);
        launch_k(ctx->stream, k_to_float, nb, 256, 0, F.n(), F.x, F.x32);
        IMPEC_LAUNCH_CHECK();
    }
    cudaEvent_t e0, e1;
    IMPEC_CUDA_TRY(cudaEventCreate(&e0));
    IMPEC_CUDA_TRY(cudaEventCreate(&e1));
    double tot = 0, best = 1e30;
    for (int r = 0; r < reps; ++r) {
        IMPEC_CUDA_TRY(cudaMemsetAsync(flush, r & 0xff, flush_bytes, ctx->stream));
        IMPEC_CUDA_TRY(cudaEventRecord(e0, ctx->stream));
        if (which == 0) smooth<double>(ctx, F, 1, false);
        else smooth<float>(ctx, F, 1, false);
        IMPEC_CUDA_TRY(cudaEventRecord(e1, ctx->stream));
        IMPEC_CUDA_TRY(cudaEventSynchronize(e1));
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        tot += t;
        best = t < best ? t : best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms) *ms = tot / reps;
    if (ms_min) *ms_min = best;
    // algorithmic bytes of one five-point sweep: x read and written, b, and the two face planes
    if (bytes) *bytes = n * (which == 0 ? 8.0 : 4.0) * 5.0;
    return IMPEC_OK;
}

extern "C" impec_status impec_time_kernel(impec_ctx* ctx, int which, int reps, double* ms, double* bytes) {
    if (!ctx || reps <= 0 || which < 0 || which > 4) return IMPEC_ERR_ARG;
    Level& F = ctx->L[0];
    const double n = (double)F.n();
    if (which == 1 && ctx->P.precision != IMPEC_PREC_MIXED) {  // FP32 copies of the fine level
        const int nb = ctx->num_sms * 4;
        if (F.kind == FACE5) {
            launch_k(ctx->stream, k_to_float, nb, 256, 0, (size_t)(F.n1 + 1) * F.n2, F.tx, F.tx32);
            launch_k(ctx->stream, k_to_float, nb, 256, 0, (size_t)F.n1 * (F.n2 + 1), F.ty, F.ty32);
        } else {
            launch_k(ctx->stream, k_to_float, nb, 256, 0, F.n() * 9, F.a9, F.a932);
        }
        launch_k(ctx->stream, k_to_float, nb, 256, 0, F.n(), F.idiag, F.idiag32);
        launch_k(ctx->stream, k_to_float, nb, 256, 0, F.n(), F.b, F.b32);
        launch_k(ctx->stream, k_to_float, nb, 256, 0, F.n(), F.x, F.x32);
        IMPEC_LAUNCH_CHECK();
    }
    cudaEvent_t e0, e1;
    IMPEC_CUDA_TRY(cudaEventCreate(&e0));
    IMPEC_CUDA_TRY(cudaEventCreate(&e1));
    const double coef = F.kind == FACE5 ? 2.0 : 9.0;  // operator planes per cell
    double b = 0;
    IMPEC_CUDA_TRY(cudaEventRecord(e0, ctx->stream));
    for (int r = 0; r < reps; ++r) {
        switch (which) {
            case 0: smooth<double>(ctx, F, 1, false); b = n * 8 * (4 + coef); break;  // x,b,idiag r + x w + operator
            case 1: smooth<float>(ctx, F, 1, false); b = n * 4 * (4 + coef); break;
            case 2: IMPEC_TRY(pressure_residual(ctx)); b = n * 8 * (2 + coef) + (ctx->P.precision ? 4 * n : 0); break;
            case 3: IMPEC_TRY(advect_x_dev(ctx, ctx->c, ctx->t1, ctx->u, 1.0, &ctx->dscal->dt)); b = n * 24; break;
            case 4: IMPEC_TRY(advect_y_dev(ctx, ctx->c, ctx->t1, ctx->v, 1.0, &ctx->dscal->dt)); b = n * 24; break;
        }
    }
    IMPEC_CUDA_TRY(cudaEventRecord(e1, ctx->stream));
    IMPEC_CUDA_TRY(cudaEventSynchronize(e1));
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms) *ms = t / reps;
    if (bytes) *bytes = b;
    return IMPEC_OK;
}
