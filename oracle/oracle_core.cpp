// Impec2D CPU oracle -- TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// Each function restates the reference arithmetic in the same operation order
// (compiled with -ffp-contract=off) and cites the reference file:line it follows.
#include "oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

namespace {

// Ghost-indexed views over the flat layouts documented in oracle.h.
struct S2 {
    double* d; int g, n2t;
    double& operator()(int i, int j) const { return d[(size_t)(i + g) * n2t + (j + g)]; }
};
struct V3 {
    double* d; int g, n2t;
    double& operator()(int i, int j, int k) const { return d[((size_t)(i + g) * n2t + (j + g)) * 2 + k]; }
};
inline S2 sview(const or_params* P, const double* a) { return S2{const_cast<double*>(a), P->g, P->N2 + 2 * P->g}; }
inline V3 vview(const or_params* P, const double* v) { return V3{const_cast<double*>(v), P->g, P->N2 + 1 + 2 * P->g}; }

// Grid constants (src/EllipticSolver.cpp:59-100).
struct Geo {
    double dx, dy, dA, alpha, theta, dxi, deta, secamt, secamt2, cosa2, sina2, costsina,
        cosasint, cost2, sint2, cosa, sint, cost, sina, mob1over4;
    explicit Geo(const or_params* P) {
        dx = (P->x_ub - P->x_lb) / (P->N1);
        dy = (P->y_ub - P->y_lb) / (P->N2);
        dA = dx * dy;
        alpha = atan(dx / dy);
        theta = atan(dy / dx);
        dxi = dx / cos(theta);
        deta = dy / cos(alpha);
        secamt = 1. / cos(alpha - theta);
        secamt2 = secamt * secamt;
        cosa2 = cos(alpha) * cos(alpha);
        sina2 = sin(alpha) * sin(alpha);
        costsina = cos(theta) * sin(alpha);
        cosasint = cos(alpha) * sin(theta);
        cost2 = cos(theta) * cos(theta);
        sint2 = sin(theta) * sin(theta);
        cosa = cos(alpha);
        sint = sin(theta);
        cost = cos(theta);
        sina = sin(alpha);
        mob1over4 = pow(P->mu_res / P->mu_inj, 0.25);  // src/EllipticSolver.cpp:126
    }
};

// ---- permeability: analytic test cases (src/EllipticSolver.cpp:418-470) or per-cell field ----
inline double cell_index_from_x(double v, double lb, double h) { return floor((v - lb) / h); }

double K_11(const or_params* P, const Geo& G, double x, double y) {
    const double t = 2.;
    if (P->is_test) {
        switch (P->testno) {
            case 1: return 1.;
            case 2: return exp(-0.3 * x);
            case 3: return 2. + sin(t * x) * sin(y);
            case 4: return 2. + sin(t * x) * sin(y);
            default: return 1.;
        }
    }
    if (P->K11) {  // extension: heterogeneous field looked up by cell (x,y are cell centres)
        int i = (int)cell_index_from_x(x, P->x_lb, G.dx), j = (int)cell_index_from_x(y, P->y_lb, G.dy);
        i = i < 0 ? -1 - i : (i >= P->N1 ? 2 * P->N1 - 1 - i : i);
        j = j < 0 ? -1 - j : (j >= P->N2 ? 2 * P->N2 - 1 - j : j);
        return P->K11[(size_t)i * P->N2 + j];
    }
    return 1.;
}

double K_22(const or_params* P, const Geo& G, double x, double y) {
    const double t = 2.;
    if (P->is_test) {
        switch (P->testno) {
            case 1: return 1.;
            case 2: return exp(-0.3 * y);
            case 3: return 2. + sin(t * x) * sin(y);
            case 4: return 2. + sin(x) * sin(t * y);
            default: return 1.;
        }
    }
    const double* K = P->K22 ? P->K22 : P->K11;
    if (K) {
        int i = (int)cell_index_from_x(x, P->x_lb, G.dx), j = (int)cell_index_from_x(y, P->y_lb, G.dy);
        i = i < 0 ? -1 - i : (i >= P->N1 ? 2 * P->N1 - 1 - i : i);
        j = j < 0 ? -1 - j : (j >= P->N2 ? 2 * P->N2 - 1 - j : j);
        return K[(size_t)i * P->N2 + j];
    }
    return 1.;
}

// mu(c) (src/EllipticSolver.cpp:692-695)
inline double mu(const or_params* P, const Geo& G, double c) {
    double x = (1. - c + G.mob1over4 * c);
    return 1. / (x * x * x * x) * P->mu_res;
}

// KoverMu_11_im12j (src/EllipticSolver.cpp:478-500)
double KoverMu_11_im12j(const or_params* P, const Geo& G, double c_im1j, double c_ij, int i, int j) {
    double x = P->x_lb + (i + 0.5) * G.dx;
    double y = P->y_lb + (j + 0.5) * G.dy;
    double K11_im1j = K_11(P, G, x - G.dx, y);
    double K11_ij = K_11(P, G, x, y);
    double mu_ij = mu(P, G, c_ij);
    double mu_im1j = mu(P, G, c_im1j);
    if (P->avgproc == OR_HARMONIC) return 2. / (mu_im1j / K11_im1j + mu_ij / K11_ij);
    return 1. / 2 * (K11_im1j / mu_im1j + K11_ij / mu_ij);
}

// KoverMu_22_ijm12 (src/EllipticSolver.cpp:502-524)
double KoverMu_22_ijm12(const or_params* P, const Geo& G, double c_ijm1, double c_ij, int i, int j) {
    double x = P->x_lb + (i + 0.5) * G.dx;
    double y = P->y_lb + (j + 0.5) * G.dy;
    double K22_ijm1 = K_22(P, G, x, y - G.dy);
    double K22_ij = K_22(P, G, x, y);
    double mu_ij = mu(P, G, c_ij);
    double mu_ijm1 = mu(P, G, c_ijm1);
    if (P->avgproc == OR_HARMONIC) return 2. / (mu_ijm1 / K22_ijm1 + mu_ij / K22_ij);
    return 1. / 2 * (K22_ijm1 / mu_ijm1 + K22_ij / mu_ij);
}

// KoverMu_11_ip12jp12 / KoverMu_22_ip12jp12 (src/EllipticSolver.cpp:697-754)
double KoverMu_11_c(const or_params* P, const Geo& G, int i, int j, double c_ij, double c_ip1j,
                    double c_ijp1, double c_ip1jp1) {
    double x = P->x_lb + (i + 0.5) * G.dx;
    double y = P->y_lb + (j + 0.5) * G.dy;
    double K11_ip1j = K_11(P, G, x + G.dx, y);
    double K11_ij = K_11(P, G, x, y);
    double K11_ijp1 = K_11(P, G, x, y + G.dy);
    double K11_ip1jp1 = K_11(P, G, x + G.dx, y + G.dy);
    double mu_ip1j = mu(P, G, c_ip1j), mu_ij = mu(P, G, c_ij), mu_ijp1 = mu(P, G, c_ijp1),
           mu_ip1jp1 = mu(P, G, c_ip1jp1);
    if (P->avgproc == OR_HARMONIC)
        return 4. / (mu_ip1j / K11_ip1j + mu_ij / K11_ij + mu_ijp1 / K11_ijp1 + mu_ip1jp1 / K11_ip1jp1);
    return 1. / 4 * (K11_ip1j / mu_ip1j + K11_ij / mu_ij + K11_ijp1 / mu_ijp1 + K11_ip1jp1 / mu_ip1jp1);
}
double KoverMu_22_c(const or_params* P, const Geo& G, int i, int j, double c_ij, double c_ip1j,
                    double c_ijp1, double c_ip1jp1) {
    double x = P->x_lb + (i + 0.5) * G.dx;
    double y = P->y_lb + (j + 0.5) * G.dy;
    double K22_ip1j = K_22(P, G, x + G.dx, y);
    double K22_ij = K_22(P, G, x, y);
    double K22_ijp1 = K_22(P, G, x, y + G.dy);
    double K22_ip1jp1 = K_22(P, G, x + G.dx, y + G.dy);
    double mu_ip1j = mu(P, G, c_ip1j), mu_ij = mu(P, G, c_ij), mu_ijp1 = mu(P, G, c_ijp1),
           mu_ip1jp1 = mu(P, G, c_ip1jp1);
    if (P->avgproc == OR_HARMONIC)
        return 4. / (mu_ip1j / K22_ip1j + mu_ij / K22_ij + mu_ijp1 / K22_ijp1 + mu_ip1jp1 / K22_ip1jp1);
    return 1. / 4 * (K22_ip1j / mu_ip1j + K22_ij / mu_ij + K22_ijp1 / mu_ijp1 + K22_ip1jp1 / mu_ip1jp1);
}

// GetParallelCoefficientsForCell (src/MGSolver.cpp:760-773)
void parallel_coeffs(const or_params* P, const Geo& G, const S2& c, int i, int j, double& W, double& S,
                     double& C, double& N, double& E) {
    double K11_im12j = KoverMu_11_im12j(P, G, c(i - 1, j), c(i, j), i, j);
    double K11_ip12j = KoverMu_11_im12j(P, G, c(i, j), c(i + 1, j), i + 1, j);
    double K22_ijm12 = KoverMu_22_ijm12(P, G, c(i, j - 1), c(i, j), i, j);
    double K22_ijp12 = KoverMu_22_ijm12(P, G, c(i, j), c(i, j + 1), i, j + 1);
    const double dx = G.dx, dy = G.dy;
    W = 1. / (dx * dx) * K11_im12j;
    E = 1. / (dx * dx) * K11_ip12j;
    S = 1. / (dy * dy) * K22_ijm12;
    N = 1. / (dy * dy) * K22_ijp12;
    C = -1. / (dy * dy) * (K22_ijm12 + K22_ijp12) - 1. / (dx * dx) * (K11_im12j + K11_ip12j);
}

// GetDiagonalCoefficientsForCell + GetTransformedMobilityTensor (src/MGSolver.cpp:777-841)
void diagonal_coeffs(const or_params* P, const Geo& G, const S2& c, int i, int j, double& W, double& NW,
                     double& N, double& NE, double& E, double& SE, double& S, double& SW, double& C) {
    const double K11_ip12jp12 = KoverMu_11_c(P, G, i, j, c(i, j), c(i + 1, j), c(i, j + 1), c(i + 1, j + 1));
    const double K11_im12jm12 = KoverMu_11_c(P, G, i - 1, j - 1, c(i - 1, j - 1), c(i, j - 1), c(i - 1, j), c(i, j));
    const double K11_im12jp12 = KoverMu_11_c(P, G, i - 1, j, c(i - 1, j), c(i, j), c(i - 1, j + 1), c(i, j + 1));
    const double K11_ip12jm12 = KoverMu_11_c(P, G, i, j - 1, c(i, j - 1), c(i + 1, j - 1), c(i, j), c(i + 1, j));
    const double K22_ip12jp12 = KoverMu_22_c(P, G, i, j, c(i, j), c(i + 1, j), c(i, j + 1), c(i + 1, j + 1));
    const double K22_im12jm12 = KoverMu_22_c(P, G, i - 1, j - 1, c(i - 1, j - 1), c(i, j - 1), c(i - 1, j), c(i, j));
    const double K22_im12jp12 = KoverMu_22_c(P, G, i - 1, j, c(i - 1, j), c(i, j), c(i - 1, j + 1), c(i, j + 1));
    const double K22_ip12jm12 = KoverMu_22_c(P, G, i, j - 1, c(i, j - 1), c(i + 1, j - 1), c(i, j), c(i + 1, j));
    double M11_ip12j = G.secamt2 * (K11_ip12jp12 * G.cosa2 + K22_ip12jp12 * G.sina2);
    double M11_im12j = G.secamt2 * (K11_im12jm12 * G.cosa2 + K22_im12jm12 * G.sina2);
    double M22_ijp12 = G.secamt2 * (K22_im12jp12 * G.cost2 + K11_im12jp12 * G.sint2);
    double M22_ijm12 = G.secamt2 * (K22_ip12jm12 * G.cost2 + K11_ip12jm12 * G.sint2);
    double M12_ip12j = G.secamt2 * (K22_ip12jp12 * G.costsina - K11_ip12jp12 * G.cosasint);
    double M21_ijp12 = G.secamt2 * (K22_im12jp12 * G.costsina - K11_im12jp12 * G.cosasint);
    double M12_im12j = G.secamt2 * (K22_im12jm12 * G.costsina - K11_im12jm12 * G.cosasint);
    double M21_ijm12 = G.secamt2 * (K22_ip12jm12 * G.costsina - K11_ip12jm12 * G.cosasint);
    const double dxi = G.dxi, deta = G.deta;
    NE = M11_ip12j / (dxi * dxi);
    SW = M11_im12j / (dxi * dxi);
    NW = M22_ijp12 / (deta * deta);
    SE = M22_ijm12 / (deta * deta);
    C = -1. / (dxi * dxi) * (M11_ip12j + M11_im12j) - 1. / (deta * deta) * (M22_ijp12 + M22_ijm12);
    N = 1. / (deta * dxi) * (M12_ip12j + M21_ijp12);
    W = -1. / (deta * dxi) * (M21_ijp12 + M12_im12j);
    E = -1. / (deta * dxi) * (M12_ip12j + M21_ijm12);
    S = 1. / (deta * dxi) * (M12_im12j + M21_ijm12);
}

// GetWeightedMatrixCoefficientsForCell (src/MGSolver.cpp:710-757); v[] in HYPRE order
void weighted_coeffs(const or_params* P, const Geo& G, const S2& c, int i, int j, double* v) {
    double C_p = 0, W_p = 0, SW_p = 0, S_p = 0, SE_p = 0, E_p = 0, NE_p = 0, N_p = 0, NW_p = 0;
    double C_d = 0, W_d = 0, SW_d = 0, S_d = 0, SE_d = 0, E_d = 0, NE_d = 0, N_d = 0, NW_d = 0;
    parallel_coeffs(P, G, c, i, j, W_p, S_p, C_p, N_p, E_p);
    diagonal_coeffs(P, G, c, i, j, W_d, NW_d, N_d, NE_d, E_d, SE_d, S_d, SW_d, C_d);
    const double nu = P->nu;
    v[0] = nu * C_p + (1 - nu) * C_d;
    v[1] = nu * W_p + (1 - nu) * W_d;
    v[2] = nu * SW_p + (1 - nu) * SW_d;
    v[3] = nu * S_p + (1 - nu) * S_d;
    v[4] = nu * SE_p + (1 - nu) * SE_d;
    v[5] = nu * E_p + (1 - nu) * E_d;
    v[6] = nu * NE_p + (1 - nu) * NE_d;
    v[7] = nu * N_p + (1 - nu) * N_d;
    v[8] = nu * NW_p + (1 - nu) * NW_d;
}

// Neumann folding of a 9-point row (src/MGSolver.cpp:304-515 and :1031-1289, identical pattern).
// Entry order: 0 C, 1 W, 2 SW, 3 S, 4 SE, 5 E, 6 NE, 7 N, 8 NW.  Edge rows are set first,
// then the four corners are overwritten, as in the reference.
void fold_row(int k, int l, int N1, int N2, const double* s, double* out) {
    const double C = s[0], W = s[1], SW = s[2], S = s[3], SE = s[4], E = s[5], NE = s[6], N = s[7],
                 NW = s[8];
    for (int e = 0; e < 9; ++e) out[e] = s[e];
    auto set = [&](double a0, double a1, double a2, double a3, double a4, double a5, double a6, double a7,
                   double a8) {
        out[0] = a0; out[1] = a1; out[2] = a2; out[3] = a3; out[4] = a4;
        out[5] = a5; out[6] = a6; out[7] = a7; out[8] = a8;
    };
    if (l == 0) set(C + S, W + SW, 0, 0, 0, E + SE, NE, N, NW);
    if (l == N2 - 1) set(C + N, W + NW, SW, S, SE, E + NE, 0, 0, 0);
    if (k == 0) set(C + W, 0, 0, S + SW, SE, E, NE, N + NW, 0);
    if (k == N1 - 1) set(C + E, W, SW, S + SE, 0, 0, 0, N + NE, NW);
    if (k == 0 && l == 0) set(C + W + S + SW, 0, 0, 0, 0, E + SE, NE, N + NW, 0);
    if (k == 0 && l == N2 - 1) set(C + W + N + NW, 0, 0, S + SW, SE, E + NE, 0, 0, 0);
    if (k == N1 - 1 && l == N2 - 1) set(C + N + NE + E, W + NW, SW, S + SE, 0, 0, 0, 0, 0);
    if (k == N1 - 1 && l == 0) set(C + S + E + SE, W + SW, 0, 0, 0, 0, 0, N + NE, NW);
}

// Test source terms (src/EllipticSolver.cpp:319-353)
double qTest(const or_params* P, double x, double y) {
    double mr = P->mu_res;
    switch (P->testno) {
        case 1: return 2. / mr * cos(x) * cos(y);
        case 2: {
            double c1 = -0.3, c2 = -0.3;
            double a1 = exp(c1 * x), a2 = exp(c2 * y), a1_x = c1 * exp(c1 * x), a2_y = c2 * exp(c2 * y);
            return 1. / mr * ((a1 + a2) * cos(x) * cos(y) + a1_x * sin(x) * cos(y) + a2_y * cos(x) * sin(y));
        }
        case 3: {
            double t = 2.;
            double a1 = 2. + sin(t * x) * sin(y), a2 = 2. + sin(t * x) * sin(y);
            double a1_x = t * cos(t * x) * sin(y), a2_y = cos(y) * sin(t * x);
            return 1. / mr * ((a1 + a2) * cos(x) * cos(y) + a1_x * sin(x) * cos(y) + a2_y * cos(x) * sin(y));
        }
        case 4: {
            double t = 2.;
            double a1 = 2. + sin(t * x) * sin(y), a2 = 2. + sin(x) * sin(t * y);
            double a1_x = t * cos(t * x) * sin(y), a2_y = t * cos(t * y) * sin(x);
            return 1. / mr * ((a1 + a2) * cos(x) * cos(y) + a1_x * sin(x) * cos(y) + a2_y * cos(x) * sin(y));
        }
    }
    return 0.;
}
inline double pTest(double x, double y) { return cos(x) * cos(y); }

// Cells pinned by a Dirichlet row in the elliptic matrix (src/MGSolver.cpp:109-140).
void pinned_cells(const or_params* P, std::vector<std::pair<int, int>>& cells) {
    cells.clear();
    if (P->stype == OR_HORIZONTAL) {
        for (int j = 0; j < P->N2; ++j) cells.push_back({1, j});
    } else {
        cells.push_back({1, 1});
    }
}

// Dirichlet row value kappa/dA (src/MGSolver.cpp:518-567)
double pin_kappa(const or_params* P, const Geo& G, int di, int dj) {
    if (P->is_test) {
        double x = P->x_lb + (di + 0.5) * (P->x_ub - P->x_lb) / P->N1;
        double y = P->y_lb + (dj + 0.5) * (P->y_ub - P->y_lb) / P->N2;
        double qij = qTest(P, x, y);
        double pij = pTest(x, y);
        return -G.dA * qij / pij;
    }
    return 1.;
}

void assemble_pressure(const or_params* P, const double* cflat, double* A9, bool pin) {
    Geo G(P);
    S2 c = sview(P, cflat);
    const int N1 = P->N1, N2 = P->N2;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < N1; ++k) {
        double s[9];
        for (int l = 0; l < N2; ++l) {
            weighted_coeffs(P, G, c, k, l, s);
            fold_row(k, l, N1, N2, s, A9 + ((size_t)k * N2 + l) * 9);
        }
    }
    if (pin) {
        std::vector<std::pair<int, int>> cells;
        pinned_cells(P, cells);
        for (auto& pc : cells) {
            if (pc.first < 0 || pc.first >= N1 || pc.second < 0 || pc.second >= N2) continue;
            double* row = A9 + ((size_t)pc.first * N2 + pc.second) * 9;
            row[0] = pin_kappa(P, G, pc.first, pc.second) / G.dA;
            for (int e = 1; e < 9; ++e) row[e] = 0;
        }
    }
}

const int OFF[9][2] = {{0, 0}, {-1, 0}, {-1, -1}, {0, -1}, {1, -1}, {1, 0}, {1, 1}, {0, 1}, {-1, 1}};

}  // namespace

extern "C" {

// ---------------------------------------------------------------- ghost fills
// FillGhostCellsNeumannScalar (src/Util.cpp:283-324)
void or_fill_scalar_neumann(const or_params* P, double* a) {
    S2 arr = sview(P, a);
    const int n = P->g, xN = P->N1 - 1, yN = P->N2 - 1;
    for (int i = 0; i <= xN; i++)
        for (int j = 0; j < n; j++) {
            arr(i, yN + j + 1) = arr(i, yN - j);
            arr(i, -(j + 1)) = arr(i, j);
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j <= yN; j++) {
            arr(-(i + 1), j) = arr(i, j);
            arr(xN + i + 1, j) = arr(xN - i, j);
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            arr(-(i + 1), -(j + 1)) = arr(i, j);
            arr(xN + i + 1, -(j + 1)) = arr(xN - i, j);
            arr(-(i + 1), yN + j + 1) = arr(i, yN - j);
            arr(xN + i + 1, yN + j + 1) = arr(xN - i, yN - j);
        }
}

// FillGhostCellsPeriodicScalar (src/Util.cpp:215-256)
void or_fill_scalar_periodic(const or_params* P, double* a) {
    S2 arr = sview(P, a);
    const int n = P->g, xN = P->N1 - 1, yN = P->N2 - 1;
    for (int i = 0; i <= xN; i++)
        for (int j = 0; j < n; j++) {
            arr(i, yN + j + 1) = arr(i, j);
            arr(i, -(j + 1)) = arr(i, yN - j);
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j <= yN; j++) {
            arr(-(i + 1), j) = arr(xN - i, j);
            arr(xN + i + 1, j) = arr(i, j);
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            arr(-(i + 1), -(j + 1)) = arr(xN - i, yN - j);
            arr(xN + i + 1, -(j + 1)) = arr(i, yN - j);
            arr(-(i + 1), yN + j + 1) = arr(xN - i, j);
            arr(xN + i + 1, yN + j + 1) = arr(i, j);
        }
}

// FillGhostCellsNeumannVelocity (src/Util.cpp:331-438)
void or_fill_velocity_neumann(const or_params* P, double* vflat) {
    V3 v = vview(P, vflat);
    const int n = P->g, xN = P->N1, yN = P->N2;
    for (int i = 0; i <= xN; i++)
        for (int j = 0; j < n; j++) {
            v(i, -(j + 1), 0) = v(i, j, 0);
            v(i, yN + j, 0) = v(i, yN - 1 - j, 0);
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            v(-(i + 1), yN + j, 0) = -v(i + 1, yN + j, 0);
            v(-(i + 1), -(j + 1), 0) = -v(i + 1, -(j + 1), 0);
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            v(xN + i + 1, yN + j, 0) = -v(xN - 1 - i, yN + j, 0);
            v(xN + i + 1, -(j + 1), 0) = -v(xN - i - 1, -(j + 1), 0);
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < yN; j++) {
            v(-(i + 1), j, 0) = -v(i + 1, j, 0);
            v(xN + i + 1, j, 0) = -v(xN - i - 1, j, 0);
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j <= yN; j++) {
            v(-(i + 1), j, 1) = v(i, j, 1);
            v(xN + i, j, 1) = v(xN - i - 1, j, 1);
        }
    for (int i = 0; i < xN; i++)
        for (int j = 0; j < n; j++) {
            v(i, -(j + 1), 1) = -v(i, j + 1, 1);
            v(i, yN + j + 1, 1) = -v(i, yN - 1 - j, 1);
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            v(-(i + 1), yN + 1 + j, 1) = v(i, yN + 1 + j, 1);
            v(-(i + 1), -(j + 1), 1) = v(i, -(j + 1), 1);
        }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            v(xN + i, yN + 1 + j, 1) = v(xN - 1 - i, yN + j + 1, 1);
            v(xN + i, -(j + 1), 1) = v(xN - 1 - i, -(j + 1), 1);
        }
}

// ---------------------------------------------------------------- elliptic
double or_mu(const or_params* P, double c) {
    Geo G(P);
    return mu(P, G, c);
}

// SetMatrixCoefficients_Elliptic (src/MGSolver.cpp:268-570)
void or_pressure_matrix(const or_params* P, const double* c, double* A9) { assemble_pressure(P, c, A9, true); }
void or_pressure_matrix_neumann(const or_params* P, const double* c, double* A9) {
    assemble_pressure(P, c, A9, false);
}

// Face mobilities as used by GetParallelCoefficientsForCell / GetParallelU*:
// lamx(i,j) = KoverMu_11_im12j(c(i-1,j), c(i,j), i, j) for i in [0,N1], j in [0,N2);
// lamy(i,j) = KoverMu_22_ijm12(c(i,j-1), c(i,j), i, j) for i in [0,N1), j in [0,N2].
void or_face_mobility(const or_params* P, const double* cflat, double* lamx, double* lamy) {
    Geo G(P);
    S2 c = sview(P, cflat);
    for (int i = 0; i <= P->N1; ++i)
        for (int j = 0; j < P->N2; ++j)
            lamx[(size_t)i * P->N2 + j] = KoverMu_11_im12j(P, G, c(i - 1, j), c(i, j), i, j);
    for (int i = 0; i < P->N1; ++i)
        for (int j = 0; j <= P->N2; ++j)
            lamy[(size_t)i * (P->N2 + 1) + j] = KoverMu_22_ijm12(P, G, c(i, j - 1), c(i, j), i, j);
}

// SetRHS_Elliptic (src/MGSolver.cpp:573-590): b = -q
void or_pressure_rhs(const or_params* P, const double* q, double* b) {
    const size_t M = (size_t)P->N1 * P->N2;
    for (size_t k = 0; k < M; ++k) b[k] = -q[k];
}

void or_matvec9(const or_params* P, const double* A9, const double* x, double* y) {
    const int N1 = P->N1, N2 = P->N2;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N1; ++i)
        for (int j = 0; j < N2; ++j) {
            const double* a = A9 + ((size_t)i * N2 + j) * 9;
            double s = 0;
            for (int e = 0; e < 9; ++e) {
                int ii = i + OFF[e][0], jj = j + OFF[e][1];
                if (ii < 0 || ii >= N1 || jj < 0 || jj >= N2) continue;
                s += a[e] * x[(size_t)ii * N2 + jj];
            }
            y[(size_t)i * N2 + j] = s;
        }
}

double or_relres9(const or_params* P, const double* A9, const double* x, const double* b) {
    const size_t M = (size_t)P->N1 * P->N2;
    std::vector<double> y(M);
    or_matvec9(P, A9, x, y.data());
    long double rr = 0, bb = 0;
    for (size_t k = 0; k < M; ++k) {
        long double r = (long double)b[k] - y[k];
        rr += r * r;
        bb += (long double)b[k] * b[k];
    }
    return bb > 0 ? (double)sqrtl(rr / bb) : (double)sqrtl(rr);
}

// CalcVelocities (src/EllipticSolver.cpp:541-683)
void or_calc_velocities(const or_params* P, double* pflat, double* vflat, const double* cflat) {
    Geo G(P);
    or_fill_scalar_neumann(P, pflat);
    S2 p = sview(P, pflat), c = sview(P, cflat);
    V3 v = vview(P, vflat);
    const double nu = P->nu, dx = G.dx, dy = G.dy;
    auto M_im12j = [&](int i, int j, double& M11, double& M12, double& M21, double& M22) {
        const double K11 = KoverMu_11_c(P, G, i - 1, j - 1, c(i - 1, j - 1), c(i, j - 1), c(i - 1, j), c(i, j));
        const double K22 = KoverMu_22_c(P, G, i - 1, j - 1, c(i - 1, j - 1), c(i, j - 1), c(i - 1, j), c(i, j));
        M11 = G.secamt2 * (K11 * G.cosa2 + K22 * G.sina2);
        M12 = G.secamt2 * (K22 * G.costsina - K11 * G.cosasint);
        M21 = G.secamt2 * (K22 * G.costsina - K11 * G.cosasint);
        M22 = G.secamt2 * (K11 * G.sint2 + K22 * G.cost2);
    };
    auto W_im12j = [&](int i, int j, double& w1, double& w2) {
        double d1dp = 1. / G.dxi * (p(i, j) - p(i - 1, j - 1));
        double d2dp = 1. / G.deta * (p(i - 1, j) - p(i, j - 1));
        double M11, M12, M21, M22;
        M_im12j(i, j, M11, M12, M21, M22);
        w1 = -d1dp * M11 - d2dp * M12;
        w2 = -d1dp * M21 - d2dp * M22;
    };
    auto fromXiEta = [&](double& v1, double& v2, double w1, double w2) {
        v1 = G.cost * w1 - G.sina * w2;
        v2 = G.sint * w1 + G.cosa * w2;
    };
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= P->N1; i++)
        for (int j = 0; j < P->N2; j++) {
            double par = -KoverMu_11_im12j(P, G, c(i - 1, j), c(i, j), i, j) * (p(i, j) - p(i - 1, j)) / dx;
            double w1m, w2m, w1p, w2p, u1m, u2m, u1p, u2p;
            W_im12j(i, j, w1m, w2m);
            W_im12j(i, j + 1, w1p, w2p);
            fromXiEta(u1m, u2m, w1m, w2m);
            fromXiEta(u1p, u2p, w1p, w2p);
            double diag = 0.5 * (u1p + u1m);
            v(i, j, 0) = nu * par + (1. - nu) * diag;
        }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < P->N1; i++)
        for (int j = 0; j <= P->N2; j++) {
            double par = -KoverMu_22_ijm12(P, G, c(i, j - 1), c(i, j), i, j) * (p(i, j) - p(i, j - 1)) / dy;
            double w1m, w2m, w1p, w2p, u1m, u2m, u1p, u2p;
            W_im12j(i, j, w1m, w2m);
            W_im12j(i + 1, j, w1p, w2p);
            fromXiEta(u1m, u2m, w1m, w2m);
            fromXiEta(u1p, u2p, w1p, w2p);
            double diag = 0.5 * (u2m + u2p);
            v(i, j, 1) = nu * par + (1. - nu) * diag;
        }
    or_fill_velocity_neumann(P, vflat);
}

// MaxStableTimestepCombined (src/HyperbolicSolver.cpp:123-198)
double or_max_stable_dt(const or_params* P, const double* vflat) {
    Geo G(P);
    V3 v = vview(P, vflat);
    double maxvel = 0;
    for (int i = 0; i < P->N1; i++)
        for (int j = 0; j < P->N2; j++) {
            double u_c = fabs((double)(0.5 * (v(i, j, 0) + v(i + 1, j, 0))));
            double v_c = fabs((double)(0.5 * (v(i, j, 1) + v(i, j + 1, 1))));
            if (u_c < std::numeric_limits<double>::min()) u_c = std::numeric_limits<double>::min();
            if (v_c < std::numeric_limits<double>::min()) v_c = std::numeric_limits<double>::min();
            if (maxvel < fabs(u_c)) maxvel = fabs(u_c);
            if (maxvel < fabs(v_c)) maxvel = fabs(v_c);
        }
    double dt_advec = std::min(G.dx / maxvel, G.dy / maxvel);
    dt_advec *= P->cfl;
    double dt_diff = std::numeric_limits<double>::max();
    if (P->diffusion) {
        double dmin = 1.e10;
        const double al = P->alpha_l, at = P->alpha_t, dx = G.dx;
        for (int i = 0; i < P->N1; i++)
            for (int j = 0; j < P->N2; j++) {
                double vij = 0.5 * (v(i, j, 1) + v(i, j + 1, 1));
                double uij = 0.5 * (v(i, j, 0) + v(i + 1, j, 0));
                double vij2 = vij * vij, uij2 = uij * uij;
                double absu = sqrt(vij2 + uij2);
                double d11 = dx / absu * (al * uij2 + at * vij2);
                double d22 = dx / absu * (al * vij2 + at * uij2);
                double dt = 1. / 2 * dx * dx / (d11 + d22);
                if (dt < dmin) dmin = dt;
            }
        dt_diff = dmin * P->dt_diff_limit;
    }
    if (P->ptype == OR_CRANKNICOLSON) return dt_advec;
    return std::min(dt_diff, dt_advec);
}

// MaxStableAdvectionTimestep (src/HyperbolicSolver.cpp:96-121)
double or_max_stable_advection_dt(const or_params* P, const double* vflat) {
    Geo G(P);
    V3 v = vview(P, vflat);
    double dt_max = std::numeric_limits<double>::max();
    for (int i = 0; i < P->N1; i++)
        for (int j = 0; j < P->N2; j++) {
            double u_c = fabs((double)(0.5 * (v(i, j, 0) + v(i + 1, j, 0))));
            double v_c = fabs((double)(0.5 * (v(i, j, 1) + v(i, j + 1, 1))));
            if (u_c < std::numeric_limits<double>::min()) u_c = std::numeric_limits<double>::min();
            if (v_c < std::numeric_limits<double>::min()) v_c = std::numeric_limits<double>::min();
            double dt = std::min(G.dx / u_c, G.dy / v_c);
            if (dt < dt_max) dt_max = dt;
        }
    return dt_max * P->cfl;
}

// ---------------------------------------------------------------- hyperbolic
// TRIntegrator::Integrate (src/TRIntegrator.cpp:49-71); returns total_mass_outflux
double or_tr_integrate(const or_params* P, double* cflat, const double* q, double dt) {
    S2 c = sview(P, cflat);
    double tmo = 0;
    for (int i = 0; i < P->N1; i++)
        for (int j = 0; j < P->N2; j++) {
            double qij = q[(size_t)i * P->N2 + j];
            if (qij < 0) {
                double massdiff = c(i, j);
                c(i, j) = c(i, j) * (1 + 0.5 * dt * qij) / (1 - 0.5 * dt * qij);
                massdiff = c(i, j) - massdiff;
                tmo += massdiff;
            } else if (qij > 0)
                c(i, j) += dt * P->inj_fluid_conc * qij;
        }
    return tmo;
}

}  // extern "C"

namespace {

inline double flux(const or_params* P, double vel, double conc) { return vel * conc / P->porosity; }  // HyperbolicSolver::Flux :208

// MUSCLSplitSolver::SlopeLimiter / GetSlope / Reconstruct (src/MUSCLSplitSolver.cpp:54-93)
inline double slope_limiter(double du_m, double du_p) {
    double w = 0.;
    if (du_m * du_p > 0) {
        double r = du_m / du_p;
        if (r > std::numeric_limits<double>::max()) r = std::numeric_limits<double>::max();
        double beta_plus = 1;
        double zr = 2 * beta_plus / (1 - w + (1 + w) * r);
        return std::min(2. * r / (1. + r), zr);
    }
    return 0;
}
inline double get_slope(double a, double b) {
    double w = 0.;
    return slope_limiter(a, b) * 0.5 * ((1 + w) * a + (1 - w) * b);
}
inline void reconstruct(double U_i, double U_ip1, double U_im1, double& UL, double& UR) {
    double dU_prev = U_i - U_im1;
    double dU_next = U_ip1 - U_i;
    double d_i = get_slope(dU_prev, dU_next);
    UR = U_i + 0.5 * d_i;
    UL = U_i - 0.5 * d_i;
}
inline double upwind(const or_params* P, double speed, double UL, double UR) {  // src/UpwindSplitSolver.cpp:63-65
    return (speed > 0) ? flux(P, speed, UL) : flux(P, speed, UR);
}

// WAF intercell flux for the linear flux f = vel c / phi (hyper_method "waf_split" / "waf";
// parsed by the reference, src/SimParams.cpp:200-208, which ships no source for it).  Toro's
// weighted average flux, Riemann Solvers and Numerical Methods for Fluid Dynamics (3rd ed.),
// ch. 13-14: F = (1 + s A)/2 f(cL) + (1 - s A)/2 f(cR), s = sign of the Courant number
// cr = vel dt / (phi dx), A = 1 - (1 - |cr|) psi(r) with the van Leer limiter
// psi(r) = 2r / (1 + r) for r > 0, else 0 (the limiter the recorded WAF order names,
// examples/hyperbolic_test.cfg:136), r = upwind jump / local jump.  psi = 1 gives Lax-Wendroff,
// psi = 0 the upwind (Godunov) flux.
inline double waf_flux(const or_params* P, double vel, double dtdx, double cLL, double cL, double cR, double cRR) {
    const double cr = vel / P->porosity * dtdx;
    const double dloc = cR - cL;
    double A = 1.0;
    if (dloc != 0.0) {
        const double dupw = cr >= 0 ? cL - cLL : cRR - cR;
        const double r = dupw / dloc;
        if (r > 0) A = 1.0 - (1.0 - std::fabs(cr)) * (2.0 * r / (1.0 + r));
    }
    const double s = cr > 0 ? 1.0 : (cr < 0 ? -1.0 : 0.0);
    return 0.5 * (1.0 + s * A) * flux(P, vel, cL) + 0.5 * (1.0 - s * A) * flux(P, vel, cR);
}

inline bool is_waf(const or_params* P) { return P->hmtype == OR_WAFSPLIT || P->hmtype == OR_WAF; }

}  // namespace

extern "C" {

// F has (N1+1) x (N2+2g) entries, F(i,j) at i*(N2+2g) + (j+g).
void or_flux_F(const or_params* P, double* Fflat, const double* cflat, const double* vflat, double dt) {
    Geo G(P);
    S2 c = sview(P, cflat);
    V3 v = vview(P, vflat);
    const int g = P->g, N1 = P->N1, N2 = P->N2, w = N2 + 2 * g;
    auto F = [&](int i, int j) -> double& { return Fflat[(size_t)i * w + (j + g)]; };
    if (P->hmtype == OR_UPWINDSPLIT) {  // src/UpwindSplitSolver.cpp:43-51
        for (int i = 0; i <= N1; i++)
            for (int j = -g; j < N2 + g; j++) F(i, j) = upwind(P, v(i, j, 0), c(i - 1, j), c(i, j));
        return;
    }
    if (is_waf(P)) {
        for (int i = 0; i <= N1; i++)
            for (int j = -g; j < N2 + g; j++)
                F(i, j) = waf_flux(P, v(i, j, 0), dt / G.dx, c(i - 2, j), c(i - 1, j), c(i, j), c(i + 1, j));
        return;
    }
    // src/MUSCLSplitSolver.cpp:102-141; U_Lin base (-1,-g,0), extent (N1+3)
    std::vector<double> U((size_t)(N1 + 3) * w * 2, 0.0);
    auto UL_ = [&](int i, int j, int k) -> double& { return U[((size_t)(i + 1) * w + (j + g)) * 2 + k]; };
#pragma omp parallel for schedule(static)
    for (int i = -1; i <= N1; i++)
        for (int j = -g; j < N2 + g; j++) {
            double UL, UR;
            reconstruct(c(i, j), c(i + 1, j), c(i - 1, j), UL, UR);
            double df = 0.5 * dt / G.dx * (flux(P, v(i, j, 0), UL) - flux(P, v(i + 1, j, 0), UR));
            UL_(i + 1, j, 0) = UR + df;
            UL_(i, j, 1) = UL + df;
        }
    for (int i = 0; i <= N1; i++)
        for (int j = -g; j < N2 + g; j++) F(i, j) = upwind(P, v(i, j, 0), UL_(i, j, 0), UL_(i, j, 1));
}

// G has (N1+2g) x (N2+1) entries, G(i,j) at (i+g)*(N2+1) + j.
void or_flux_G(const or_params* P, double* Gflat, const double* cflat, const double* vflat, double dt) {
    Geo Ge(P);
    S2 c = sview(P, cflat);
    V3 v = vview(P, vflat);
    const int g = P->g, N1 = P->N1, N2 = P->N2, w = N2 + 1;
    auto Gf = [&](int i, int j) -> double& { return Gflat[(size_t)(i + g) * w + j]; };
    if (P->hmtype == OR_UPWINDSPLIT) {  // src/UpwindSplitSolver.cpp:53-61
        for (int i = -g; i < N1 + g; i++)
            for (int j = 0; j <= N2; j++) Gf(i, j) = upwind(P, v(i, j, 1), c(i, j - 1), c(i, j));
        return;
    }
    if (is_waf(P)) {
        for (int i = -g; i < N1 + g; i++)
            for (int j = 0; j <= N2; j++)
                Gf(i, j) = waf_flux(P, v(i, j, 1), dt / Ge.dy, c(i, j - 2), c(i, j - 1), c(i, j), c(i, j + 1));
        return;
    }
    // src/MUSCLSplitSolver.cpp:152-189; U_Lin base (-g,-1,0), extent (N2+3)
    const int wu = N2 + 3;
    std::vector<double> U((size_t)(N1 + 1 + 2 * g) * wu * 2, 0.0);
    auto UL_ = [&](int i, int j, int k) -> double& { return U[((size_t)(i + g) * wu + (j + 1)) * 2 + k]; };
#pragma omp parallel for schedule(static)
    for (int i = -g; i < N1 + g; i++)
        for (int j = -1; j <= N2; j++) {
            double UL, UR;
            reconstruct(c(i, j), c(i, j + 1), c(i, j - 1), UL, UR);
            double df = 0.5 * dt / Ge.dy * (flux(P, v(i, j, 1), UL) - flux(P, v(i, j + 1, 1), UR));
            UL_(i, j + 1, 0) = UR + df;
            UL_(i, j, 1) = UL + df;
        }
    for (int i = -g; i < N1 + g; i++)
        for (int j = 0; j <= N2; j++) Gf(i, j) = upwind(P, v(i, j, 1), UL_(i, j, 0), UL_(i, j, 1));
}

// Advect_X (src/HyperbolicSplitSolver.cpp:113-133)
void or_advect_x(const or_params* P, double* cflat, const double* v, double dt) {
    Geo G(P);
    const int g = P->g, w = P->N2 + 2 * g;
    std::vector<double> F((size_t)(P->N1 + 1) * w, 0.0);
    or_flux_F(P, F.data(), cflat, v, dt);
    S2 c = sview(P, cflat);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < P->N1; i++)
        for (int j = -g; j < P->N2 + g; j++)
            c(i, j) += dt / G.dx * (F[(size_t)i * w + (j + g)] - F[(size_t)(i + 1) * w + (j + g)]);
}

// Advect_Y (src/HyperbolicSplitSolver.cpp:139-159)
void or_advect_y(const or_params* P, double* cflat, const double* v, double dt) {
    Geo G(P);
    const int g = P->g, w = P->N2 + 1;
    std::vector<double> Gf((size_t)(P->N1 + 2 * g) * w, 0.0);
    or_flux_G(P, Gf.data(), cflat, v, dt);
    S2 c = sview(P, cflat);
#pragma omp parallel for schedule(static)
    for (int i = -g; i < P->N1 + g; i++)
        for (int j = 0; j < P->N2; j++)
            c(i, j) += dt / G.dy * (Gf[(size_t)(i + g) * w + j] - Gf[(size_t)(i + g) * w + j + 1]);
}

static void fill_boundaries(const or_params* P, double* c) {  // HyperbolicSolver::FillBoundaries :56-61
    if (P->is_test)
        or_fill_scalar_periodic(P, c);
    else
        or_fill_scalar_neumann(P, c);
}

// Corner transport upwind (hyper_method "ctu"; parsed by the reference, src/SimParams.cpp:
// 200-208, which ships no source for it): Colella's unsplit second-order scheme, J. Comput.
// Phys. 87 (1990) 171-200, for c_t + div(V c) / phi = 0 with face velocities.  Each face takes
// the state of its upwind cell m extrapolated to the face and the half time level,
//   c(m) +- (1 -+ a dt/dx) sx(m) / 2 - dt/(2 dy) b(m) dyc(m),
// with a the face speed, sx(m) the central slope (c(m+1) - c(m-1)) / 2 (unlimited: the
// recorded CTU order is labelled "2nd order", examples/hyperbolic_test.cfg:137), b(m) the
// cell-centred transverse speed and dyc(m) its upwind difference; then the conservative
// unsplit update of the interior.  Speeds are velocity / phi; CFL <= 1 per direction.
void or_ctu_advect(const or_params* P, double* cflat, const double* vflat, double dt) {
    Geo G(P);
    S2 c = sview(P, cflat);
    V3 v = vview(P, vflat);
    const int g = P->g, N1 = P->N1, N2 = P->N2;
    const double lx = dt / G.dx, ly = dt / G.dy, phi = P->porosity;
    auto bcen = [&](int i, int j) { return 0.5 * (v(i, j, 1) + v(i, j + 1, 1)) / phi; };
    auto acen = [&](int i, int j) { return 0.5 * (v(i, j, 0) + v(i + 1, j, 0)) / phi; };
    auto ty = [&](int i, int j) {  // b dc/dy, upwind difference, at cell (i, j)
        const double b = bcen(i, j);
        return b * (b >= 0 ? c(i, j) - c(i, j - 1) : c(i, j + 1) - c(i, j));
    };
    auto tx = [&](int i, int j) {
        const double a = acen(i, j);
        return a * (a >= 0 ? c(i, j) - c(i - 1, j) : c(i + 1, j) - c(i, j));
    };
    auto Fx = [&](int i, int j) {  // x-face i (between cells i-1 and i)
        const double vel = v(i, j, 0), a = vel / phi;
        double st;
        if (a >= 0) {
            const int m = i - 1;
            st = c(m, j) + 0.5 * (1.0 - a * lx) * (0.5 * (c(m + 1, j) - c(m - 1, j))) - 0.5 * ly * ty(m, j);
        } else {
            const int m = i;
            st = c(m, j) - 0.5 * (1.0 + a * lx) * (0.5 * (c(m + 1, j) - c(m - 1, j))) - 0.5 * ly * ty(m, j);
        }
        return flux(P, vel, st);
    };
    auto Fy = [&](int i, int j) {  // y-face j (between cells j-1 and j)
        const double vel = v(i, j, 1), b = vel / phi;
        double st;
        if (b >= 0) {
            const int m = j - 1;
            st = c(i, m) + 0.5 * (1.0 - b * ly) * (0.5 * (c(i, m + 1) - c(i, m - 1))) - 0.5 * lx * tx(i, m);
        } else {
            const int m = j;
            st = c(i, m) - 0.5 * (1.0 + b * ly) * (0.5 * (c(i, m + 1) - c(i, m - 1))) - 0.5 * lx * tx(i, m);
        }
        return flux(P, vel, st);
    };
    std::vector<double> out((size_t)N1 * N2);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N1; i++)
        for (int j = 0; j < N2; j++)
            out[(size_t)i * N2 + j] = c(i, j) + lx * (Fx(i, j) - Fx(i + 1, j)) + ly * (Fy(i, j) - Fy(i, j + 1));
    for (int i = 0; i < N1; i++)
        for (int j = 0; j < N2; j++) c(i, j) = out[(size_t)i * N2 + j];
    (void)g;
}

// AdvectSplit (src/HyperbolicSplitSolver.cpp:51-106); hyper_method "ctu" advects unsplit.
void or_advect_split(const or_params* P, double* c, const double* v, double dt, int* prev_first_sweep) {
    fill_boundaries(P, c);
    if (P->hmtype == OR_CTU) {
        or_ctu_advect(P, c, v, dt);
        fill_boundaries(P, c);
        return;
    }
    const size_t n = (size_t)(P->N1 + 2 * P->g) * (P->N2 + 2 * P->g);
    switch (P->dim_splitting) {
        case OR_ALTERNATING:
            if (*prev_first_sweep == 1) {
                or_advect_x(P, c, v, dt);
                or_advect_y(P, c, v, dt);
                *prev_first_sweep = 0;
            } else {
                or_advect_y(P, c, v, dt);
                or_advect_x(P, c, v, dt);
                *prev_first_sweep = 1;
            }
            break;
        case OR_X_FIRST:
            or_advect_x(P, c, v, dt);
            or_advect_y(P, c, v, dt);
            *prev_first_sweep = 0;
            break;
        case OR_Y_FIRST:
            or_advect_y(P, c, v, dt);
            or_advect_x(P, c, v, dt);
            *prev_first_sweep = 1;
            break;
        case OR_STRANG:
            or_advect_x(P, c, v, 0.5 * dt);
            or_advect_y(P, c, v, dt);
            or_advect_x(P, c, v, 0.5 * dt);
            *prev_first_sweep = 0;
            break;
        default: {  // SYMMETRIC_PARALLEL
            std::vector<double> ct(c, c + n);
            or_advect_x(P, c, v, dt);
            or_advect_y(P, c, v, dt);
            or_advect_y(P, ct.data(), v, dt);
            or_advect_x(P, ct.data(), v, dt);
            for (size_t k = 0; k < n; ++k) c[k] = 0.5 * (c[k] + ct[k]);
            *prev_first_sweep = 0;
        }
    }
}

// SetupDiffusionTensorF (src/MGSolver.cpp:846-881), + optional molecular diffusion phi*Dm
void or_peaceman_F(const or_params* P, const double* vflat, int i, int j, double* d11, double* d12) {
    Geo G(P);
    V3 v = vview(P, vflat);
    double u = v(i, j, 0);
    double vv = 1. / 4 * (v(i - 1, j + 1, 1) + v(i, j + 1, 1) + v(i - 1, j, 1) + v(i, j, 1));
    double u2 = u * u, v2 = vv * vv;
    double phi = P->porosity;
    double maxdx = std::max(G.dx, G.dy);
    double al = P->alpha_l * maxdx, at = P->alpha_t * maxdx;
    double fac_l = phi * al / (sqrt(u2 + v2));
    double fac_t = phi * at / (sqrt(u2 + v2));
    if (P->peaceman_guard && u2 + v2 == 0) fac_l = fac_t = 0;
    double d11_l = fac_l * u2, d12_l = fac_l * (u * vv);
    double d11_t = fac_t * v2, d12_t = fac_t * (-u * vv);
    *d11 = d11_l + d11_t;
    *d12 = d12_l + d12_t;
    if (P->Dm != 0) *d11 += phi * P->Dm;
}

// SetupDiffusionTensorG (src/MGSolver.cpp:886-919)
void or_peaceman_G(const or_params* P, const double* vflat, int i, int j, double* d22, double* d21) {
    Geo G(P);
    V3 v = vview(P, vflat);
    double uu = 1. / 4 * (v(i + 1, j - 1, 0) + v(i + 1, j, 0) + v(i, j - 1, 0) + v(i, j, 0));
    double vv = v(i, j, 1);
    double u2 = uu * uu, v2 = vv * vv;
    double phi = P->porosity;
    double maxdx = std::max(G.dx, G.dy);
    double al = P->alpha_l * maxdx, at = P->alpha_t * maxdx;
    double fac_l = phi * al / (sqrt(u2 + v2));
    double fac_t = phi * at / (sqrt(u2 + v2));
    if (P->peaceman_guard && u2 + v2 == 0) fac_l = fac_t = 0;
    double d21_l = fac_l * (uu * vv), d22_l = fac_l * v2;
    double d21_t = fac_t * (-uu * vv), d22_t = fac_t * u2;
    *d21 = d21_l + d21_t;
    *d22 = d22_l + d22_t;
    if (P->Dm != 0) *d22 += phi * P->Dm;
}

}  // extern "C"

namespace {
struct Faces {  // Peaceman tensor at the four faces of cell (i,j)
    double d11_im, d12_im, d22_jm, d21_jm, d22_jp, d21_jp, d11_ip, d12_ip;
};
inline Faces faces_at(const or_params* P, const double* v, int i, int j) {
    Faces f;
    or_peaceman_F(P, v, i, j, &f.d11_im, &f.d12_im);
    or_peaceman_G(P, v, i, j, &f.d22_jm, &f.d21_jm);
    or_peaceman_G(P, v, i, j + 1, &f.d22_jp, &f.d21_jp);
    or_peaceman_F(P, v, i + 1, j, &f.d11_ip, &f.d12_ip);
    return f;
}
}  // namespace

extern "C" {

// SetMatrixCoefficients_Parabolic + GetCoefficients_Parabolic (src/MGSolver.cpp:923-948, 997-1321)
void or_cn_matrix(const or_params* P, const double* v, double dt, double* A9) {
    Geo G(P);
    const double dx = G.dx, dy = G.dy;
    const int N1 = P->N1, N2 = P->N2;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < N1; ++k)
        for (int l = 0; l < N2; ++l) {
            Faces f = faces_at(P, v, k, l);
            double s[9];
            double NW = dt / (8. * dx * dy) * (f.d12_im + f.d21_jp);
            double NE = -dt / (8. * dx * dy) * (f.d12_ip + f.d21_jp);
            double N = -dt / 8. * (4. / (dy * dy) * f.d22_jp + 1. / (dx * dy) * (-f.d12_im + f.d12_ip));
            double SW = -dt / (8. * dx * dy) * (f.d12_im + f.d21_jm);
            double SE = dt / (8. * dx * dy) * (f.d12_ip + f.d21_jm);
            double S = -dt / 8. * (4. / (dy * dy) * f.d22_jm + 1. / (dx * dy) * (-f.d12_ip + f.d12_im));
            double W = -dt / 8. * (4. / (dx * dx) * f.d11_im + 1. / (dx * dy) * (-f.d21_jp + f.d21_jm));
            double C = 1. + dt / (2. * dx * dx) * (f.d11_ip + f.d11_im) + dt / (2. * dy * dy) * (f.d22_jp + f.d22_jm);
            double E = -dt / 8. * (4. / (dx * dx) * f.d11_ip + 1. / (dx * dy) * (-f.d21_jm + f.d21_jp));
            s[0] = C; s[1] = W; s[2] = SW; s[3] = S; s[4] = SE; s[5] = E; s[6] = NE; s[7] = N; s[8] = NW;
            fold_row(k, l, N1, N2, s, A9 + ((size_t)k * N2 + l) * 9);
        }
    if (P->stype == OR_HORIZONTAL) {  // para_dir cells (N1-2, j): src/MGSolver.cpp:1295-1317
        for (int j = 0; j < N2; ++j) {
            double* row = A9 + ((size_t)(N1 - 2) * N2 + j) * 9;
            row[0] = 1. / G.dA;
            for (int e = 1; e < 9; ++e) row[e] = 0;
        }
    }
}

// SetRHS_Parabolic (src/MGSolver.cpp:1324-1371)
void or_cn_rhs(const or_params* P, const double* cflat, const double* v, double dt, double* b) {
    Geo G(P);
    S2 c = sview(P, cflat);
    const double dx = G.dx, dy = G.dy;
    const int N1 = P->N1, N2 = P->N2;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N1; i++)
        for (int j = 0; j < N2; j++) {
            Faces f = faces_at(P, v, i, j);
            b[(size_t)i * N2 + j] =
                c(i, j) + dt / 8. * (4. / (dx * dx) * (f.d11_ip * (c(i + 1, j) - c(i, j)) - f.d11_im * (c(i, j) - c(i - 1, j))) +
                                     1. / (dx * dy) * (f.d12_ip * (c(i, j + 1) + c(i + 1, j + 1) - c(i, j - 1) - c(i + 1, j - 1)) -
                                                       f.d12_im * (c(i, j + 1) + c(i - 1, j + 1) - c(i - 1, j - 1) - c(i, j - 1))) +
                                     1. / (dx * dy) * (f.d21_jp * (c(i + 1, j) + c(i + 1, j + 1) - c(i - 1, j + 1) - c(i - 1, j)) -
                                                       f.d21_jm * (c(i + 1, j) + c(i + 1, j - 1) - c(i - 1, j) - c(i - 1, j - 1))) +
                                     4. / (dy * dy) * (f.d22_jp * (c(i, j + 1) - c(i, j)) - f.d22_jm * (c(i, j) - c(i, j - 1))));
        }
    if (P->stype == OR_HORIZONTAL)
        for (int j = 0; j < N2; ++j) b[(size_t)(N1 - 2) * N2 + j] = 0;
}

// ---------------------------------------------------------------- diagnostics
double or_total_mass(const or_params* P, const double* cflat) {  // GetTotalMass :608-620
    S2 c = sview(P, cflat);
    double s = 0;
    for (int i = 0; i < P->N1; i++)
        for (int j = 0; j < P->N2; j++) s += c(i, j);
    return s;
}

double or_mass_error(const or_params* P, const double* c, double t, double outflux) {  // :530-540
    Geo G(P);
    double mass = or_total_mass(P, c);
    double ncpv = 1. / (G.dx * G.dy);
    double influx = (t - P->tstart) * P->I * ncpv;
    if (P->stype == OR_PARALLEL) influx *= 2.;
    return fabs((mass + outflux - influx) / influx);
}

double or_divergence_error(const or_params* P, const double* vflat, const double* q) {  // :542-557
    Geo G(P);
    V3 v = vview(P, vflat);
    double err = 0;
    for (int i = 0; i < P->N1; i++)
        for (int j = 0; j < P->N2; j++) {
            double div = (v(i, j + 1, 1) - v(i, j, 1)) / G.dy + (v(i + 1, j, 0) - v(i, j, 0)) / G.dx;
            err += fabs(div - q[(size_t)i * P->N2 + j]);
        }
    return err * G.dx * G.dx;
}

double or_velocity_boundary_error(const or_params* P, const double* vflat) {  // :562-588
    V3 v = vview(P, vflat);
    double e = 0;
    for (int i = 0; i < P->N1; i++) {
        e += fabs((double)v(i, 0, 1));
        e += fabs((double)v(i, P->N2, 1));
    }
    for (int j = 0; j < P->N2; j++) {
        e += fabs((double)v(0, j, 0));
        e += fabs((double)v(P->N1, j, 0));
    }
    return e;
}

// ---------------------------------------------------------------- wells and profiles
// ExactVolFracCircle (src/Util.cpp:444-487)
double or_exact_vol_frac_circle(double x1, double y1, double r, double dx, double dy) {
    if (x1 * x1 + y1 * y1 < r * r) {
        double y2 = y1 + dy;
        double x2 = x1 + dx;
        if (x2 * x2 + y2 * y2 > r * r) {
            double xs = sqrt(r * r - y1 * y1);
            double ys = sqrt(r * r - x1 * x1);
            double area = 0;
            double xub, xlb, yub;
            if (ys <= y2 && xs <= x2) {
                xlb = x1; xub = xs; yub = ys;
            } else if (ys < y2 && xs > x2) {
                yub = ys; xlb = x1; xub = x2;
            } else if (ys > y2 && xs < x2) {
                yub = y2; xlb = sqrt(r * r - yub * yub); xub = xs;
                area += (xlb - x1) * dy;
            } else {
                yub = y2; xlb = sqrt(r * r - yub * yub); xub = x2;
                area += dy * (xlb - x1);
            }
            (void)yub;
            double t1 = asin(xlb / r);
            double t2 = asin(xub / r);
            area += r * r / 2 * (sin(2 * t2) / 2. + t2 - sin(2 * t1) / 2. - t1);
            area -= y1 * (xub - xlb);
            return area / (dx * dy);
        }
        return 1.;
    }
    return 0;
}

// InitializeSource (src/Impec2DSolver.cpp:241-280) and Util.cpp well initialisers :508-639
void or_init_source(const or_params* P, double* q, double t) {
    Geo G(P);
    const int N1 = P->N1, N2 = P->N2, M = N1 * N2;
    const double dx = G.dx, dy = G.dy;
    double r = P->well_rc * (P->x_ub - P->x_lb);
    double circval = P->I * 4. / (M_PI * r * r);
    double qval = P->I / (dx * dy);
    for (int k = 0; k < M; ++k) q[k] = 0;
    if (P->stype == OR_HORIZONTAL) {  // InitHorizontalFront :607-639
        int w = (int)lround(P->well_width * (P->x_ub - P->x_lb) / dx);
        if (w < 1) return;
        double val = P->I / (N2 * dx * dy * w);
        if (P->inj_mode == OR_PULSING) {
            double tau = 1. / P->q_freq;
            double x = fmod(t, tau);
            if (x > tau / 2.) val *= P->q_high_multiple;
        } else if (P->inj_mode == OR_LINEAR) {
            double vl = val, vh = val * P->q_high_multiple;
            val = vl + (t - P->tstart) * (vh - vl) / (P->tfinal - P->tstart);
        }
        for (int i = 0; i < N2 * w; i++) {
            q[i] = val;
            q[M - 1 - i] = -val;
        }
        return;
    }
    if (P->well_profile == OR_ONECELL) {
        if (P->stype == OR_PARALLEL) {  // InitOneCellParallel :565-573
            q[0] = qval;
            q[M - 1] = qval;
            q[N2 - 1] = -qval;
            q[(N1 - 1) * N2] = -qval;
        } else {  // InitOneCellDiagonal :580-586
            q[0] = qval;
            q[M - 1] = -qval;
        }
        return;
    }
    if (P->well_profile == OR_CIRCULAR) {  // InitQuarterCircle* :508-559
        std::vector<double> I((size_t)M);
        for (int i = 0; i < N1; ++i)
            for (int j = 0; j < N2; ++j)
                I[(size_t)i * N2 + j] = circval * or_exact_vol_frac_circle(P->x_lb + i * dx, P->y_lb + j * dy, r, dx, dy);
        auto at = [&](int i, int j) { return I[(size_t)i * N2 + j]; };
        for (int i = 0; i < N1; ++i)
            for (int j = 0; j < N2; ++j) {
                if (P->stype == OR_DIAGONAL)
                    q[(size_t)i * N2 + j] = at(i, j) - at(N1 - 1 - i, N2 - 1 - j);
                else
                    q[(size_t)i * N2 + j] = at(i, j) + at(N1 - 1 - i, N2 - 1 - j) - at(i, N2 - 1 - j) - at(N1 - 1 - i, j);
            }
    }
    // GAUSSIAN: the reference leaves q untouched (:253-254, :265-266); q stays zero here.
}

// Advection test profiles (src/Util.cpp:55-114)
double or_profile(const or_params* P, int profile, double x, double y) {
    Geo G(P);
    const double dx = G.dx, dy = G.dy;
    switch (profile) {
        case 0:
            return 1. + 1. / (dx * dy * 4. * M_PI * M_PI) * (cos(2. * M_PI * (x + dx / 2.)) - cos(2. * M_PI * (x - dx / 2.))) *
                            (cos(2. * M_PI * (y + dy / 2.)) - cos(2. * M_PI * (y - dy / 2.)));
        case 1: {
            double width = 0.3 * (P->x_ub - P->x_lb), height = 0.3 * (P->y_ub - P->y_lb);
            double xc = (P->x_ub - P->x_lb) / 2., yc = (P->y_ub - P->y_lb) / 2.;
            return (fabs(x - xc) <= width / 2. && fabs(y - yc) <= height / 2.) ? 1. : 0.;
        }
        case 2: {
            double xc = (P->x_ub - P->x_lb) / 2., yc = (P->y_ub - P->y_lb) / 2.;
            double intx = 1. / 16 * sqrt(M_PI) * (-erf(8. * xc - 4. * dx - 8. * x) + erf(8. * xc + 4. * dx - 8. * x));
            double inty = 1. / 16 * sqrt(M_PI) * (-erf(8. * yc - 4. * dy - 8. * y) + erf(8. * yc + 4. * dy - 8. * y));
            return 1. / (dx * dy) * intx * inty;
        }
        case 3:
            return 1. + 1. / (dy) * (-1. / (2. * M_PI)) * (cos(2 * M_PI * (y + dy / 2.)) - cos(2 * M_PI * (y - dy / 2.)));
        case 4: {
            double xc = (P->x_ub - P->x_lb) / 2., yc = (P->y_ub - P->y_lb) / 2.;
            return 1. + 0.2 * sin(4. * M_PI * ((x - xc) + (y - yc)));
        }
    }
    return 0;
}

// CalcAdvectionL1Norm / CalcAdvectionL2Norm (src/Util.cpp:119-147); norm 1 or 2
double or_advection_norm(const or_params* P, const double* cflat, int profile, int norm) {
    Geo G(P);
    S2 c = sview(P, cflat);
    double s = 0;
    for (int i = 0; i < P->N1; i++)
        for (int j = 0; j < P->N2; j++) {
            double x = P->x_lb + (i + 0.5) * G.dx, y = P->y_lb + (j + 0.5) * G.dy;
            double ex = or_profile(P, profile, x, y);
            if (norm == 2)
                s += (ex - c(i, j)) * (ex - c(i, j));
            else
                s += fabs((double)(ex - c(i, j)));
        }
    if (norm == 2) return sqrt(G.dx * G.dy * s);
    return s * G.dx * G.dy;
}

// ParallelProjector::FillDiagonal + GetFromParallel (src/ParallelProjector.cpp:95-199), with
// the projector set up as in Impec2DSolver::Project (src/Impec2DSolver.cpp:690-716): angle
// -pi/4, parallel resolution N1 x N2, diagonal spacing L / (sqrt 2 dN).
void or_project_diagonal(const or_params* P, const double* f, int dN1, int dN2, double* out) {
    const int g = P->g, N2g = P->N2 + 2 * g;
    auto at = [&](int i, int j) { return f[(size_t)(i + g) * N2g + (j + g)]; };
    const double angle = -M_PI / 4.;
    const double pN1 = P->N1, pN2 = P->N2;
    const double p_dx = (P->x_ub - P->x_lb) / pN1, p_dy = (P->y_ub - P->y_lb) / pN2;
    const double d_dx = (P->x_ub - P->x_lb) / (sqrt(2.) * dN1), d_dy = (P->y_ub - P->y_lb) / (sqrt(2.) * dN2);
    auto centred = [](double lb, double dx, int idx) { return lb + (idx + 0.5) * dx; };
    for (int i = 0; i < dN1; ++i)
        for (int j = 0; j < dN2; ++j) {
            const double xd = centred(P->x_lb, d_dx, i), yd = centred(P->y_lb, d_dy, j);
            const double x = cos(angle) * xd - sin(angle) * yd;
            double y = sin(angle) * xd + cos(angle) * yd;
            y = fabs(y);
            const int x00 = (int)floor(x / (P->x_ub - P->x_lb) * pN1);
            const int y00 = (int)floor(y / (P->y_ub - P->y_lb) * pN2);
            const int x11 = x00 + 1, y11 = y00 + 1;
            const double x_00 = centred(P->x_lb, p_dx, x00), x_11 = centred(P->x_lb, p_dx, x11);
            const double y_00 = centred(P->y_lb, p_dy, y00), y_11 = centred(P->y_lb, p_dy, y11);
            out[(size_t)i * dN2 + j] = 1. / ((x_11 - x_00) * (y_11 - y_00)) * (x_11 - x) * (y_11 - y) * at(x00, y00) +
                                       1. / ((x_11 - x_00) * (y_11 - y_00)) * (x - x_00) * (y_11 - y) * at(x11, y00) +
                                       1. / ((x_11 - x_00) * (y_11 - y_00)) * (x_11 - x) * (y - y_00) * at(x00, y11) +
                                       1. / ((x_11 - x_00) * (y_11 - y_00)) * (x - x_00) * (y - y_00) * at(x11, y11);
        }
}

}  // extern "C"
