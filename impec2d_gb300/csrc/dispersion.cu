// Crank-Nicolson Peaceman dispersion (HyperbolicSolver::DiffusionSplitCN ->
// MGSolver::Solve_Parabolic_cc_to_c, src/MGSolver.cpp:846-1392).
//
// D = phi/|u| (alpha_l u u^T + alpha_t (|u|^2 I - u u^T)) (+ phi Dm I, engine option) at
// x-faces (v from a four-face average) and y-faces (u from a four-face average); alpha is
// the configured value times max(dx,dy).  The nine-point CN matrix (I - dt/2 L) and the
// right-hand side (I + dt/2 L) c are assembled exactly as the reference does (including the
// Neumann folding) and solved by four-colour Gauss-Seidel to the relative residual tol.
#include <cmath>

#include "internal.cuh"
#include "reduce.cuh"

namespace impec {

constexpr int DBX = 32, DBY = 8;
#define IX(i, j, n2) ((size_t)(i) * (n2) + (j))
__constant__ int d_off[9][2] = {{0, 0}, {-1, 0}, {-1, -1}, {0, -1}, {1, -1}, {1, 0}, {1, 1}, {0, 1}, {-1, 1}};

struct PeaceArgs {
    int n1, n2;
    double phi, al, at, phiDm;
    int guard;
};

// SetupDiffusionTensorF (src/MGSolver.cpp:846-881) at x-face (i,j): out (d11, d12)
// SetupDiffusionTensorG (src/MGSolver.cpp:886-919) at y-face (i,j): out (d22, d21)
__global__ void k_peaceman(PeaceArgs A, const double* __restrict__ u, const double* __restrict__ v,
                           double* __restrict__ dfx, double* __restrict__ dfy) {
    int j = blockIdx.x * DBX + threadIdx.x, i = blockIdx.y * DBY + threadIdx.y;
    const int n1 = A.n1, n2 = A.n2;
    if (i <= n1 && j < n2) {
        double uu = u[IX(i, j, n2)];
        // tangential v mirrored (even) across x-boundaries: v(-1,j) = v(0,j), v(N1,j) = v(N1-1,j)
        int im = refl_cell(i - 1, n1), i0 = refl_cell(i, n1);
        double vv = 1. / 4 * (v[IX(im, j + 1, n2 + 1)] + v[IX(i0, j + 1, n2 + 1)] + v[IX(im, j, n2 + 1)] +
                              v[IX(i0, j, n2 + 1)]);
        double u2 = uu * uu, v2 = vv * vv;
        double nrm = sqrt(u2 + v2);
        double fl = A.phi * A.al / nrm, ft = A.phi * A.at / nrm;
        if (A.guard && u2 + v2 == 0) fl = ft = 0;
        double d11 = fl * u2 + ft * v2;
        double d12 = fl * (uu * vv) + ft * (-uu * vv);
        d11 += A.phiDm;
        size_t k = IX(i, j, n2);
        dfx[2 * k] = d11;
        dfx[2 * k + 1] = d12;
    }
    if (i < n1 && j <= n2) {
        int jm = refl_cell(j - 1, n2), j0 = refl_cell(j, n2);
        double uu = 1. / 4 * (u[IX(i + 1, jm, n2)] + u[IX(i + 1, j0, n2)] + u[IX(i, jm, n2)] + u[IX(i, j0, n2)]);
        double vv = v[IX(i, j, n2 + 1)];
        double u2 = uu * uu, v2 = vv * vv;
        double nrm = sqrt(u2 + v2);
        double fl = A.phi * A.al / nrm, ft = A.phi * A.at / nrm;
        if (A.guard && u2 + v2 == 0) fl = ft = 0;
        double d21 = fl * (uu * vv) + ft * (-uu * vv);
        double d22 = fl * v2 + ft * u2;
        d22 += A.phiDm;
        size_t k = IX(i, j, n2 + 1);
        dfy[2 * k] = d22;
        dfy[2 * k + 1] = d21;
    }
}

struct CNArgs {
    int n1, n2;
    double dx, dy;
};

// GetCoefficients_Parabolic (src/MGSolver.cpp:923-948), folding (:1031-1289), and
// SetRHS_Parabolic (:1324-1371).  dt = scale * dt_dev[0].
__global__ void k_cn_assemble(CNArgs A, const double* __restrict__ dfx, const double* __restrict__ dfy,
                              const double* __restrict__ c, const double* __restrict__ dt_dev, double scale,
                              double* __restrict__ a9, double* __restrict__ idiag, double* __restrict__ rhs) {
    int j = blockIdx.x * DBX + threadIdx.x, i = blockIdx.y * DBY + threadIdx.y;
    const int n1 = A.n1, n2 = A.n2;
    if (i >= n1 || j >= n2) return;
    const double dt = scale * dt_dev[0];
    const double dx = A.dx, dy = A.dy;
    size_t kx0 = IX(i, j, n2), kx1 = IX(i + 1, j, n2), ky0 = IX(i, j, n2 + 1), ky1 = IX(i, j + 1, n2 + 1);
    double d11_im = dfx[2 * kx0], d12_im = dfx[2 * kx0 + 1], d11_ip = dfx[2 * kx1], d12_ip = dfx[2 * kx1 + 1];
    double d22_jm = dfy[2 * ky0], d21_jm = dfy[2 * ky0 + 1], d22_jp = dfy[2 * ky1], d21_jp = dfy[2 * ky1 + 1];
    double NW = dt / (8. * dx * dy) * (d12_im + d21_jp);
    double NE = -dt / (8. * dx * dy) * (d12_ip + d21_jp);
    double N = -dt / 8. * (4. / (dy * dy) * d22_jp + 1. / (dx * dy) * (-d12_im + d12_ip));
    double SW = -dt / (8. * dx * dy) * (d12_im + d21_jm);
    double SE = dt / (8. * dx * dy) * (d12_ip + d21_jm);
    double S = -dt / 8. * (4. / (dy * dy) * d22_jm + 1. / (dx * dy) * (-d12_ip + d12_im));
    double W = -dt / 8. * (4. / (dx * dx) * d11_im + 1. / (dx * dy) * (-d21_jp + d21_jm));
    double C = 1. + dt / (2. * dx * dx) * (d11_ip + d11_im) + dt / (2. * dy * dy) * (d22_jp + d22_jm);
    double E = -dt / 8. * (4. / (dx * dx) * d11_ip + 1. / (dx * dy) * (-d21_jm + d21_jp));
    double o[9] = {C, W, SW, S, SE, E, NE, N, NW};
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
    const size_t n = (size_t)n1 * n2, kk = IX(i, j, n2);
    for (int e = 0; e < 9; ++e) a9[e * n + kk] = o[e];
    idiag[kk] = 1.0 / o[0];
    // right-hand side with mirrored ghost values
    auto cc = [&](int a, int b) { return c[IX(refl_cell(a, n1), refl_cell(b, n2), n2)]; };
    rhs[kk] = cc(i, j) + dt / 8. * (4. / (dx * dx) * (d11_ip * (cc(i + 1, j) - cc(i, j)) - d11_im * (cc(i, j) - cc(i - 1, j))) +
                                    1. / (dx * dy) * (d12_ip * (cc(i, j + 1) + cc(i + 1, j + 1) - cc(i, j - 1) - cc(i + 1, j - 1)) -
                                                      d12_im * (cc(i, j + 1) + cc(i - 1, j + 1) - cc(i - 1, j - 1) - cc(i, j - 1))) +
                                    1. / (dx * dy) * (d21_jp * (cc(i + 1, j) + cc(i + 1, j + 1) - cc(i - 1, j + 1) - cc(i - 1, j)) -
                                                      d21_jm * (cc(i + 1, j) + cc(i + 1, j - 1) - cc(i - 1, j) - cc(i - 1, j - 1))) +
                                    4. / (dy * dy) * (d22_jp * (cc(i, j + 1) - cc(i, j)) - d22_jm * (cc(i, j) - cc(i, j - 1))));
}

__device__ __forceinline__ double cn_off(int i, int j, int n1, int n2, const double* __restrict__ a9,
                                         const double* __restrict__ x) {
    const size_t n = (size_t)n1 * n2, k = IX(i, j, n2);
    double s = 0;
#pragma unroll
    for (int e = 1; e < 9; ++e) {
        int ii = i + d_off[e][0], jj = j + d_off[e][1];
        if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
        s += a9[e * n + k] * x[IX(ii, jj, n2)];
    }
    return s;
}

__global__ void k_cn_gs(int n1, int n2, const double* __restrict__ a9, const double* __restrict__ idiag,
                        const double* __restrict__ b, double* __restrict__ x, int ci, int cj) {
    int j = 2 * (blockIdx.x * DBX + threadIdx.x) + cj, i = 2 * (blockIdx.y * DBY + threadIdx.y) + ci;
    if (i >= n1 || j >= n2) return;
    x[IX(i, j, n2)] = (b[IX(i, j, n2)] - cn_off(i, j, n1, n2, a9, x)) * idiag[IX(i, j, n2)];
}

// ||b - A x||^2 and ||b||^2
__global__ void __launch_bounds__(RED_THREADS) k_cn_resid(int n1, int n2, const double* __restrict__ a9,
                                                          const double* __restrict__ b, const double* __restrict__ x,
                                                          double* partials, int mb, unsigned* counter, double* out) {
    double acc[2] = {0.0, 0.0};
    const size_t n = (size_t)n1 * n2;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(k / n2), j = (int)(k % n2);
        double r = b[k] - (a9[k] * x[k] + cn_off(i, j, n1, n2, a9, x));
        acc[0] += r * r;
        acc[1] += b[k] * b[k];
    }
    grid_reduce<2>(acc, 0u, partials, mb, counter, out);
}

impec_status dispersion_cn_dev(impec_ctx* ctx, double* c, const double* u, const double* v, double dt_scale,
                               const double* dt_dev, double tol, int* its, double* relres) {
    const impec_params& P = ctx->P;
    const int n1 = P.N1, n2 = P.N2;
    const Geo& G = ctx->G;
    const double maxdx = G.dx > G.dy ? G.dx : G.dy;
    PeaceArgs pa{n1, n2, P.porosity, P.alpha_l * maxdx, P.alpha_t * maxdx, P.porosity * P.Dm, P.peaceman_guard};
    dim3 b(DBX, DBY);
    k_peaceman<<<dim3((n2 + 1 + DBX - 1) / DBX, (n1 + 1 + DBY - 1) / DBY), b, 0, ctx->stream>>>(pa, u, v, ctx->dfx,
                                                                                                 ctx->dfy);
    IMPEC_LAUNCH_CHECK();
    CNArgs ca{n1, n2, G.dx, G.dy};
    k_cn_assemble<<<dim3((n2 + DBX - 1) / DBX, (n1 + DBY - 1) / DBY), b, 0, ctx->stream>>>(
        ca, ctx->dfx, ctx->dfy, c, dt_dev, dt_scale, ctx->cn_a9, ctx->cn_idiag, ctx->cn_b);
    IMPEC_LAUNCH_CHECK();
    // x starts from c (the reference starts from 0; only the iteration count differs)
    const int rb = ctx->num_sms * 2;
    dim3 g4(((n2 + 1) / 2 + DBX - 1) / DBX, ((n1 + 1) / 2 + DBY - 1) / DBY);
    int k = 0;
    double rr = 0;
    impec_status st = IMPEC_OK;
    for (;;) {
        k_cn_resid<<<rb, RED_THREADS, 0, ctx->stream>>>(n1, n2, ctx->cn_a9, ctx->cn_b, c, ctx->partials,
                                                         ctx->max_blocks, ctx->counter, ctx->dscal->red + 2);
        IMPEC_LAUNCH_CHECK();
        IMPEC_TRY(sync_scalars(ctx));
        double bn = ctx->hscal->red[3];
        rr = bn > 0 ? sqrt(ctx->hscal->red[2] / bn) : sqrt(ctx->hscal->red[2]);
        if (!std::isfinite(rr)) { st = IMPEC_ERR_NAN; break; }
        if (rr <= tol) break;
        if (k >= P.max_cycles) { st = IMPEC_ERR_NOT_CONVERGED; break; }
        for (int col = 0; col < 4; ++col)
            k_cn_gs<<<g4, b, 0, ctx->stream>>>(n1, n2, ctx->cn_a9, ctx->cn_idiag, ctx->cn_b, c, col >> 1, col & 1);
        IMPEC_LAUNCH_CHECK();
        ++k;
    }
    if (its) *its = k;
    if (relres) *relres = rr;
    ctx->last_para_its = k;
    return st;
}

}  // namespace impec
