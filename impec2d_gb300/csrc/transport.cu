// Transport: trapezoidal source integrator and dimensionally split MUSCL / upwind advection.
//
// Ghost cells of the reference (two layers, src/Util.cpp:283-438) are replaced by index
// reflection inside the kernels.  The reference's X sweep also updates the ghost rows
// j < 0, j >= N2 (src/HyperbolicSplitSolver.cpp:128-131); those rows are exact mirror images
// of the updated interior rows (mirrored c and mirrored tangential velocity give the same
// fluxes), so the following Y sweep reads them here by reflecting the interior result.
#include <cmath>

#include "internal.cuh"
#include "reduce.cuh"

namespace impec {

constexpr int TBX = 32, TBY = 8;
#define IX(i, j, n2) ((size_t)(i) * (n2) + (j))

// ---------------------------------------------------------------- TR source integrator
// TRIntegrator::Integrate (src/TRIntegrator.cpp:49-71) over the well list (q != 0 cells):
// producers c <- c (1 + dt q/2) / (1 - dt q/2), injectors c <- c + dt c_inj q.
// slot 0/1 receives total_mass_outflux of this call; S->total_outflux += |tmo|.
__global__ void __launch_bounds__(RED_THREADS) k_tr(int nw, const int* __restrict__ idx, const double* __restrict__ qv,
                                                    double* __restrict__ c, const double* __restrict__ dt_dev,
                                                    double scale, double cinj, DevScalars* S, int slot) {
    const double dt = scale * dt_dev[0];
    double acc[1] = {0.0};
    for (int w = threadIdx.x; w < nw; w += blockDim.x) {
        const int k = idx[w];
        const double qij = qv[w];
        if (qij < 0) {
            double m = c[k];
            double cn = c[k] * (1 + 0.5 * dt * qij) / (1 - 0.5 * dt * qij);
            c[k] = cn;
            acc[0] += cn - m;
        } else if (qij > 0) {
            c[k] += dt * cinj * qij;
        }
    }
    block_reduce<1>(acc, 0u);
    if (threadIdx.x == 0) {
        if (slot == 0) S->tmo_pre = acc[0]; else S->tmo_post = acc[0];
        S->total_outflux += fabs(acc[0]);
    }
}

impec_status tr_integrate_dev(impec_ctx* ctx, double* c, double dt_scale, const double* dt_dev, int slot) {
    if (!ctx->have_source || ctx->nwells == 0) return IMPEC_OK;
    k_tr<<<1, RED_THREADS, 0, ctx->stream>>>(ctx->nwells, ctx->well_idx, ctx->well_q, c, dt_dev, dt_scale,
                                             ctx->P.inj_fluid_conc, ctx->dscal, slot);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

// ---------------------------------------------------------------- MUSCL-Hancock / upwind
// Cell reconstruction and Hancock half step (src/MUSCLSplitSolver.cpp:54-93, :121-129).
// The reference limiter xi(r) = min(2r/(1+r), 2/(1+r)) times (a+b)/2 equals, in exact
// arithmetic, minmod(a, b) (r = a/b <= 1 gives a, r > 1 gives b, a*b <= 0 gives 0); the
// selection below evaluates that value without the three divisions.
// kap = 0.5 dt / (dx phi).  sl: state at the cell's left face, sr: at its right face.
__device__ __forceinline__ void hancock(double cm, double c0, double cp, double ul, double ur, double kap,
                                        double& sl, double& sr) {
    double a = c0 - cm, b = cp - c0;
    double d = (a * b > 0.0) ? (fabs(a) <= fabs(b) ? a : b) : 0.0;
    double UR = fma(0.5, d, c0), UL = fma(-0.5, d, c0);
    double df = kap * (ul * UL - ur * UR);
    sl = UL + df;
    sr = UR + df;
}

template <int BC>
__device__ __forceinline__ int cell_at(int i, int n) { return BC == IMPEC_BC_PERIODIC ? wrap_cell(i, n) : refl_cell(i, n); }

// Normal face velocity along the sweep direction, ghost faces by odd reflection (Neumann)
// or wrap-around (periodic).
template <int BC>
__device__ __forceinline__ double face_at(const double* __restrict__ u, int f, int n, size_t stride_f, size_t off) {
    if (BC == IMPEC_BC_PERIODIC) return u[(size_t)wrap_face(f, n) * stride_f + off];
    double s = 1.0;
    int ff = refl_face(f, n, s);
    return s * u[(size_t)ff * stride_f + off];
}

// One sweep along a line: cells k in [0,n) at positions base + k*cs of c, faces f in [0,n]
// at base_f + f*fs of the face array.  Computes the update of cell k.
// cg (may be null) supplies the cells outside [0,n) instead of the reflection of c.
template <int SCHEME, int BC>
__device__ __forceinline__ double sweep_cell(const double* __restrict__ c, const double* __restrict__ cg,
                                             size_t cbase, size_t cs, const double* __restrict__ u, size_t ubase,
                                             size_t us, int k, int n, double kap, double lam) {
    auto C = [&](int m) {
        const double* src = (cg && (m < 0 || m >= n)) ? cg : c;
        return src[cbase + (size_t)cell_at<BC>(m, n) * cs];
    };
    auto U = [&](int f) { return face_at<BC>(u, f, n, us, ubase); };
    double uw = U(k), ue = U(k + 1);
    double Fw, Fe;
    if (SCHEME == IMPEC_UPWINDSPLIT) {  // src/UpwindSplitSolver.cpp:43-65
        double cm = C(k - 1), c0 = C(k), cp = C(k + 1);
        Fw = uw * (uw > 0 ? cm : c0);
        Fe = ue * (ue > 0 ? c0 : cp);
        return c0 + lam * (Fw - Fe);
    }
    double cmm = C(k - 2), cm = C(k - 1), c0 = C(k), cp = C(k + 1), cpp = C(k + 2);
    double uww = U(k - 1), uee = U(k + 2);
    double slm, srm, sl0, sr0, slp, srp;
    hancock(cmm, cm, c0, uww, uw, kap, slm, srm);
    hancock(cm, c0, cp, uw, ue, kap, sl0, sr0);
    hancock(c0, cp, cpp, ue, uee, kap, slp, srp);
    (void)slm;
    (void)srp;
    Fw = uw * (uw > 0 ? srm : sl0);
    Fe = ue * (ue > 0 ? sr0 : slp);
    return c0 + lam * (Fw - Fe);
}

// X sweep: lines along i (stride N2), faces u (N1+1) x N2.
template <int SCHEME, int BC>
__global__ void k_sweep_x(int n1, int n2, const double* __restrict__ cin, const double* __restrict__ cghost,
                          double* __restrict__ cout, const double* __restrict__ u, const double* __restrict__ dt_dev,
                          double dt_scale, double inv_dx_phi) {
    int j = blockIdx.x * TBX + threadIdx.x, i = blockIdx.y * TBY + threadIdx.y;
    if (i >= n1 || j >= n2) return;
    const double dt = dt_scale * dt_dev[0];
    const double lam = dt * inv_dx_phi, kap = 0.5 * lam;
    cout[IX(i, j, n2)] = sweep_cell<SCHEME, BC>(cin, cghost, j, n2, u, j, n2, i, n1, kap, lam);
}

// Y sweep: lines along j (stride 1), faces v N1 x (N2+1).
template <int SCHEME, int BC>
__global__ void k_sweep_y(int n1, int n2, const double* __restrict__ cin, double* __restrict__ cout,
                          const double* __restrict__ v, const double* __restrict__ dt_dev, double dt_scale,
                          double inv_dy_phi) {
    int j = blockIdx.x * TBX + threadIdx.x, i = blockIdx.y * TBY + threadIdx.y;
    if (i >= n1 || j >= n2) return;
    const double dt = dt_scale * dt_dev[0];
    const double lam = dt * inv_dy_phi, kap = 0.5 * lam;
    cout[IX(i, j, n2)] = sweep_cell<SCHEME, BC>(cin, nullptr, IX(i, 0, n2), 1, v, IX(i, 0, n2 + 1), 1, j, n2, kap, lam);
}

__global__ void k_average(size_t n, double* __restrict__ c, const double* __restrict__ a, const double* __restrict__ b) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        c[k] = 0.5 * (a[k] + b[k]);
}

static dim3 tgrid(int n1, int n2) { return dim3((n2 + TBX - 1) / TBX, (n1 + TBY - 1) / TBY); }

impec_status advect_x_dev(impec_ctx* ctx, const double* cin, double* cout, const double* u, double dt_scale,
                          const double* dt_dev, const double* cghost) {
    const impec_params& P = ctx->P;
    const double f = 1.0 / (ctx->G.dx * P.porosity);
    dim3 g = tgrid(P.N1, P.N2), b(TBX, TBY);
    const bool per = P.bc == IMPEC_BC_PERIODIC;
    if (P.hmtype == IMPEC_MUSCL) {
        if (per) k_sweep_x<IMPEC_MUSCL, IMPEC_BC_PERIODIC><<<g, b, 0, ctx->stream>>>(P.N1, P.N2, cin, cghost, cout, u, dt_dev, dt_scale, f);
        else k_sweep_x<IMPEC_MUSCL, IMPEC_BC_NEUMANN><<<g, b, 0, ctx->stream>>>(P.N1, P.N2, cin, cghost, cout, u, dt_dev, dt_scale, f);
    } else {
        if (per) k_sweep_x<IMPEC_UPWINDSPLIT, IMPEC_BC_PERIODIC><<<g, b, 0, ctx->stream>>>(P.N1, P.N2, cin, cghost, cout, u, dt_dev, dt_scale, f);
        else k_sweep_x<IMPEC_UPWINDSPLIT, IMPEC_BC_NEUMANN><<<g, b, 0, ctx->stream>>>(P.N1, P.N2, cin, cghost, cout, u, dt_dev, dt_scale, f);
    }
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

impec_status advect_y_dev(impec_ctx* ctx, const double* cin, double* cout, const double* v, double dt_scale,
                          const double* dt_dev) {
    const impec_params& P = ctx->P;
    const double f = 1.0 / (ctx->G.dy * P.porosity);
    dim3 g = tgrid(P.N1, P.N2), b(TBX, TBY);
    const bool per = P.bc == IMPEC_BC_PERIODIC;
    if (P.hmtype == IMPEC_MUSCL) {
        if (per) k_sweep_y<IMPEC_MUSCL, IMPEC_BC_PERIODIC><<<g, b, 0, ctx->stream>>>(P.N1, P.N2, cin, cout, v, dt_dev, dt_scale, f);
        else k_sweep_y<IMPEC_MUSCL, IMPEC_BC_NEUMANN><<<g, b, 0, ctx->stream>>>(P.N1, P.N2, cin, cout, v, dt_dev, dt_scale, f);
    } else {
        if (per) k_sweep_y<IMPEC_UPWINDSPLIT, IMPEC_BC_PERIODIC><<<g, b, 0, ctx->stream>>>(P.N1, P.N2, cin, cout, v, dt_dev, dt_scale, f);
        else k_sweep_y<IMPEC_UPWINDSPLIT, IMPEC_BC_NEUMANN><<<g, b, 0, ctx->stream>>>(P.N1, P.N2, cin, cout, v, dt_dev, dt_scale, f);
    }
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

impec_status average_dev(impec_ctx* ctx, double* c, const double* a, const double* b) {
    const size_t n = (size_t)ctx->P.N1 * ctx->P.N2;
    k_average<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(n, c, a, b);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

// AdvectSplit (src/HyperbolicSplitSolver.cpp:51-106); pfs 0 = X_SWEEP, 1 = Y_SWEEP.
impec_status advect_split_dev(impec_ctx* ctx, double* c, const double* u, const double* v, const double* dt_dev,
                              int* pfs) {
    const impec_params& P = ctx->P;
    const size_t bytes = (size_t)P.N1 * P.N2 * 8;
    double *t1 = ctx->t1, *t2 = ctx->t2, *t3 = ctx->t3;
    switch (P.dim_splitting) {
        case IMPEC_ALTERNATING:
            if (*pfs == 1) {
                IMPEC_TRY(advect_x_dev(ctx, c, t1, u, 1.0, dt_dev));
                IMPEC_TRY(advect_y_dev(ctx, t1, c, v, 1.0, dt_dev));
                *pfs = 0;
            } else {
                IMPEC_TRY(advect_y_dev(ctx, c, t1, v, 1.0, dt_dev));
                IMPEC_TRY(advect_x_dev(ctx, t1, c, u, 1.0, dt_dev));
                *pfs = 1;
            }
            break;
        case IMPEC_X_FIRST:
            IMPEC_TRY(advect_x_dev(ctx, c, t1, u, 1.0, dt_dev));
            IMPEC_TRY(advect_y_dev(ctx, t1, c, v, 1.0, dt_dev));
            *pfs = 0;
            break;
        case IMPEC_Y_FIRST:
            IMPEC_TRY(advect_y_dev(ctx, c, t1, v, 1.0, dt_dev));
            IMPEC_TRY(advect_x_dev(ctx, t1, c, u, 1.0, dt_dev));
            *pfs = 1;
            break;
        case IMPEC_STRANG:
            // Advect_X leaves the ghost columns i < 0, i >= N1 untouched, so after X(dt/2), Y(dt)
            // they hold Y(dt) applied to the mirrored input, not mirrors of the new interior; the
            // last X(dt/2) reads them there (src/HyperbolicSplitSolver.cpp:80-85, :128-131, :152-155).
            IMPEC_TRY(advect_y_dev(ctx, c, t3, v, 1.0, dt_dev));
            IMPEC_TRY(advect_x_dev(ctx, c, t1, u, 0.5, dt_dev));
            IMPEC_TRY(advect_y_dev(ctx, t1, t2, v, 1.0, dt_dev));
            IMPEC_TRY(advect_x_dev(ctx, t2, c, u, 0.5, dt_dev, t3));
            *pfs = 0;
            break;
        default:  // SYMMETRIC_PARALLEL: average of XY and YX applied to copies of c
            IMPEC_TRY(advect_x_dev(ctx, c, t1, u, 1.0, dt_dev));
            IMPEC_TRY(advect_y_dev(ctx, t1, t2, v, 1.0, dt_dev));
            IMPEC_TRY(advect_y_dev(ctx, c, t1, v, 1.0, dt_dev));
            IMPEC_TRY(advect_x_dev(ctx, t1, t3, u, 1.0, dt_dev));
            IMPEC_TRY(average_dev(ctx, c, t2, t3));
            *pfs = 0;
    }
    (void)bytes;
    return IMPEC_OK;
}

}  // namespace impec
