// IMPES step orchestration, diagnostics, host-layout transfers and the per-operation C ABI.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.cuh"
#include "reduce.cuh"

namespace impec {

#define IX(i, j, n2) ((size_t)(i) * (n2) + (j))

static impec_status set_dt(impec_ctx* ctx, double dt) {
    IMPEC_CUDA_TRY(cudaMemcpyAsync(&ctx->dscal->dt, &dt, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    return IMPEC_OK;
}

static impec_status cn_solve_host(impec_ctx* ctx, double* c, double tol) {
    IMPEC_TRY(cn_prepare(ctx, c, 0.5, &ctx->dscal->dt, false));
    IMPEC_TRY(cn_iteration(ctx, c));  // the first sweep before the first check, as in the step graph
    IMPEC_TRY(cn_check(ctx, tol, 1, 0, 0));
    for (;;) {
        IMPEC_TRY(sync_scalars(ctx));
        if (!ctx->hscal->go) break;
        IMPEC_TRY(cn_iteration(ctx, c));
        IMPEC_TRY(cn_check(ctx, tol, 1, 0, 0));
    }
    if (ctx->hscal->flags & FLAG_CN_NAN) return IMPEC_ERR_NAN;
    if (ctx->hscal->flags & FLAG_CN_NOT_CONVERGED) return IMPEC_ERR_NOT_CONVERGED;
    return IMPEC_OK;
}

// HyperbolicSplitSolver::Solve with SPLIT2ND (src/HyperbolicSplitSolver.cpp:162-198), host
// driven.  Both Crank-Nicolson half steps share v and dt/2, hence one matrix per call.
impec_status hyperbolic_solve_dev(impec_ctx* ctx, double* c, const double* u, const double* v, const double* dt_dev,
                                  int* pfs) {
    const impec_params& P = ctx->P;
    IMPEC_CUDA_TRY(cudaMemsetAsync(&ctx->dscal->flags, 0, sizeof(int), ctx->stream));
    IMPEC_TRY(tr_integrate_dev(ctx, c, 0.5, dt_dev, 0));
    if (P.diffusion) {
        IMPEC_TRY(cn_setup(ctx, u, v, 0.5, dt_dev));
        IMPEC_TRY(cn_solve_host(ctx, c, P.para_eps));
    }
    IMPEC_TRY(advect_split_dev(ctx, c, u, v, dt_dev, pfs));
    IMPEC_TRY(tr_integrate_dev(ctx, c, 0.5, dt_dev, 1));
    if (P.diffusion) IMPEC_TRY(cn_solve_host(ctx, c, P.para_eps));
    return IMPEC_OK;
}

// GetTotalMass, CalculateDivergenceError, CalculateVelocityBoundaryError, max/min c
// (src/Impec2DSolver.cpp:430-431, 542-620).
__global__ void __launch_bounds__(RED_THREADS) k_diag(int n1, int n2, const double* __restrict__ c,
                                                      const double* __restrict__ u, const double* __restrict__ v,
                                                      const double* __restrict__ q, double inv_dx, double inv_dy,
                                                      double* partials, int mb, unsigned* counter, double* out) {
    pdl_enter();
    double acc[5] = {0.0, 0.0, 0.0, -INFINITY, -INFINITY};
    for_cells(n1, n2, [&](int i, int j, size_t k) {
        double cc = c[k];
        acc[0] += cc;
        double div = (v[IX(i, j + 1, n2 + 1)] - v[IX(i, j, n2 + 1)]) * inv_dy + (u[IX(i + 1, j, n2)] - u[IX(i, j, n2)]) * inv_dx;
        acc[1] += fabs(div - (q ? q[k] : 0.0));
        double be = 0;
        if (j == 0) be += fabs(v[IX(i, 0, n2 + 1)]);
        if (j == n2 - 1) be += fabs(v[IX(i, n2, n2 + 1)]);
        if (i == 0) be += fabs(u[IX(0, j, n2)]);
        if (i == n1 - 1) be += fabs(u[IX(n1, j, n2)]);
        acc[2] += be;
        acc[3] = fmax(acc[3], cc);
        acc[4] = fmax(acc[4], -cc);
    });
    grid_reduce<5>(acc, (1u << 3) | (1u << 4), partials, mb, counter, out);
}

static impec_status diagnostics_dev(impec_ctx* ctx, const double* c, const double* u, const double* v) {
    const impec_params& P = ctx->P;
    ++ctx->nlaunch, launch_k(ctx->stream, k_diag, seg_blocks(P.N1, P.N2, red_cap(ctx->num_sms, ctx->max_blocks)), RED_THREADS, 0, P.N1, P.N2, c, u, v, ctx->have_source ? ctx->q : nullptr,
                                                              1.0 / ctx->G.dx, 1.0 / ctx->G.dy, ctx->partials,
                                                              ctx->max_blocks, ctx->counter, ctx->dscal->red);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

// CalculateMassError (src/Impec2DSolver.cpp:530-540)
static double mass_error(const impec_ctx* ctx, double mass, double t) {
    double influx = (t - ctx->t0) * ctx->P.I * (1. / (ctx->G.dx * ctx->G.dy));
    if (ctx->P.stype == IMPEC_PARALLEL) influx *= 2.;
    return fabs((mass + ctx->total_outflux - influx) / influx);
}

// One resident IMPES step through the step graph; with info, waits and reports.
static impec_status one_step(impec_ctx* ctx, double t_clip, impec_step_info* info) {
    ctx->host_flags = 0;
    IMPEC_TRY(launch_step_graph(ctx, t_clip));
    ctx->counter_steps++;
    if (!info) return IMPEC_OK;
    IMPEC_TRY(sync_scalars(ctx));
    const DevScalars& H = *ctx->hscal;
    ctx->t = H.t;
    ctx->total_outflux = H.total_outflux;
    ctx->last_its = H.mg_cycles;
    ctx->last_relres = H.relres;
    ctx->last_para_its = H.cn_cycles_total;
    info->t = H.t;
    info->dt = H.dt;
    info->total_outflux = H.total_outflux;
    info->relres = H.relres;
    info->counter = ctx->counter_steps;
    info->its = H.mg_cycles;
    info->para_its = H.cn_cycles_total;
    info->prev_first_sweep = ctx->prev_first_sweep;
    info->clipped = H.clipped;
    const int flags = H.flags | ctx->host_flags;
    ctx->host_flags = 0;
    IMPEC_TRY(diagnostics_dev(ctx, ctx->c, ctx->u, ctx->v));
    IMPEC_TRY(sync_scalars(ctx));
    info->mass_err = mass_error(ctx, ctx->hscal->red[0], ctx->t);
    if (flags & (FLAG_MG_NAN | FLAG_CN_NAN)) { set_error("NaN in a residual"); return IMPEC_ERR_NAN; }
    if (flags & (FLAG_MG_NOT_CONVERGED | FLAG_CN_NOT_CONVERGED)) {
        set_error(flags & FLAG_MG_NOT_CONVERGED ? "pressure multigrid hit max_cycles" : "Crank-Nicolson hit max_cycles");
        return IMPEC_ERR_NOT_CONVERGED;
    }
    return IMPEC_OK;
}

}  // namespace impec

using namespace impec;

extern "C" {

impec_status impec_pressure_solve(impec_ctx* ctx, const double* c, double* p, double tol, int* cycles, double* relres) {
    IMPEC_RANGE("impec_pressure_solve");
    if (!ctx || !c || !p) return IMPEC_ERR_ARG;
    impec_status s = pressure_solve(ctx, c, p, tol, cycles, relres);
    if (s == IMPEC_OK) IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return s;
}

impec_status impec_face_mobility(impec_ctx* ctx, const double* c, double* lamx, double* lamy) {
    if (!ctx || !c) return IMPEC_ERR_ARG;
    IMPEC_TRY(face_mobility(ctx, c));
    const size_t nu = (size_t)(ctx->P.N1 + 1) * ctx->P.N2, nv = (size_t)ctx->P.N1 * (ctx->P.N2 + 1);
    if (lamx) IMPEC_CUDA_TRY(cudaMemcpyAsync(lamx, ctx->lamx, nu * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    if (lamy) IMPEC_CUDA_TRY(cudaMemcpyAsync(lamy, ctx->lamy, nv * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

impec_status impec_pressure_apply(impec_ctx* ctx, const double* c, const double* x, double* y) {
    if (!ctx || !c || !x || !y) return IMPEC_ERR_ARG;
    ctx->eliminate = 0;  // the reference's matrix, Dirichlet rows included, not the reduced system
    impec_status s = pressure_setup(ctx, c);
    ctx->eliminate = 1;
    IMPEC_TRY(s);
    IMPEC_TRY(pressure_apply_ref(ctx, x, y));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

impec_status impec_velocity(impec_ctx* ctx, const double* p, const double* c, double* u, double* v) {
    IMPEC_RANGE("impec_velocity");
    if (!ctx || !p || !c || !u || !v) return IMPEC_ERR_ARG;
    IMPEC_TRY(face_mobility(ctx, c));
    IMPEC_TRY(velocity(ctx, p, c, u, v));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

impec_status impec_max_stable_dt(impec_ctx* ctx, const double* u, const double* v, double* dt) {
    if (!ctx || !u || !v || !dt) return IMPEC_ERR_ARG;
    IMPEC_TRY(max_stable_dt_dev(ctx, u, v));
    IMPEC_TRY(sync_scalars(ctx));
    *dt = ctx->hscal->dt;
    return IMPEC_OK;
}

impec_status impec_tr_integrate(impec_ctx* ctx, double* c, double dt, double* tmo) {
    if (!ctx || !c) return IMPEC_ERR_ARG;
    IMPEC_TRY(set_dt(ctx, dt));
    IMPEC_CUDA_TRY(cudaMemsetAsync(&ctx->dscal->tmo_pre, 0, sizeof(double), ctx->stream));
    IMPEC_TRY(tr_integrate_dev(ctx, c, 1.0, &ctx->dscal->dt, 0));
    IMPEC_TRY(sync_scalars(ctx));
    if (tmo) *tmo = ctx->hscal->tmo_pre;
    return IMPEC_OK;
}

impec_status impec_advect_x(impec_ctx* ctx, double* c, const double* u, double dt) {
    if (!ctx || !c || !u) return IMPEC_ERR_ARG;
    IMPEC_TRY(set_dt(ctx, dt));
    IMPEC_TRY(advect_x_dev(ctx, c, ctx->t1, u, 1.0, &ctx->dscal->dt));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(c, ctx->t1, (size_t)ctx->P.N1 * ctx->P.N2 * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

impec_status impec_advect_y(impec_ctx* ctx, double* c, const double* v, double dt) {
    if (!ctx || !c || !v) return IMPEC_ERR_ARG;
    IMPEC_TRY(set_dt(ctx, dt));
    IMPEC_TRY(advect_y_dev(ctx, c, ctx->t1, v, 1.0, &ctx->dscal->dt));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(c, ctx->t1, (size_t)ctx->P.N1 * ctx->P.N2 * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

impec_status impec_advect_split(impec_ctx* ctx, double* c, const double* u, const double* v, double dt, int* pfs) {
    IMPEC_RANGE("impec_advect_split");
    if (!ctx || !c || !u || !v || !pfs) return IMPEC_ERR_ARG;
    IMPEC_TRY(set_dt(ctx, dt));
    IMPEC_TRY(advect_split_dev(ctx, c, u, v, &ctx->dscal->dt, pfs));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

impec_status impec_dispersion_cn(impec_ctx* ctx, double* c, const double* u, const double* v, double dt, double tol,
                                 int* its, double* relres) {
    IMPEC_RANGE("impec_dispersion_cn");
    if (!ctx || !c || !u || !v) return IMPEC_ERR_ARG;
    IMPEC_TRY(set_dt(ctx, dt));
    impec_status s = dispersion_cn_dev(ctx, c, u, v, 1.0, &ctx->dscal->dt, tol, its, relres);
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return s;
}

impec_status impec_hyperbolic_solve(impec_ctx* ctx, double* c, const double* u, const double* v, double dt, int* pfs,
                                    double* outflux) {
    IMPEC_RANGE("impec_hyperbolic_solve");
    if (!ctx || !c || !u || !v || !pfs) return IMPEC_ERR_ARG;
    IMPEC_TRY(set_dt(ctx, dt));
    double z = outflux ? *outflux : 0.0;
    IMPEC_CUDA_TRY(cudaMemcpyAsync(&ctx->dscal->total_outflux, &z, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_TRY(hyperbolic_solve_dev(ctx, c, u, v, &ctx->dscal->dt, pfs));
    IMPEC_TRY(sync_scalars(ctx));
    if (outflux) *outflux = ctx->hscal->total_outflux;
    return IMPEC_OK;
}

impec_status impec_diagnostics(impec_ctx* ctx, const double* c, const double* u, const double* v, double out[5]) {
    if (!ctx || !c || !u || !v || !out) return IMPEC_ERR_ARG;
    IMPEC_TRY(diagnostics_dev(ctx, c, u, v));
    IMPEC_TRY(sync_scalars(ctx));
    const double* r = ctx->hscal->red;
    out[0] = r[0];
    out[1] = r[1] * ctx->G.dx * ctx->G.dx;
    out[2] = r[2];
    out[3] = r[3];
    out[4] = -r[4];
    return IMPEC_OK;
}

impec_status impec_step(impec_ctx* ctx, double t_clip, impec_step_info* info) {
    IMPEC_RANGE("impec_step");
    if (!ctx) return IMPEC_ERR_ARG;
    impec_step_info tmp;
    return one_step(ctx, t_clip, info ? info : &tmp);
}

impec_status impec_run_steps(impec_ctx* ctx, int n, impec_step_info* info) {
    IMPEC_RANGE("impec_run_steps");
    if (!ctx || n < 0) return IMPEC_ERR_ARG;
    for (int s = 0; s + 1 < n; ++s) IMPEC_TRY(one_step(ctx, -1.0, nullptr));
    if (n > 0 && info) return one_step(ctx, -1.0, info);
    if (n > 0) IMPEC_TRY(one_step(ctx, -1.0, nullptr));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

impec_status impec_set_time(impec_ctx* ctx, double t0) {
    if (!ctx) return IMPEC_ERR_ARG;
    ctx->t = ctx->t0 = t0;
    ctx->total_outflux = 0;
    ctx->counter_steps = 0;
    double z = 0.0;
    IMPEC_CUDA_TRY(cudaMemcpyAsync(&ctx->dscal->total_outflux, &z, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(&ctx->dscal->t, &ctx->t0, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

impec_status impec_set_pin_kappa(impec_ctx* ctx, double kappa) {
    if (!ctx || !(kappa != 0.0) || !std::isfinite(kappa)) return IMPEC_ERR_ARG;
    ctx->pin_kappa = kappa;
    return IMPEC_OK;
}

impec_status impec_velocity_upload(impec_ctx* ctx, const double* v_host, int g) {
    if (!ctx || !v_host || g < 0) return IMPEC_ERR_ARG;
    const int N1 = ctx->P.N1, N2 = ctx->P.N2, wv = N2 + 1 + 2 * g;
    std::vector<double> hu((size_t)(N1 + 1) * N2), hv((size_t)N1 * (N2 + 1));
    for (int i = 0; i <= N1; ++i)
        for (int j = 0; j < N2; ++j) hu[IX(i, j, N2)] = v_host[((size_t)(i + g) * wv + (j + g)) * 2 + 0];
    for (int i = 0; i < N1; ++i)
        for (int j = 0; j <= N2; ++j) hv[IX(i, j, N2 + 1)] = v_host[((size_t)(i + g) * wv + (j + g)) * 2 + 1];
    IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->u, hu.data(), hu.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->v, hv.data(), hv.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

impec_status impec_pressure_upload(impec_ctx* ctx, const double* p_host, int g) {
    if (!ctx || !p_host || g < 0) return IMPEC_ERR_ARG;
    const int N1 = ctx->P.N1, N2 = ctx->P.N2, w = N2 + 2 * g;
    std::vector<double> buf((size_t)N1 * N2);
    for (int i = 0; i < N1; ++i) std::memcpy(&buf[IX(i, 0, N2)], p_host + (size_t)(i + g) * w + g, N2 * 8);
    IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->p, buf.data(), buf.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

impec_status impec_pressure_solve_resident(impec_ctx* ctx, int sync, int* cycles, double* relres) {
    IMPEC_RANGE("impec_pressure_solve_resident");
    if (!ctx) return IMPEC_ERR_ARG;
    IMPEC_TRY(launch_pressure_graph(ctx));
    if (!sync) return IMPEC_OK;
    IMPEC_TRY(sync_scalars(ctx));
    if (cycles) *cycles = ctx->hscal->mg_cycles;
    if (relres) *relres = ctx->hscal->relres;
    if (ctx->hscal->flags & FLAG_MG_NAN) return IMPEC_ERR_NAN;
    if (ctx->hscal->flags & FLAG_MG_NOT_CONVERGED) return IMPEC_ERR_NOT_CONVERGED;
    return IMPEC_OK;
}

// Cycles, final and initial relative residual of the last pressure solve (waits for the
// context's stream).
impec_status impec_last_solve(impec_ctx* ctx, int* cycles, double* relres, double* relres0) {
    if (!ctx) return IMPEC_ERR_ARG;
    IMPEC_TRY(sync_scalars(ctx));
    if (cycles) *cycles = ctx->hscal->mg_cycles;
    if (relres) *relres = ctx->hscal->relres;
    if (relres0) *relres0 = ctx->hscal->relres0;
    return IMPEC_OK;
}

impec_status impec_launch_count(impec_ctx* ctx, long long* n) {
    if (!ctx || !n) return IMPEC_ERR_ARG;
    IMPEC_TRY(sync_scalars(ctx));
    *n = ctx->nlaunch + ctx->hscal->graph_launches;
    return IMPEC_OK;
}

// Reference ghost layouts on the host <-> engine device layout.
impec_status impec_state_upload(impec_ctx* ctx, const double* c_host, const double* q_host, int g) {
    IMPEC_RANGE("impec_state_upload");
    if (!ctx || g < 0) return IMPEC_ERR_ARG;
    const int N1 = ctx->P.N1, N2 = ctx->P.N2, w = N2 + 2 * g;
    if (c_host) {  // interior rows straight from the ghosted host array (one strided copy)
        IMPEC_CUDA_TRY(cudaMemcpy2DAsync(ctx->c, (size_t)N2 * 8, c_host + (size_t)g * w + g, (size_t)w * 8,
                                         (size_t)N2 * 8, N1, cudaMemcpyHostToDevice, ctx->stream));
        IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    }
    if (q_host) {
        IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->q, q_host, (size_t)N1 * N2 * 8, cudaMemcpyHostToDevice, ctx->stream));
        IMPEC_TRY(impec_set_source(ctx, ctx->q));
    }
    return IMPEC_OK;
}

impec_status impec_state_download(impec_ctx* ctx, double* c_host, double* p_host, double* v_host, int g) {
    IMPEC_RANGE("impec_state_download");
    if (!ctx || g < 0) return IMPEC_ERR_ARG;
    const int N1 = ctx->P.N1, N2 = ctx->P.N2, w = N2 + 2 * g;
    auto get = [&](const double* dev, double* host) -> impec_status {  // interior rows, one strided copy
        IMPEC_CUDA_TRY(cudaMemcpy2DAsync(host + (size_t)g * w + g, (size_t)w * 8, dev, (size_t)N2 * 8, (size_t)N2 * 8,
                                         N1, cudaMemcpyDeviceToHost, ctx->stream));
        return IMPEC_OK;
    };
    if (c_host) IMPEC_TRY(get(ctx->c, c_host));
    if (p_host) IMPEC_TRY(get(ctx->p, p_host));
    if (c_host || p_host) IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (v_host) {
        const int wv = N2 + 1 + 2 * g;
        std::vector<double> hu((size_t)(N1 + 1) * N2), hv((size_t)N1 * (N2 + 1));
        IMPEC_CUDA_TRY(cudaMemcpyAsync(hu.data(), ctx->u, hu.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
        IMPEC_CUDA_TRY(cudaMemcpyAsync(hv.data(), ctx->v, hv.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
        IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        for (int i = 0; i <= N1; ++i)
            for (int j = 0; j < N2; ++j) v_host[((size_t)(i + g) * wv + (j + g)) * 2 + 0] = hu[IX(i, j, N2)];
        for (int i = 0; i < N1; ++i)
            for (int j = 0; j <= N2; ++j) v_host[((size_t)(i + g) * wv + (j + g)) * 2 + 1] = hv[IX(i, j, N2 + 1)];
    }
    return IMPEC_OK;
}


// ---------------------------------------------------------------- tuning and autotuner
static long* tuning_field(impec_ctx* ctx, const char* name) {
    Tuning& t = ctx->tune;
    struct { const char* n; long* v; } tab[] = {
        {"mg_pre", &t.pre},          {"mg_post", &t.post},         {"cluster", &t.cluster},
        {"cluster_cells", &t.cl_cells}, {"cluster_cta0", &t.cl_cta0}, {"coarse_cells64", &t.coarse_cells64},
        {"coarse_cells32", &t.coarse_cells32}, {"tile_cells", &t.tile_cells},
        {"tile_cells32", &t.tile_cells32}};
    for (auto& e : tab)
        if (!strcmp(e.n, name)) return e.v;
    return nullptr;
}

impec_status impec_set_tuning(impec_ctx* ctx, const char* name, long value) {
    if (!ctx || !name) return IMPEC_ERR_ARG;
    long* f = tuning_field(ctx, name);
    if (!f) {
        set_error(std::string("unknown tunable ") + name);
        return IMPEC_ERR_ARG;
    }
    if (value < 0 || ((!strcmp(name, "mg_pre") || !strcmp(name, "mg_post")) && value > 8)) {
        set_error(std::string("tunable out of range: ") + name);
        return IMPEC_ERR_ARG;
    }
    if (*f != value) {
        const long old = *f;
        *f = value;
        if (ctx->tune.pre + ctx->tune.post < 1) {
            *f = old;
            set_error("mg_pre + mg_post must be at least 1");
            return IMPEC_ERR_ARG;
        }
        invalidate_step_graph(ctx);  // the captured graphs bake the launch structure in
    }
    return IMPEC_OK;
}

impec_status impec_get_tuning(impec_ctx* ctx, const char* name, long* value) {
    if (!ctx || !name || !value) return IMPEC_ERR_ARG;
    long* f = tuning_field(ctx, name);
    if (!f) {
        set_error(std::string("unknown tunable ") + name);
        return IMPEC_ERR_ARG;
    }
    *value = *f;
    return IMPEC_OK;
}

// Times the resident pressure solve (graph replay, CUDA events on the context stream) on the
// context's current state for each candidate smoother schedule and cluster choice, keeps the
// fastest, and leaves it set.  Every candidate still solves to the context's tolerance.
impec_status impec_autotune(impec_ctx* ctx, int reps, char* report, int report_len) {
    IMPEC_RANGE("impec_autotune");
    if (!ctx || reps < 1) return IMPEC_ERR_ARG;
    struct Cand { long pre, post, cluster; };
    const Cand cands[] = {{2, 2, 1}, {1, 1, 1}, {2, 1, 1}, {1, 2, 1}, {3, 3, 1}, {2, 2, 0}, {1, 1, 0}};
    const Tuning saved = ctx->tune;
    cudaEvent_t e0, e1;
    IMPEC_CUDA_TRY(cudaEventCreate(&e0));
    IMPEC_CUDA_TRY(cudaEventCreate(&e1));
    std::string rep;
    double best = 1e300;
    Cand pick = {saved.pre, saved.post, saved.cluster};
    for (const Cand& c : cands) {
        if (c.cluster && ctx->cl_size < 2) continue;
        IMPEC_TRY(impec_set_tuning(ctx, "mg_pre", c.pre));
        IMPEC_TRY(impec_set_tuning(ctx, "mg_post", c.post));
        IMPEC_TRY(impec_set_tuning(ctx, "cluster", c.cluster));
        int cyc = 0;
        double rr = 0;
        impec_status s = impec_pressure_solve_resident(ctx, 1, &cyc, &rr);  // capture + warm-up
        if (s != IMPEC_OK) continue;
        std::vector<float> ms;
        for (int r = 0; r < reps; ++r) {
            IMPEC_CUDA_TRY(cudaEventRecord(e0, ctx->stream));
            IMPEC_TRY(impec_pressure_solve_resident(ctx, 0, nullptr, nullptr));
            IMPEC_CUDA_TRY(cudaEventRecord(e1, ctx->stream));
            IMPEC_CUDA_TRY(cudaEventSynchronize(e1));
            float t = 0;
            cudaEventElapsedTime(&t, e0, e1);
            ms.push_back(t);
        }
        std::sort(ms.begin(), ms.end());
        const double med = ms[ms.size() / 2];
        char line[160];
        snprintf(line, sizeof line, "pre=%ld post=%ld cluster=%ld: %.4f ms, %d iterations\n", c.pre, c.post,
                 c.cluster, med, cyc);
        rep += line;
        if (med < best) {
            best = med;
            pick = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->tune = saved;
    invalidate_step_graph(ctx);
    IMPEC_TRY(impec_set_tuning(ctx, "mg_pre", pick.pre));
    IMPEC_TRY(impec_set_tuning(ctx, "mg_post", pick.post));
    IMPEC_TRY(impec_set_tuning(ctx, "cluster", pick.cluster));
    if (report && report_len > 0) {
        snprintf(report, (size_t)report_len, "%schosen: pre=%ld post=%ld cluster=%ld\n", rep.c_str(), pick.pre,
                 pick.post, pick.cluster);
    }
    return IMPEC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- checkpoint of the run
// File layout (native byte order): a fixed header, then c and p (N1*N2 doubles each, row-major,
// no ghost cells), u ((N1+1)*N2) and v (N1*(N2+1)).  The header's checksum is FNV-1a (64 bit)
// over the payload bytes.  Everything a later step reads from the run is in it: the fields,
// the clock and start time, the outflux accumulator of the mass balance, the step counter and
// the sweep order of alternating splittings.
struct CheckpointHeader {
    char magic[8];  // "IMPECCK1"
    int32_t version, n1, n2, prev_first_sweep;
    int64_t steps;
    double t, t0, total_outflux;
    uint64_t checksum;
};
static const char kCkptMagic[8] = {'I', 'M', 'P', 'E', 'C', 'C', 'K', '1'};

static uint64_t fnv1a(const void* data, size_t bytes, uint64_t h) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (size_t k = 0; k < bytes; ++k) h = (h ^ p[k]) * 1099511628211ull;
    return h;
}

extern "C" impec_status impec_checkpoint_save(impec_ctx* ctx, const char* path) {
    IMPEC_RANGE("impec_checkpoint_save");
    if (!ctx || !path) return IMPEC_ERR_ARG;
    const int N1 = ctx->P.N1, N2 = ctx->P.N2;
    const size_t nc = (size_t)N1 * N2, nu = (size_t)(N1 + 1) * N2, nv = (size_t)N1 * (N2 + 1);
    std::vector<double> buf(2 * nc + nu + nv);
    IMPEC_TRY(sync_scalars(ctx));  // the clock and outflux as the last step left them
    double* h = buf.data();
    IMPEC_CUDA_TRY(cudaMemcpyAsync(h, ctx->c, nc * 8, cudaMemcpyDeviceToHost, ctx->stream));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(h + nc, ctx->p, nc * 8, cudaMemcpyDeviceToHost, ctx->stream));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(h + 2 * nc, ctx->u, nu * 8, cudaMemcpyDeviceToHost, ctx->stream));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(h + 2 * nc + nu, ctx->v, nv * 8, cudaMemcpyDeviceToHost, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    CheckpointHeader H;
    std::memset(&H, 0, sizeof(H));
    std::memcpy(H.magic, kCkptMagic, 8);
    H.version = 1;
    H.n1 = N1;
    H.n2 = N2;
    H.prev_first_sweep = ctx->prev_first_sweep;
    H.steps = ctx->counter_steps;
    H.t = ctx->hscal->t;
    H.t0 = ctx->t0;
    H.total_outflux = ctx->hscal->total_outflux;
    H.checksum = fnv1a(h, buf.size() * 8, 1469598103934665603ull);
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        set_error(std::string("impec_checkpoint_save: cannot open ") + path);
        return IMPEC_ERR_ARG;
    }
    const bool ok = std::fwrite(&H, sizeof(H), 1, f) == 1 && std::fwrite(h, 8, buf.size(), f) == buf.size();
    if (std::fclose(f) != 0 || !ok) {
        set_error(std::string("impec_checkpoint_save: write failed: ") + path);
        return IMPEC_ERR_ARG;
    }
    return IMPEC_OK;
}

extern "C" impec_status impec_checkpoint_load(impec_ctx* ctx, const char* path) {
    IMPEC_RANGE("impec_checkpoint_load");
    if (!ctx || !path) return IMPEC_ERR_ARG;
    if (ctx->ensembles > 0) {  // an ensemble's graph reads this context's clock from the device
        set_error("impec_checkpoint_load: the context is a member of a live ensemble");
        return IMPEC_ERR_ARG;
    }
    const int N1 = ctx->P.N1, N2 = ctx->P.N2;
    const size_t nc = (size_t)N1 * N2, nu = (size_t)(N1 + 1) * N2, nv = (size_t)N1 * (N2 + 1);
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        set_error(std::string("impec_checkpoint_load: cannot open ") + path);
        return IMPEC_ERR_ARG;
    }
    CheckpointHeader H;
    std::vector<double> buf(2 * nc + nu + nv);
    bool ok = std::fread(&H, sizeof(H), 1, f) == 1 && std::memcmp(H.magic, kCkptMagic, 8) == 0 && H.version == 1 &&
              H.n1 == N1 && H.n2 == N2;
    ok = ok && std::fread(buf.data(), 8, buf.size(), f) == buf.size();
    std::fclose(f);
    if (!ok) {
        set_error(std::string("impec_checkpoint_load: not a checkpoint of a ") + std::to_string(N1) + "x" +
                  std::to_string(N2) + " run: " + path);
        return IMPEC_ERR_ARG;
    }
    if (fnv1a(buf.data(), buf.size() * 8, 1469598103934665603ull) != H.checksum) {
        set_error(std::string("impec_checkpoint_load: checksum mismatch: ") + path);
        return IMPEC_ERR_ARG;
    }
    const double* h = buf.data();
    IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->c, h, nc * 8, cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->p, h + nc, nc * 8, cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->u, h + 2 * nc, nu * 8, cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->v, h + 2 * nc + nu, nv * 8, cudaMemcpyHostToDevice, ctx->stream));
    const double clock[2] = {H.t, H.total_outflux};
    IMPEC_CUDA_TRY(cudaMemcpyAsync(&ctx->dscal->t, &clock[0], 8, cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(&ctx->dscal->total_outflux, &clock[1], 8, cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));  // the host buffers above go out of scope
    ctx->t = H.t;
    ctx->t0 = H.t0;
    ctx->total_outflux = H.total_outflux;
    ctx->counter_steps = (int)H.steps;
    ctx->prev_first_sweep = H.prev_first_sweep;
    return IMPEC_OK;
}
