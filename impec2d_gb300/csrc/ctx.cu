// Context management, parameters, and shared reductions of the C ABI.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "internal.cuh"
#include "reduce.cuh"

namespace impec {

static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }

Geo make_geo(const impec_params& P) {
    // src/EllipticSolver.cpp:59-100 and :126
    Geo G;
    G.dx = (P.x_ub - P.x_lb) / P.N1;
    G.dy = (P.y_ub - P.y_lb) / P.N2;
    G.dA = G.dx * G.dy;
    double alpha = atan(G.dx / G.dy), theta = atan(G.dy / G.dx);
    G.dxi = G.dx / cos(theta);
    G.deta = G.dy / cos(alpha);
    double secamt = 1. / cos(alpha - theta);
    G.secamt2 = secamt * secamt;
    G.cosa2 = cos(alpha) * cos(alpha);
    G.sina2 = sin(alpha) * sin(alpha);
    G.costsina = cos(theta) * sin(alpha);
    G.cosasint = cos(alpha) * sin(theta);
    G.cost2 = cos(theta) * cos(theta);
    G.sint2 = sin(theta) * sin(theta);
    G.cosa = cos(alpha);
    G.sint = sin(theta);
    G.cost = cos(theta);
    G.sina = sin(alpha);
    G.mob1over4 = pow(P.mu_res / P.mu_inj, 0.25);
    return G;
}

// Off by default: measured on GB300, the multigrid solve at 1024^2 is about 7 % slower with
// programmatic launches than with plain stream order.
bool pdl_enabled() {
    static const bool on = [] {
        const char* e = getenv("IMPEC_PDL");
        return e && e[0] == '1';
    }();
    return on;
}

// ---------------------------------------------------------------- FP64 throughput probe
// Eight independent fused multiply-add chains per thread (values stay bounded: |a| < 1); the
// result is stored only under a condition that never holds, which keeps the chains live.
__global__ void __launch_bounds__(256) k_fp64_fma(int iters, double a, double* out) {
    double v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = threadIdx.x * 1e-3 + k;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = fma(v[k], a, 1e-9);
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += v[k];
    if (s == -1.0) out[0] = s;
}

// ---------------------------------------------------------------- reductions
__global__ void __launch_bounds__(RED_THREADS) k_sum(const double* __restrict__ x, size_t n, double* partials,
                                                     int mb, unsigned* counter, double* out) {
    pdl_enter();
    double v[1] = {0.0};
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        v[0] += x[k];
    grid_reduce<1>(v, 0u, partials, mb, counter, out);
}

impec_status reduce_launch_sum(impec_ctx* ctx, const double* x, size_t n, double* out_dev) {
    const int blocks = flat_blocks(n, red_cap(ctx->num_sms, ctx->max_blocks));
    ++ctx->nlaunch, launch_k(ctx->stream, k_sum, blocks, RED_THREADS, 0, x, n, ctx->partials, ctx->max_blocks, ctx->counter, out_dev);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

impec_status sync_scalars(impec_ctx* ctx) {
    IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->hscal, ctx->dscal, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

}  // namespace impec

using namespace impec;

namespace impec {
bool buffers_movable(const impec_ctx* ctx, const char* what) {
    if (ctx->ensembles == 0) return true;
    set_error(std::string(what) + ": the context belongs to a live ensemble whose graph holds its buffers "
                                  "(destroy the ensemble first)");
    return false;
}
}  // namespace impec

extern "C" {

const char* impec_last_error(void) { return g_err.c_str(); }

void impec_default_params(impec_params* P, int N1, int N2) {
    std::memset(P, 0, sizeof(*P));
    P->N1 = N1;
    P->N2 = N2;
    P->x_lb = 0.0; P->x_ub = 1.0; P->y_lb = 0.0; P->y_ub = 1.0;
    P->mu_res = 41.0; P->mu_inj = 1.0;
    P->avgproc = IMPEC_HARMONIC;
    P->nu = 1.0;
    P->porosity = 1.0; P->cfl = 0.5; P->inj_fluid_conc = 1.0; P->I = 1.0;
    P->diffusion = 0; P->alpha_l = 1.0; P->alpha_t = 1.0; P->Dm = 0.0;
    P->ptype = IMPEC_CRANKNICOLSON; P->dt_diff_limit = 0.9;
    P->dim_splitting = IMPEC_SYMMETRIC_PARALLEL;
    P->hmtype = IMPEC_MUSCL;
    P->stype = IMPEC_DIAGONAL;
    P->is_test = 0; P->testno = 1;
    P->bc = IMPEC_BC_NEUMANN;
    P->eps = 1e-10; P->para_eps = 1e-14;
    P->peaceman_guard = 1;
    P->cfl_porosity = 0;
    P->precision = IMPEC_PREC_FP64;
    P->max_cycles = 100;
    P->warm_start = 0;
}

static impec_status validate(const impec_params* P) {
    if (P->N1 < 2 || P->N2 < 2) { set_error("N1 and N2 must be >= 2"); return IMPEC_ERR_ARG; }
    if ((long long)P->N1 * P->N2 > (1ll << 31)) { set_error("grid too large"); return IMPEC_ERR_ARG; }
    if (!(P->x_ub > P->x_lb) || !(P->y_ub > P->y_lb)) { set_error("empty domain"); return IMPEC_ERR_ARG; }
    if (!(P->nu >= 0.0 && P->nu <= 1.0)) { set_error("nu must lie in [0,1] (EllipticSolver::SetNu)"); return IMPEC_ERR_ARG; }
    if (!(P->porosity > 0)) { set_error("porosity must be > 0"); return IMPEC_ERR_ARG; }
    if (!(P->mu_res > 0) || !(P->mu_inj > 0)) { set_error("viscosities must be > 0"); return IMPEC_ERR_ARG; }
    if (P->hmtype < IMPEC_UPWINDSPLIT || P->hmtype > IMPEC_MUSCL) {
        set_error("unknown hyper_method (src/SimParams.h:15)");
        return IMPEC_ERR_ARG;
    }
    if (P->dim_splitting < 0 || P->dim_splitting > 4) { set_error("unknown dimensional_splitting"); return IMPEC_ERR_ARG; }
    if (P->stype == IMPEC_HORIZONTAL && (P->N1 < 4 || P->bc != IMPEC_BC_NEUMANN)) {
        set_error("source_type horizontal needs N1 >= 4 and Neumann boundaries");
        return IMPEC_ERR_ARG;
    }
    if (P->precision != IMPEC_PREC_FP64 && P->precision != IMPEC_PREC_MIXED) { set_error("unknown precision"); return IMPEC_ERR_ARG; }
    return IMPEC_OK;
}

impec_status impec_ctx_create(const impec_params* P, void* stream, impec_ctx** out) {
    IMPEC_RANGE("impec_ctx_create");
    if (!P || !out) { set_error("null argument"); return IMPEC_ERR_ARG; }
    *out = nullptr;
    IMPEC_TRY(validate(P));
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return IMPEC_ERR_NO_DEVICE;
    }
    impec_ctx* ctx = new impec_ctx();
    ctx->P = *P;
    if (ctx->P.max_cycles <= 0) ctx->P.max_cycles = 100;
    ctx->G = make_geo(*P);
    ctx->stream = (cudaStream_t)stream;
    cudaGetDevice(&ctx->device);
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const size_t n = (size_t)P->N1 * P->N2;
    const size_t nu = (size_t)(P->N1 + 1) * P->N2, nv = (size_t)P->N1 * (P->N2 + 1);
    auto fail = [&](impec_status s) { impec_ctx_destroy(ctx); return s; };
#define ALLOC(ptr, bytes)                                                          \
    do {                                                                           \
        cudaError_t e_ = cudaMalloc((void**)&(ptr), (bytes));                      \
        if (e_ != cudaSuccess) {                                                   \
            set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e_));       \
            return fail(IMPEC_ERR_CUDA);                                           \
        }                                                                          \
    } while (0)
    ALLOC(ctx->c, n * 8); ALLOC(ctx->p, n * 8); ALLOC(ctx->q, n * 8);
    ALLOC(ctx->u, nu * 8); ALLOC(ctx->v, nv * 8);
    ALLOC(ctx->t1, n * 8); ALLOC(ctx->t2, n * 8); ALLOC(ctx->t3, n * 8);
    ALLOC(ctx->muK11, n * 8);
    ALLOC(ctx->lamx, nu * 8); ALLOC(ctx->lamy, nv * 8);
    ALLOC(ctx->f, n * 8); ALLOC(ctx->r, n * 8);
    ALLOC(ctx->dfx, nu * 2 * 8); ALLOC(ctx->dfy, nv * 2 * 8);
    ALLOC(ctx->cn_a9, n * 9 * 8); ALLOC(ctx->cn_b, n * 8); ALLOC(ctx->cn_idiag, n * 8);
    ctx->max_blocks = 4096;
    ALLOC(ctx->partials, (size_t)8 * ctx->max_blocks * 8);
    ALLOC(ctx->counter, sizeof(unsigned) * 16);
    ALLOC(ctx->dscal, sizeof(DevScalars));
#undef ALLOC
    if (cudaMallocHost((void**)&ctx->hscal, sizeof(DevScalars)) != cudaSuccess) {
        set_error("cudaMallocHost failed");
        return fail(IMPEC_ERR_CUDA);
    }
    cudaMemsetAsync(ctx->counter, 0, sizeof(unsigned) * 16, ctx->stream);
    cudaMemsetAsync(ctx->dscal, 0, sizeof(DevScalars), ctx->stream);
    cudaMemsetAsync(ctx->c, 0, n * 8, ctx->stream);
    cudaMemsetAsync(ctx->p, 0, n * 8, ctx->stream);
    cudaMemsetAsync(ctx->q, 0, n * 8, ctx->stream);
    cudaMemsetAsync(ctx->u, 0, nu * 8, ctx->stream);
    cudaMemsetAsync(ctx->v, 0, nv * 8, ctx->stream);
    ctx->pin_i = 1;
    ctx->pin_j = 1;
    if (P->stype == IMPEC_HORIZONTAL) {
        ctx->dir_row = 1;
        ctx->cn_dir_row = P->N1 - 2;
        ctx->singular = 0;
    }
    impec_status s = pressure_alloc(ctx);
    if (s != IMPEC_OK) return fail(s);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        set_error("context initialisation failed");
        return fail(IMPEC_ERR_CUDA);
    }
    *out = ctx;
    return IMPEC_OK;
}

impec_status impec_ctx_destroy(impec_ctx* ctx) {
    if (!ctx) return IMPEC_OK;
    if (!buffers_movable(ctx, "impec_ctx_destroy")) return IMPEC_ERR_ARG;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream); else cudaDeviceSynchronize();
    invalidate_step_graph(ctx);
    learned_release(ctx);
    if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
    if (ctx->body_stream) cudaStreamDestroy(ctx->body_stream);
    pressure_free(ctx);
    double* bufs[] = {ctx->c, ctx->p, ctx->q, ctx->u, ctx->v, ctx->t1, ctx->t2, ctx->t3, ctx->muK11,
                      ctx->muK22 == ctx->muK11 ? nullptr : ctx->muK22, ctx->lamx, ctx->lamy, ctx->f, ctx->r,
                      ctx->dfx, ctx->dfy, ctx->cn_a9, ctx->cn_b, ctx->cn_idiag, ctx->partials, ctx->K11,
                      ctx->K22, ctx->well_q};
    for (double* b : bufs)
        if (b) cudaFree(b);
    if (ctx->counter) cudaFree(ctx->counter);
    if (ctx->dscal) cudaFree(ctx->dscal);
    if (ctx->well_idx) cudaFree(ctx->well_idx);
    if (ctx->hscal) cudaFreeHost(ctx->hscal);
    delete ctx;
    return IMPEC_OK;
}

impec_status impec_ctx_params(const impec_ctx* ctx, impec_params* P) {
    if (!ctx || !P) return IMPEC_ERR_ARG;
    *P = ctx->P;
    return IMPEC_OK;
}

impec_status impec_set_permeability(impec_ctx* ctx, const double* K11, const double* K22) {
    if (!ctx) return IMPEC_ERR_ARG;
    const size_t n = (size_t)ctx->P.N1 * ctx->P.N2;
    const bool aniso = K22 && K22 != K11, was_aniso = ctx->K22 && ctx->K22 != ctx->K11;
    if (K11 && ctx->K11 && aniso == was_aniso) {  // same layout: new values in place (graphs stay valid)
        IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->K11, K11, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
        if (aniso) IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->K22, K22, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
        IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        return IMPEC_OK;
    }
    if (!buffers_movable(ctx, "impec_set_permeability")) return IMPEC_ERR_ARG;
    invalidate_step_graph(ctx);
    if (ctx->K22 && ctx->K22 != ctx->K11) cudaFree(ctx->K22);
    if (ctx->K11) cudaFree(ctx->K11);
    ctx->K11 = ctx->K22 = nullptr;
    if (ctx->muK22 && ctx->muK22 != ctx->muK11) cudaFree(ctx->muK22);
    ctx->muK22 = nullptr;
    if (K11) {
        IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->K11, n * 8));
        IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->K11, K11, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    if (K22 && K22 != K11) {
        IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->K22, n * 8));
        IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->K22, K22, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->muK22, n * 8));
    }
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

impec_status impec_set_source(impec_ctx* ctx, const double* q_dev) {
    if (!ctx || !q_dev) return IMPEC_ERR_ARG;
    const size_t n = (size_t)ctx->P.N1 * ctx->P.N2;
    if (q_dev != ctx->q) IMPEC_CUDA_TRY(cudaMemcpyAsync(ctx->q, q_dev, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    std::vector<double> hq(n);
    IMPEC_CUDA_TRY(cudaMemcpyAsync(hq.data(), ctx->q, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    std::vector<int> idx;
    std::vector<double> val;
    for (size_t k = 0; k < n; ++k)
        if (hq[k] != 0.0) {
            if (!std::isfinite(hq[k])) { set_error("non-finite source term"); return IMPEC_ERR_NAN; }
            idx.push_back((int)k);
            val.push_back(hq[k]);
        }
    if (ctx->have_source && idx == ctx->well_idx_host) {
        // same wells, new rates (e.g. the pulsing or linear horizontal front, src/Impec2DSolver.cpp:437-439):
        // the step graph reads q and the rates from device memory, so it stays valid
        if (ctx->nwells)
            IMPEC_CUDA_TRY(cudaMemcpy(ctx->well_q, val.data(), val.size() * 8, cudaMemcpyHostToDevice));
        return IMPEC_OK;
    }
    if (!buffers_movable(ctx, "impec_set_source (new well cells)")) return IMPEC_ERR_ARG;
    invalidate_step_graph(ctx);
    ctx->well_idx_host = idx;
    if (ctx->well_idx) cudaFree(ctx->well_idx);
    if (ctx->well_q) cudaFree(ctx->well_q);
    ctx->well_idx = nullptr;
    ctx->well_q = nullptr;
    ctx->nwells = (int)idx.size();
    if (ctx->nwells) {
        IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->well_idx, idx.size() * sizeof(int)));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&ctx->well_q, val.size() * 8));
        IMPEC_CUDA_TRY(cudaMemcpy(ctx->well_idx, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice));
        IMPEC_CUDA_TRY(cudaMemcpy(ctx->well_q, val.data(), val.size() * 8, cudaMemcpyHostToDevice));
    }
    ctx->have_source = true;
    return IMPEC_OK;
}

impec_status impec_state(impec_ctx* ctx, double** c, double** p, double** u, double** v, double** q) {
    if (!ctx) return IMPEC_ERR_ARG;
    if (c) *c = ctx->c;
    if (p) *p = ctx->p;
    if (u) *u = ctx->u;
    if (v) *v = ctx->v;
    if (q) *q = ctx->q;
    return IMPEC_OK;
}

}  // extern "C"

extern "C" impec_status impec_measure_fp64(double* fma_per_second) {
    if (!fma_per_second) return IMPEC_ERR_ARG;
    int dev = 0, sms = 0;
    IMPEC_CUDA_TRY(cudaGetDevice(&dev));
    IMPEC_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* out = nullptr;
    IMPEC_CUDA_TRY(cudaMalloc((void**)&out, sizeof(double)));
    cudaEvent_t e0, e1;
    IMPEC_CUDA_TRY(cudaEventCreate(&e0));
    IMPEC_CUDA_TRY(cudaEventCreate(&e1));
    const int blocks = sms * 8, threads = 256, iters = 8192;
    k_fp64_fma<<<blocks, threads>>>(iters / 8, 0.999999, out);  // warm-up
    IMPEC_CUDA_TRY(cudaEventRecord(e0));
    k_fp64_fma<<<blocks, threads>>>(iters, 0.999999, out);
    IMPEC_CUDA_TRY(cudaEventRecord(e1));
    IMPEC_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    IMPEC_CUDA_TRY(cudaGetLastError());
    *fma_per_second = (double)blocks * threads * iters * 8 / (ms * 1e-3);
    return IMPEC_OK;
}
