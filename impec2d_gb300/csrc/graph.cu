// The resident IMPES step as one CUDA graph.
//
// One pass of the loop body of Impec2DSolver::Solve (src/Impec2DSolver.cpp:339-415) is
// captured once per context: pressure operator + multigrid, Darcy velocities, the CFL step and
// output-time clipping, and HyperbolicSplitSolver::Solve.  The two iterative parts (multigrid
// cycles to eps, Crank-Nicolson Gauss-Seidel sweeps to para_eps) are WHILE conditional nodes
// whose condition is set on the device by the convergence-check kernel, so a step needs no
// host round trip and steps can be queued back to back.
#include <cmath>

#include "internal.cuh"
#include "reduce.cuh"

namespace impec {

__global__ void k_step_begin(DevScalars* S) {
    pdl_enter();
    S->flags = 0;
    S->cn_cycles_total = 0;
    S->clipped = 0;
}

// Output-time matching (src/Impec2DSolver.cpp:375-378) on the device.
__global__ void k_clip_dt(DevScalars* S) {
    pdl_enter();
    if (S->t_clip >= 0 && S->t + S->dt >= S->t_clip) {
        S->dt = S->t_clip - S->t;
        S->clipped = 1;
    }
}

// Advances the clock and counts the kernels this replay executed: the fixed nodes plus the
// loop bodies times their trip counts.
__global__ void k_advance(DevScalars* S, long long outer, long long mg_body, long long cn_body) {
    pdl_enter();
    S->t += S->dt;
    S->steps++;
    S->graph_launches += outer + mg_body * S->mg_cycles + cn_body * S->cn_cycles_total;
}

// Adds a WHILE node at the current position of the capture on ctx->cap_stream.  init(h)
// launches (captured) the kernel that sets the condition before the first pass; body(h) is
// captured into the node's body graph on ctx->body_stream.
template <class Init, class Body>
static impec_status capture_while(impec_ctx* ctx, Init init, Body body, long long& body_launches) {
    cudaStreamCaptureStatus st;
    unsigned long long id;
    cudaGraph_t g;
    const cudaGraphNode_t* deps;
    const cudaGraphEdgeData* ed;
    size_t nd;
    IMPEC_CUDA_TRY(cudaStreamGetCaptureInfo(ctx->cap_stream, &st, &id, &g, &deps, &ed, &nd));
    cudaGraphConditionalHandle h;
    IMPEC_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
    IMPEC_TRY(init(h));
    IMPEC_CUDA_TRY(cudaStreamGetCaptureInfo(ctx->cap_stream, &st, &id, &g, &deps, &ed, &nd));
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    IMPEC_CUDA_TRY(cudaGraphAddNode(&node, g, deps, ed, nd, &np));
    cudaGraph_t bodyg = np.conditional.phGraph_out[0];
    IMPEC_CUDA_TRY(cudaStreamUpdateCaptureDependencies(ctx->cap_stream, &node, nullptr, 1,
                                                       cudaStreamSetCaptureDependencies));
    cudaStream_t outer = ctx->stream;
    ctx->stream = ctx->body_stream;
    cudaError_t e = cudaStreamBeginCaptureToGraph(ctx->body_stream, bodyg, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
        ctx->stream = outer;
        IMPEC_CUDA_TRY(e);
    }
    const long long n0 = ctx->nlaunch;
    impec_status s = body(h);
    body_launches = ctx->nlaunch - n0;
    cudaGraph_t tmp = nullptr;
    e = cudaStreamEndCapture(ctx->body_stream, &tmp);
    ctx->stream = outer;
    IMPEC_TRY(s);
    IMPEC_CUDA_TRY(e);
    return IMPEC_OK;
}

static impec_status capture_cn_solve(impec_ctx* ctx, double* c) {
    const double tol = ctx->P.para_eps;
    IMPEC_TRY(cn_prepare(ctx, c, 0.5, &ctx->dscal->dt));
    long long nb = 0;
    IMPEC_TRY(capture_while(
        ctx, [&](cudaGraphConditionalHandle h) { return cn_check(ctx, tol, 0, h, 1); },
        [&](cudaGraphConditionalHandle h) {
            IMPEC_TRY(cn_iteration(ctx, c));
            return cn_check(ctx, tol, 1, h, 1);
        },
        nb));
    ctx->step_cn_body_launches = nb;
    return IMPEC_OK;
}

// Captures the step for the given alternating-sweep parity (0: X first, 1: Y first).
static impec_status capture_step(impec_ctx* ctx, int pfs_in, cudaGraph_t* out) {
    const impec_params& P = ctx->P;
    DevScalars* S = ctx->dscal;
    const double* dt = &S->dt;
    IMPEC_CUDA_TRY(cudaStreamBeginCapture(ctx->cap_stream, cudaStreamCaptureModeRelaxed));
    cudaStream_t saved = ctx->stream;
    ctx->stream = ctx->cap_stream;
    const long long n0 = ctx->nlaunch;
    long long mg_body = 0;
    auto body = [&]() -> impec_status {
        ++ctx->nlaunch;
        launch_k(ctx->stream, k_step_begin, 1, 1, 0, S);
        IMPEC_TRY(pressure_prepare(ctx, ctx->c, ctx->p));
        IMPEC_TRY(capture_while(
            ctx, [&](cudaGraphConditionalHandle h) { return pressure_check(ctx, P.eps, 0, h, 1); },
            [&](cudaGraphConditionalHandle h) {
                IMPEC_TRY(pressure_iteration(ctx));
                return pressure_check(ctx, P.eps, 1, h, 1);
            },
            mg_body));
        IMPEC_TRY(pressure_finish(ctx, ctx->p));
        IMPEC_TRY(velocity(ctx, ctx->p, ctx->c, ctx->u, ctx->v));
        IMPEC_TRY(max_stable_dt_dev(ctx, ctx->u, ctx->v));
        ++ctx->nlaunch;
        launch_k(ctx->stream, k_clip_dt, 1, 1, 0, S);
        // HyperbolicSplitSolver::Solve (src/HyperbolicSplitSolver.cpp:162-198)
        IMPEC_TRY(tr_integrate_dev(ctx, ctx->c, 0.5, dt, 0));
        if (P.diffusion) {
            IMPEC_TRY(cn_setup(ctx, ctx->u, ctx->v, 0.5, dt));
            IMPEC_TRY(capture_cn_solve(ctx, ctx->c));
        }
        int pfs = pfs_in;
        IMPEC_TRY(advect_split_dev(ctx, ctx->c, ctx->u, ctx->v, dt, &pfs));
        IMPEC_TRY(tr_integrate_dev(ctx, ctx->c, 0.5, dt, 1));
        if (P.diffusion) IMPEC_TRY(capture_cn_solve(ctx, ctx->c));
        ++ctx->nlaunch;
        const long long loops = mg_body + (P.diffusion ? 2 * ctx->step_cn_body_launches : 0);
        launch_k(ctx->stream, k_advance, 1, 1, 0, S, ctx->nlaunch - n0 - loops, mg_body,
                                            P.diffusion ? ctx->step_cn_body_launches : 0);
        IMPEC_LAUNCH_CHECK();
        return IMPEC_OK;
    };
    impec_status s = body();
    ctx->stream = saved;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->cap_stream, &g);
    IMPEC_TRY(s);
    IMPEC_CUDA_TRY(e);
    const long long loops = mg_body + (P.diffusion ? 2 * ctx->step_cn_body_launches : 0);
    ctx->step_outer_launches = ctx->nlaunch - n0 - loops;
    ctx->step_mg_body_launches = mg_body;
    ctx->nlaunch = n0;  // captured launches run (and are counted) on the device at each replay
    *out = g;
    return IMPEC_OK;
}

// Pressure solve on the resident state (c -> p) as one graph.
static impec_status capture_pressure(impec_ctx* ctx, cudaGraph_t* out) {
    const impec_params& P = ctx->P;
    IMPEC_CUDA_TRY(cudaStreamBeginCapture(ctx->cap_stream, cudaStreamCaptureModeRelaxed));
    cudaStream_t saved = ctx->stream;
    ctx->stream = ctx->cap_stream;
    const long long n0 = ctx->nlaunch;
    long long mg_body = 0;
    auto body = [&]() -> impec_status {
        IMPEC_CUDA_TRY(cudaMemsetAsync(&ctx->dscal->flags, 0, sizeof(int), ctx->stream));
        IMPEC_TRY(pressure_prepare(ctx, ctx->c, ctx->p));
        IMPEC_TRY(capture_while(
            ctx, [&](cudaGraphConditionalHandle h) { return pressure_check(ctx, P.eps, 0, h, 1); },
            [&](cudaGraphConditionalHandle h) {
                IMPEC_TRY(pressure_iteration(ctx));
                return pressure_check(ctx, P.eps, 1, h, 1);
            },
            mg_body));
        return pressure_finish(ctx, ctx->p);
    };
    impec_status s = body();
    ctx->stream = saved;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->cap_stream, &g);
    IMPEC_TRY(s);
    IMPEC_CUDA_TRY(e);
    ctx->pressure_outer_launches = ctx->nlaunch - n0 - mg_body;
    ctx->step_mg_body_launches = mg_body;
    ctx->nlaunch = n0;
    *out = g;
    return IMPEC_OK;
}

impec_status launch_pressure_graph(impec_ctx* ctx) {
    if (!ctx->cap_stream) {
        IMPEC_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
        IMPEC_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->body_stream, cudaStreamNonBlocking));
    }
    if (!ctx->pressure_exec) {
        IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        cudaGraph_t g;
        IMPEC_TRY(capture_pressure(ctx, &g));
        cudaError_t e = cudaGraphInstantiate(&ctx->pressure_exec, g, 0);
        cudaGraphDestroy(g);
        IMPEC_CUDA_TRY(e);
    }
    IMPEC_CUDA_TRY(cudaGraphLaunch(ctx->pressure_exec, ctx->stream));
    return IMPEC_OK;
}

void invalidate_step_graph(impec_ctx* ctx) {
    if (ctx->pressure_exec) {
        cudaGraphExecDestroy(ctx->pressure_exec);
        ctx->pressure_exec = nullptr;
    }
    for (int k = 0; k < 2; ++k)
        if (ctx->step_exec[k]) {
            cudaGraphExecDestroy(ctx->step_exec[k]);
            ctx->step_exec[k] = nullptr;
        }
}

// The same step launched kernel by kernel on the context stream with host-driven loops.
// Selected by IMPEC_NO_GRAPH=1: profilers cannot attribute kernels inside graphs that contain
// conditional nodes, so profiling runs use this path, which launches the same kernels.
static impec_status step_stream(impec_ctx* ctx, double t_clip) {
    DevScalars* S = ctx->dscal;
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_step_begin, 1, 1, 0, S);
    int cyc = 0;
    double rr = 0;
    impec_status st = pressure_solve(ctx, ctx->c, ctx->p, ctx->P.eps, &cyc, &rr);
    if (st != IMPEC_OK && st != IMPEC_ERR_NOT_CONVERGED) return st;
    IMPEC_TRY(velocity(ctx, ctx->p, ctx->c, ctx->u, ctx->v));
    IMPEC_TRY(max_stable_dt_dev(ctx, ctx->u, ctx->v));
    IMPEC_CUDA_TRY(cudaMemcpyAsync(&S->t_clip, &t_clip, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_clip_dt, 1, 1, 0, S);
    IMPEC_TRY(hyperbolic_solve_dev(ctx, ctx->c, ctx->u, ctx->v, &S->dt, &ctx->prev_first_sweep));
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_advance, 1, 1, 0, S, 0, 0, 0);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

impec_status launch_step_graph(impec_ctx* ctx, double t_clip) {
    const char* ng = getenv("IMPEC_NO_GRAPH");
    if (ng && ng[0] == '1') return step_stream(ctx, t_clip);
    if (!ctx->cap_stream) {
        IMPEC_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
        IMPEC_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->body_stream, cudaStreamNonBlocking));
    }
    const int variant = ctx->P.dim_splitting == IMPEC_ALTERNATING ? (ctx->prev_first_sweep ? 1 : 0) : 0;
    if (!ctx->step_exec[variant]) {
        IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        cudaGraph_t g;
        IMPEC_TRY(capture_step(ctx, variant, &g));
        cudaError_t e = cudaGraphInstantiate(&ctx->step_exec[variant], g, 0);
        cudaGraphDestroy(g);
        IMPEC_CUDA_TRY(e);
    }
    IMPEC_CUDA_TRY(cudaMemcpyAsync(&ctx->dscal->t_clip, &t_clip, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaGraphLaunch(ctx->step_exec[variant], ctx->stream));
    if (ctx->P.dim_splitting == IMPEC_ALTERNATING) ctx->prev_first_sweep = variant ? 0 : 1;
    else ctx->prev_first_sweep = ctx->P.dim_splitting == IMPEC_Y_FIRST ? 1 : 0;
    return IMPEC_OK;
}

}  // namespace impec
