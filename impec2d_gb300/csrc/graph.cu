// The resident IMPES step as one CUDA graph.
//
// One pass of the loop body of Impec2DSolver::Solve (src/Impec2DSolver.cpp:339-415) is
// captured once per context: pressure operator + multigrid, Darcy velocities, the CFL step and
// output-time clipping, and HyperbolicSplitSolver::Solve.  The two iterative parts (multigrid
// cycles to eps, Crank-Nicolson Gauss-Seidel sweeps to para_eps) are WHILE conditional nodes
// whose condition is set on the device by the convergence-check kernel, so a step needs no
// host round trip and steps can be queued back to back.
#include <cmath>
#include <string>
#include <vector>

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
// loop bodies times their trip counts.  Each of the cn_solves CN solves runs its first sweep
// outside the loop (it is among the fixed nodes) but counts it in cn_cycles_total.
__global__ void k_advance(DevScalars* S, long long outer, long long mg_body, long long cn_body, int cn_solves) {
    pdl_enter();
    S->t += S->dt;
    S->steps++;
    S->graph_launches += outer + mg_body * S->mg_cycles + cn_body * (S->cn_cycles_total - cn_solves);
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
    IMPEC_TRY(cn_prepare(ctx, c, 0.5, &ctx->dscal->dt, false));
    long long nb = 0;
    IMPEC_TRY(capture_while(
        ctx,
        [&](cudaGraphConditionalHandle h) {  // the first sweep runs before the first check (as dispersion_cn_dev)
            IMPEC_TRY(cn_iteration(ctx, c));
            return cn_check(ctx, tol, 1, h, 1);
        },
        [&](cudaGraphConditionalHandle h) {
            IMPEC_TRY(cn_iteration(ctx, c));
            return cn_check(ctx, tol, 1, h, 1);
        },
        nb));
    ctx->step_cn_body_launches = nb;
    return IMPEC_OK;
}

// Captures one step, for the given alternating-sweep parity (0: X first, 1: Y first), into
// the capture that is active on ctx->cap_stream (its own, or an ensemble's joined by an event).
static impec_status capture_step_into(impec_ctx* ctx, int pfs_in) {
    const impec_params& P = ctx->P;
    DevScalars* S = ctx->dscal;
    const double* dt = &S->dt;
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
                return pressure_step(ctx, P.eps, h, 1);
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
                 P.diffusion ? ctx->step_cn_body_launches : 0LL, P.diffusion ? 2 : 0);
        IMPEC_LAUNCH_CHECK();
        return IMPEC_OK;
    };
    impec_status s = body();
    ctx->stream = saved;
    ctx->nlaunch = n0;  // captured launches run (and are counted) on the device at each replay
    return s;
}

static impec_status capture_step(impec_ctx* ctx, int pfs_in, cudaGraph_t* out) {
    IMPEC_CUDA_TRY(cudaStreamBeginCapture(ctx->cap_stream, cudaStreamCaptureModeRelaxed));
    impec_status s = capture_step_into(ctx, pfs_in);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->cap_stream, &g);
    IMPEC_TRY(s);
    IMPEC_CUDA_TRY(e);
    *out = g;
    return IMPEC_OK;
}

static impec_status ensure_capture_streams(impec_ctx* ctx) {
    if (!ctx->cap_stream) {
        IMPEC_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
        IMPEC_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->body_stream, cudaStreamNonBlocking));
    }
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
                return pressure_step(ctx, P.eps, h, 1);
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
    impec_status st;
    {
        IMPEC_RANGE("pressure");
        st = pressure_solve(ctx, ctx->c, ctx->p, ctx->P.eps, &cyc, &rr);
    }
    if (st != IMPEC_OK && st != IMPEC_ERR_NOT_CONVERGED) return st;
    if (st == IMPEC_ERR_NOT_CONVERGED) ctx->host_flags |= FLAG_MG_NOT_CONVERGED;
    {
        IMPEC_RANGE("velocity and dt");
        IMPEC_TRY(velocity(ctx, ctx->p, ctx->c, ctx->u, ctx->v));
        IMPEC_TRY(max_stable_dt_dev(ctx, ctx->u, ctx->v));
    }
    IMPEC_CUDA_TRY(cudaMemcpyAsync(&S->t_clip, &t_clip, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_clip_dt, 1, 1, 0, S);
    {
        IMPEC_RANGE("transport and dispersion");
        IMPEC_TRY(hyperbolic_solve_dev(ctx, ctx->c, ctx->u, ctx->v, &S->dt, &ctx->prev_first_sweep));
    }
    ++ctx->nlaunch;
    launch_k(ctx->stream, k_advance, 1, 1, 0, S, 0LL, 0LL, 0LL, 0);
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

// ---------------------------------------------------------------- ensembles
// Independent realisations advanced together: one CUDA graph holds every member's whole IMPES
// step (its WHILE loops included) as a parallel branch, so one graph launch advances all
// members and the GPU overlaps their kernels.  Members keep their own buffers, scalars and
// reduction scratch, so the branches share nothing.
struct impec_ensemble {
    std::vector<impec_ctx*> m;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t fork = nullptr, done = nullptr;
    std::vector<cudaEvent_t> join;
};

using namespace impec;

static void ensemble_free(impec_ensemble* e) {
    if (!e) return;
    if (e->exec) cudaGraphExecDestroy(e->exec);
    for (cudaEvent_t ev : e->join)
        if (ev) cudaEventDestroy(ev);
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->done) cudaEventDestroy(e->done);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

extern "C" impec_status impec_ensemble_create(impec_ctx* const* members, int n, impec_ensemble** out) {
    IMPEC_RANGE("impec_ensemble_create");
    if (!members || n < 1 || !out) return IMPEC_ERR_ARG;
    for (int i = 0; i < n; ++i) {
        if (!members[i]) return IMPEC_ERR_ARG;
        if (members[i]->P.dim_splitting == IMPEC_ALTERNATING) {
            set_error("impec_ensemble_create: members with alternating sweeps need two step variants; not supported");
            return IMPEC_ERR_ARG;
        }
        for (int k = 0; k < i; ++k)
            if (members[k] == members[i]) {
                set_error("impec_ensemble_create: a context appears twice");
                return IMPEC_ERR_ARG;
            }
    }
    impec_ensemble* e = new impec_ensemble;
    e->m.assign(members, members + n);
    e->join.assign(n, nullptr);
    auto fail = [&](impec_status s) {
        ensemble_free(e);
        return s;
    };
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming) != cudaSuccess) {
        set_error("impec_ensemble_create: stream or event creation failed");
        return fail(IMPEC_ERR_CUDA);
    }
    const double no_clip = -1.0;
    for (int i = 0; i < n; ++i) {
        impec_ctx* c = e->m[i];
        if (cudaEventCreateWithFlags(&e->join[i], cudaEventDisableTiming) != cudaSuccess) return fail(IMPEC_ERR_CUDA);
        impec_status s = ensure_capture_streams(c);
        if (s != IMPEC_OK) return fail(s);
        if (cudaMemcpyAsync(&c->dscal->t_clip, &no_clip, sizeof(double), cudaMemcpyHostToDevice, c->stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(c->stream) != cudaSuccess) {
            set_error("impec_ensemble_create: member stream failed");
            return fail(IMPEC_ERR_CUDA);
        }
    }
    if (cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        set_error("impec_ensemble_create: capture failed to start");
        return fail(IMPEC_ERR_CUDA);
    }
    impec_status s = IMPEC_OK;
    cudaError_t ce = cudaEventRecord(e->fork, e->stream);
    for (int i = 0; i < n && s == IMPEC_OK && ce == cudaSuccess; ++i) {
        impec_ctx* c = e->m[i];
        ce = cudaStreamWaitEvent(c->cap_stream, e->fork, 0);
        if (ce != cudaSuccess) break;
        s = capture_step_into(c, 0);  // the variant a single context replays (non-alternating splitting)
        if (s != IMPEC_OK) break;
        ce = cudaEventRecord(e->join[i], c->cap_stream);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(e->stream, e->join[i], 0);
    }
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(e->stream, &g);
    if (s != IMPEC_OK) {
        if (g) cudaGraphDestroy(g);
        return fail(s);
    }
    if (ce != cudaSuccess || ee != cudaSuccess) {
        set_error(std::string("impec_ensemble_create: capture failed: ") + cudaGetErrorString(ce != cudaSuccess ? ce : ee));
        if (g) cudaGraphDestroy(g);
        return fail(IMPEC_ERR_CUDA);
    }
    ce = cudaGraphInstantiate(&e->exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
        set_error(std::string("impec_ensemble_create: instantiation failed: ") + cudaGetErrorString(ce));
        return fail(IMPEC_ERR_CUDA);
    }
    for (impec_ctx* c : e->m) ++c->ensembles;  // the graph now holds their buffers
    *out = e;
    return IMPEC_OK;
}

extern "C" impec_status impec_ensemble_step(impec_ensemble* e, int nsteps, int sync) {
    IMPEC_RANGE("impec_ensemble_step");
    if (!e || nsteps < 0) return IMPEC_ERR_ARG;
    for (impec_ctx* c : e->m) {  // work queued on a member's own stream comes first
        IMPEC_CUDA_TRY(cudaEventRecord(e->done, c->stream));
        IMPEC_CUDA_TRY(cudaStreamWaitEvent(e->stream, e->done, 0));
    }
    for (int k = 0; k < nsteps; ++k) IMPEC_CUDA_TRY(cudaGraphLaunch(e->exec, e->stream));
    IMPEC_CUDA_TRY(cudaEventRecord(e->done, e->stream));
    for (impec_ctx* c : e->m) IMPEC_CUDA_TRY(cudaStreamWaitEvent(c->stream, e->done, 0));
    if (sync) IMPEC_CUDA_TRY(cudaStreamSynchronize(e->stream));
    return IMPEC_OK;
}

extern "C" impec_status impec_ensemble_destroy(impec_ensemble* e) {
    if (!e) return IMPEC_OK;
    cudaStreamSynchronize(e->stream);
    for (impec_ctx* c : e->m) --c->ensembles;
    ensemble_free(e);
    return IMPEC_OK;
}
