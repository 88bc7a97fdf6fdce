// Internal declarations of the GB300 Impec2D engine (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/impec2d.h"

namespace impec {

// ---------------------------------------------------------------- NVTX ranges
// A named range over a host call, seen by profilers that record NVTX (Nsight Systems, ncu
// --nvtx); without such a tool attached a push or pop is a no-op.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
#define IMPEC_RANGE_CAT2(a, b) a##b
#define IMPEC_RANGE_CAT(a, b) IMPEC_RANGE_CAT2(a, b)
#define IMPEC_RANGE(name) ::impec::NvtxRange IMPEC_RANGE_CAT(impec_range_, __LINE__)(name)

// ---------------------------------------------------------------- error handling
void set_error(const std::string& msg);
#define IMPEC_CUDA_TRY(expr)                                                                   \
    do {                                                                                       \
        cudaError_t _e = (expr);                                                               \
        if (_e != cudaSuccess) {                                                               \
            ::impec::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e) + " at " +   \
                               __FILE__ + ":" + std::to_string(__LINE__));                     \
            return IMPEC_ERR_CUDA;                                                             \
        }                                                                                      \
    } while (0)
#define IMPEC_LAUNCH_CHECK() IMPEC_CUDA_TRY(cudaGetLastError())
#define IMPEC_TRY(expr)                          \
    do {                                         \
        impec_status _s = (expr);                \
        if (_s != IMPEC_OK) return _s;           \
    } while (0)

// ---------------------------------------------------------------- grid constants
// Trigonometric constants of the rotated (diagonal) stencil, src/EllipticSolver.cpp:59-100.
struct Geo {
    double dx, dy, dA, dxi, deta, secamt2, cosa2, sina2, costsina, cosasint, cost2, sint2, cosa,
        sint, cost, sina, mob1over4;
};
Geo make_geo(const impec_params& P);

// Reflection of cell and face indices that reproduces the reference ghost fills
// (src/Util.cpp:215-438): scalars are mirrored about the boundary face (even), the normal
// velocity component is mirrored with a sign change about the boundary face (odd).
__host__ __device__ inline int refl_cell(int i, int n) { return i < 0 ? -1 - i : (i >= n ? 2 * n - 1 - i : i); }
__host__ __device__ inline int wrap_cell(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
// Face index f in [0, n]; returns index in range and sets sign to -1 where reflected.
__host__ __device__ inline int refl_face(int f, int n, double& sign) {
    if (f < 0) { sign = -sign; return -f; }
    if (f > n) { sign = -sign; return 2 * n - f; }
    return f;
}
__host__ __device__ inline int wrap_face(int f, int n) { return f < 0 ? f + n : (f > n ? f - n : f); }

// ---------------------------------------------------------------- multigrid level
enum LevelKind { FACE5 = 5, EXP9 = 9 };
struct Level {
    int n1 = 0, n2 = 0, kind = FACE5;
    __host__ __device__ size_t n() const { return (size_t)n1 * n2; }
    // FP64 operator (integrated, positive-definite sign convention)
    double* tx = nullptr;    // FACE5: (n1+1)*n2 x-face transmissibilities (boundary faces 0)
    double* ty = nullptr;    // FACE5: n1*(n2+1)
    double* a9 = nullptr;    // EXP9: 9 planes of n1*n2, folded (no coupling outside the grid)
    double* idiag = nullptr; // 1 / diagonal
    double* diag = nullptr;  // diagonal (FACE5: sum of the four faces + ed; EXP9: plane 0)
    double* ed = nullptr;    // FACE5 with a Dirichlet row: couplings to known cells, moved to the diagonal
    double *x = nullptr, *b = nullptr;
    // FP32 copies for the mixed-precision cycle
    float *tx32 = nullptr, *ty32 = nullptr, *a932 = nullptr, *idiag32 = nullptr, *diag32 = nullptr;
    float *x32 = nullptr, *b32 = nullptr;
    // second iterate buffers of the one-launch red-black sweep (ping-pong; FACE5 levels)
    double* xa = nullptr;
    float* xa32 = nullptr;
};

enum { FLAG_MG_NOT_CONVERGED = 1, FLAG_MG_NAN = 2, FLAG_CN_NOT_CONVERGED = 4, FLAG_CN_NAN = 8 };

// ---- programmatic dependent launch
// Every kernel of the engine starts with pdl_enter(): it waits until the kernel before it in
// the stream has completed and its writes are visible (griddepcontrol.wait), then allows the
// next kernel's CTAs to be scheduled (griddepcontrol.launch_dependents), so the next launch's
// latency overlaps this kernel's run.  Since each kernel waits for its predecessor before
// touching memory, a kernel also sees the writes of every earlier kernel in the stream.
// Both instructions do nothing in a kernel launched without the attribute.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

bool pdl_enabled();  // programmatic launches only with IMPEC_PDL=1

// kernel<<<g, b, smem, s>>>(args...) with the programmatic-serialisation attribute.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(cudaStream_t s, void (*k)(KArgs...), dim3 g, dim3 b, size_t smem, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = b;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

// Device-resident scalars of a step (so a step needs no host round trip).
struct DevScalars {
    double dt, t, maxvel, tmo_pre, tmo_post, total_outflux;
    double fsum, fnorm2, rnorm2, pin_value;  // fsum,fnorm2 adjacent: written as a pair
    double red[8];
    double relres, cn_relres, t_clip;
    double pcg_rz, pcg_zq;  // (r, z) and (z, q_old) of the current CG iteration (written as a pair)
    double pcg_pq, pcg_alpha, pcg_rz_old;
    // the iteration's beta (for the direction) and alpha (for the update), each computed once by
    // the last block of the reduction that completes its operands instead of in every thread
    double pcg_beta, pcg_step;
    double relres0;  // relative residual of the initial iterate of the last pressure solve
    int mg_cycles, cn_cycles, cn_cycles_total, flags, go, clipped, steps;
    long long graph_launches;  // kernels executed by step-graph replays
};

}  // namespace impec

namespace impec {
// Engine tunables of one context (defaults from the IMPEC_MG_* environment at creation).
struct LearnedHook;  // learned_net.cu

struct Tuning {
    // Smoother sweeps before / after the coarse correction: V(1,2) for five-point operators
    // (1024^2 IMPES step 3.19 ms against 3.32 ms with V(2,2), 10 instead of 9 iterations;
    // at 4096^2 on heterogeneous fields the FP64 solve ties), V(1,1) for nine-point ones.
    long pre = 1, post = 2;
    long cluster = 1;              // coarse levels in one thread-block-cluster launch
    long cl_cells = 16384;         // largest level of the cluster V-cycle
    long cl_cta0 = 256;            // cluster levels up to this many cells run on CTA 0
    long coarse_cells64 = 256;     // single-CTA coarse V-cycle (nine-point path), FP64
    long coarse_cells32 = 1024;    // the same, FP32
    long rb_skip = 1;  // five-point levels: no zero fill before pre-smoothing, red-only prolongation
    long rb_resid = 1;  // five-point levels: restriction sums the red residuals only (black ones are ~0)
    // FP64 five-point levels of at least this many cells sweep both colours in one launch
    // (k_rb_tile, ping-pong iterate): every coefficient is read once per sweep instead of once
    // per colour, which pays where the level streams from HBM (4096^2 sweep 185 against 240 us
    // cold; 4096^2 solve 17.9 ms with 2048^2 and 4096^2 levels so swept, 18.0 with 4096^2
    // alone, 19.7 with none) and costs where it sits in L2 (1024^2 solve 2.23 against 2.08 ms
    // with every level so swept: the recomputed ring and one more dependent phase); 0 disables
    long tile_cells = 1L << 22;
    // the same for FP32 levels (mixed precision): 4096^2 cold sweep 110 against 130 us, mixed
    // solve 14.35 against 14.44 ms; with every level so swept the 1024^2 solve is 12% slower
    long tile_cells32 = 1L << 22;
};
}  // namespace impec

struct impec_ctx {
    impec_params P;
    impec::Geo G;
    cudaStream_t stream = nullptr;
    int device = 0, num_sms = 148;
    int cl_size = 0;  // CTAs per cluster of the cluster V-cycle (0: cluster launches unavailable)
    // resident state
    double *c = nullptr, *p = nullptr, *u = nullptr, *v = nullptr, *q = nullptr;
    double *K11 = nullptr, *K22 = nullptr;  // owned copies, or nullptr (K = 1)
    // pressure operator
    double *muK11 = nullptr, *muK22 = nullptr;    // per-cell mu/K
    double *lamx = nullptr, *lamy = nullptr;      // face mobilities (reference KoverMu)
    double *cm11 = nullptr, *cm22 = nullptr, *cm12 = nullptr;  // corner tensors (nu < 1)
    double *f = nullptr, *r = nullptr;            // integrated rhs, FP64 residual
    std::vector<impec::Level> L;
    double* dense_inv = nullptr;                  // coarsest-level inverse (n x n)
    // V-cycle preconditioned conjugate gradients: iterate, search direction, A p
    double *cg_x = nullptr, *cg_p = nullptr, *cg_q = nullptr;
    int krylov = 1;  // 1: CG with one V-cycle as preconditioner; 0: stationary V-cycles
    impec::Tuning tune;
    int cn_predict = 1;  // CN starts from the explicit-Euler predictor (IMPEC_CN_PREDICT=0: from c)
    int dense_n = 0;
    int pin_i = 1, pin_j = 1;
    double pin_kappa = 1.0;
    // source_type horizontal: Dirichlet row dir_row of the pressure system (cells (1, j),
    // src/MGSolver.cpp:119-140) and of the CN system (cells (N1-2, j), :133-139); -1 otherwise
    int dir_row = -1, cn_dir_row = -1;
    int singular = 1;            // the pressure system is the singular Neumann one (no Dirichlet row)
    int eliminate = 1;           // remove the known cells from the operator (off only to apply the reference matrix)
    unsigned char* dmask = nullptr;  // finest level: 1 at known (Dirichlet) cells
    double* dfd = nullptr;           // finest level: rhs additions from known neighbours; the value at known cells
    // transport scratch
    double *t1 = nullptr, *t2 = nullptr, *t3 = nullptr;
    // wells (TR integrator)
    int nwells = 0;
    std::vector<int> well_idx_host;  // host copy of the well cells (a source with the same cells keeps the graph)
    int* well_idx = nullptr;
    double* well_q = nullptr;
    // dispersion
    double *dfx = nullptr, *dfy = nullptr;        // Peaceman tensors at x-faces (d11,d12) and y-faces (d22,d21)
    double *cn_a9 = nullptr, *cn_b = nullptr, *cn_idiag = nullptr;
    // reductions
    double* partials = nullptr;                   // [8][max_blocks]
    unsigned* counter = nullptr;
    int max_blocks = 0;
    impec::DevScalars* dscal = nullptr;
    impec::DevScalars* hscal = nullptr;           // pinned host mirror
    // run state
    double t = 0, t0 = 0, total_outflux = 0;
    int counter_steps = 0, prev_first_sweep = 1, last_its = 0, last_para_its = 0;
    // FLAG_* bits of the current step that the kernel-by-kernel path learned on the host (its
    // later solves reset the device flags), merged into the step's report
    int host_flags = 0;
    double last_relres = 0;
    bool have_source = false;
    long long nlaunch = 0;                         // kernel launches issued (captured ones included)
    // resident-step CUDA graph
    cudaStream_t cap_stream = nullptr, body_stream = nullptr;
    cudaGraphExec_t step_exec[2] = {nullptr, nullptr};
    cudaGraphExec_t pressure_exec = nullptr;
    long long step_cn_body_launches = 0;  // kernels of one CN loop body (the step graph's launch count)
    // learned initial guess (learned_net.cu): the attached network's state, and the residual of
    // the previous pressure, the predicted direction, its image under A and the step length
    impec::LearnedHook* learned = nullptr;
    double *lrn_r0 = nullptr, *lrn_d = nullptr, *lrn_Ad = nullptr, *lrn_alpha = nullptr;
    // live ensembles whose captured graph holds this context's buffers: calls that would free
    // or move a buffer are refused while it is non-zero
    int ensembles = 0;
};

namespace impec {
// pressure.cu
impec_status pressure_setup(impec_ctx* ctx, const double* c);
impec_status pressure_solve(impec_ctx* ctx, const double* c, double* p, double tol, int* cycles, double* relres);
impec_status pressure_alloc(impec_ctx* ctx);
void pressure_free(impec_ctx* ctx);
impec_status face_mobility(impec_ctx* ctx, const double* c);
impec_status pressure_apply_ref(impec_ctx* ctx, const double* x, double* y);
impec_status pressure_prepare(impec_ctx* ctx, const double* c, const double* p);
impec_status pressure_residual(impec_ctx* ctx);
impec_status pressure_check(impec_ctx* ctx, double tol, int inc, cudaGraphConditionalHandle h, int use_h);
impec_status pressure_iteration(impec_ctx* ctx, double tol, cudaGraphConditionalHandle h, int use_h);
impec_status pressure_step(impec_ctx* ctx, double tol, cudaGraphConditionalHandle h, int use_h);
impec_status pressure_finish(impec_ctx* ctx, double* p);
// elliptic velocity
impec_status velocity(impec_ctx* ctx, const double* p, const double* c, double* u, double* v);
impec_status max_stable_dt_dev(impec_ctx* ctx, const double* u, const double* v);
// transport.cu
impec_status tr_integrate_dev(impec_ctx* ctx, double* c, double dt_scale, const double* dt_dev, int slot);
impec_status advect_x_dev(impec_ctx* ctx, const double* cin, double* cout, const double* u, double dt_scale,
                          const double* dt_dev, const double* cghost = nullptr);
impec_status advect_y_dev(impec_ctx* ctx, const double* cin, double* cout, const double* v, double dt_scale, const double* dt_dev);
impec_status advect_split_dev(impec_ctx* ctx, double* c, const double* u, const double* v, const double* dt_dev, int* pfs);
impec_status average_dev(impec_ctx* ctx, double* c, const double* a, const double* b);
// dispersion.cu
impec_status cn_setup(impec_ctx* ctx, const double* u, const double* v, double dt_scale, const double* dt_dev);
impec_status cn_prepare(impec_ctx* ctx, double* c, double dt_scale, const double* dt_dev, bool residual = true);
impec_status cn_check(impec_ctx* ctx, double tol, int inc, cudaGraphConditionalHandle h, int use_h);
impec_status cn_iteration(impec_ctx* ctx, double* c);
impec_status dispersion_cn_dev(impec_ctx* ctx, double* c, const double* u, const double* v, double dt_scale,
                               const double* dt_dev, double tol, int* its, double* relres);
// ctx.cu: false (and the error set) when ctx belongs to a live ensemble
bool buffers_movable(const impec_ctx* ctx, const char* what);
// learned_net.cu
bool learned_predicts(const impec_ctx* ctx);
impec_status learned_predict(impec_ctx* ctx, const double* x, const double* r0, double* d);
void learned_release(impec_ctx* ctx);
// graph.cu
impec_status launch_step_graph(impec_ctx* ctx, double t_clip);
impec_status launch_pressure_graph(impec_ctx* ctx);
void invalidate_step_graph(impec_ctx* ctx);
// step.cu
impec_status hyperbolic_solve_dev(impec_ctx* ctx, double* c, const double* u, const double* v, const double* dt_dev,
                                  int* pfs);
// reductions (common.cu)
impec_status reduce_launch_sum(impec_ctx* ctx, const double* x, size_t n, double* out_dev);
impec_status sync_scalars(impec_ctx* ctx);
}  // namespace impec
