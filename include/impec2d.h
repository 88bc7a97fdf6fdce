/*
 * impec2d.h -- C ABI of the GB300-native Impec2D IMPES engine (libimpec2d.so).
 *
 * Plain C types only.  Every call returns an impec_status; no call exits the process.
 * Device-pointer entry points ("_dev" arrays) take CUDA device memory in the engine's
 * device layout; the host entry points take host arrays in the reference's Blitz layout
 * and copy them across inside the call.
 *
 * Device layout (row-major, j fastest, no ghost cells; ghosts are applied by reflection
 * inside the kernels exactly as the reference's ghost fills define them):
 *   cell fields c, p, q, K:  N1 x N2,        element (i,j) at i*N2 + j
 *   x-face field u:           (N1+1) x N2,    u(i,j) is the face between cells (i-1,j), (i,j)
 *   y-face field v:           N1 x (N2+1),    v(i,j) is the face between cells (i,j-1), (i,j)
 * Host (reference) layout, src/Impec2DSolver.cpp:151-182:
 *   c, p: (N1+2g) x (N2+2g);  v: (N1+1+2g) x (N2+1+2g) x 2 (k innermost);  q: N1*N2.
 *
 * Each entry point names the reference interface it replaces (pw359/Impec2D, src/...).
 */
#ifndef IMPEC2D_H
#define IMPEC2D_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    IMPEC_OK = 0,
    IMPEC_ERR_ARG = 1,          /* invalid argument or size */
    IMPEC_ERR_CUDA = 2,         /* a CUDA call failed; see impec_last_error() */
    IMPEC_ERR_NOT_CONVERGED = 3,/* solver hit its cycle limit above tolerance */
    IMPEC_ERR_NAN = 4,          /* a NaN/Inf appeared in a residual or field */
    IMPEC_ERR_NO_DEVICE = 5,    /* no CUDA device / extension not usable */
    IMPEC_ERR_CONFIG = 6        /* .cfg parse or validation error */
} impec_status;

/* Enumerations keep the reference's values (src/SimParams.h:14-27). */
enum { IMPEC_MEANCONC = 0, IMPEC_HARMONIC = 1 };
enum { IMPEC_EXPLICIT = 0, IMPEC_CRANKNICOLSON = 1 };
enum { IMPEC_ALTERNATING = 0, IMPEC_X_FIRST = 1, IMPEC_Y_FIRST = 2, IMPEC_STRANG = 3,
       IMPEC_SYMMETRIC_PARALLEL = 4 };
/* hyper_method: upwind_split, waf_split and waf (the WAF flux in the split sweeps), ctu
 * (unsplit corner transport upwind), muscl. */
enum { IMPEC_UPWINDSPLIT = 0, IMPEC_WAFSPLIT = 1, IMPEC_WAF = 2, IMPEC_CTU = 3, IMPEC_MUSCL = 4 };
enum { IMPEC_PARALLEL = 0, IMPEC_DIAGONAL = 1, IMPEC_HORIZONTAL = 2 };
enum { IMPEC_BC_NEUMANN = 0, IMPEC_BC_PERIODIC = 1 };
/* Pressure-solver precision: plain FP64 multigrid, or FP32 V-cycles inside FP64
 * iterative refinement (residual, update, coarsest solve in FP64). */
enum { IMPEC_PREC_FP64 = 0, IMPEC_PREC_MIXED = 1 };

/* Numerical parameters: the subset of SimParams (src/SimParams.h:29-164) that the hot
 * path reads, plus the engine's own options (marked "engine"). */
typedef struct {
    int N1, N2;
    double x_lb, x_ub, y_lb, y_ub;
    double mu_res, mu_inj;
    int avgproc;              /* IMPEC_HARMONIC | IMPEC_MEANCONC */
    double nu;                /* stencil weight: 1 = 5-point, <1 = 9-point */
    double porosity, cfl, inj_fluid_conc, I;
    int diffusion;            /* Crank-Nicolson Peaceman dispersion on/off */
    double alpha_l, alpha_t;  /* cell units (multiplied by max(dx,dy)) */
    double Dm;                /* engine: molecular diffusion, 0 = reference */
    int ptype;                /* dt rule: IMPEC_CRANKNICOLSON ignores the diffusion limit */
    double dt_diff_limit;
    int dim_splitting;        /* IMPEC_SYMMETRIC_PARALLEL etc. */
    int hmtype;               /* IMPEC_MUSCL | IMPEC_UPWINDSPLIT | IMPEC_WAFSPLIT | IMPEC_WAF | IMPEC_CTU */
    int stype;                /* IMPEC_PARALLEL | IMPEC_DIAGONAL (sets the pinned cell) */
    int is_test, testno;      /* analytic permeability of the elliptic tests */
    int bc;                   /* IMPEC_BC_NEUMANN, or IMPEC_BC_PERIODIC (advection test) */
    double eps, para_eps;     /* elliptic / parabolic relative-residual tolerances */
    int peaceman_guard;       /* engine: Peaceman term := 0 where |u| = 0 (reference: NaN) */
    int cfl_porosity;         /* engine: CFL on interstitial speed |u|/phi (reference: 0) */
    int precision;            /* engine: IMPEC_PREC_FP64 | IMPEC_PREC_MIXED */
    int max_cycles;           /* engine: multigrid cycle limit per solve */
    int warm_start;           /* engine: 1 = start from the previous pressure (reference: 0) */
} impec_params;

typedef struct impec_ctx impec_ctx;

/* Last error message of this thread (static storage). */
const char* impec_last_error(void);
/* Fill *P with the defaults of examples/parallel.cfg for an N1 x N2 unit-square grid. */
void impec_default_params(impec_params* P, int N1, int N2);

/* Context: device workspaces for one grid.  stream may be NULL (legacy default stream).
 * Replaces the constructors MGSolver::MGSolver (src/MGSolver.cpp:52-143) and
 * HyperbolicSolver::HyperbolicSolver (src/HyperbolicSolver.cpp:63-67). */
impec_status impec_ctx_create(const impec_params* P, void* cuda_stream, impec_ctx** out);
impec_status impec_ctx_destroy(impec_ctx* ctx);
impec_status impec_ctx_params(const impec_ctx* ctx, impec_params* P);
/* Engine: per-cell permeability (device N1*N2 arrays, K22 may be NULL = K11; both NULL = 1).
 * Replaces K_11/K_22 (src/EllipticSolver.cpp:418-470). */
impec_status impec_set_permeability(impec_ctx* ctx, const double* K11_dev, const double* K22_dev);
/* Source term (device N1*N2).  Builds the well list used by the TR integrator. */
impec_status impec_set_source(impec_ctx* ctx, const double* q_dev);

/* Pressure solve: EllipticSolver::Solve -> MGSolver::SolveLinearMultigrid
 * (src/EllipticSolver.cpp:133-142, src/MGSolver.cpp:145-248).  Solves the reference's
 * pinned 9-point (nu<1) or 5-point (nu=1) system to ||b-Ap||/||b|| <= tol.
 * p_dev is the initial guess when warm_start is set, else it is overwritten. */
impec_status impec_pressure_solve(impec_ctx* ctx, const double* c_dev, double* p_dev,
                                  double tol, int* cycles, double* relres);
/* Pressure operator assembly only (engine diagnostics / tests): writes the face
 * mobilities lamx ((N1+1)*N2) and lamy (N1*(N2+1)) used by the solve. */
impec_status impec_face_mobility(impec_ctx* ctx, const double* c_dev, double* lamx_dev,
                                 double* lamy_dev);
/* y = A x with the reference's pinned pressure matrix (src/MGSolver.cpp:268-570). */
impec_status impec_pressure_apply(impec_ctx* ctx, const double* c_dev, const double* x_dev,
                                  double* y_dev);

/* Darcy face velocities: EllipticSolver::CalcVelocities (src/EllipticSolver.cpp:660-683). */
impec_status impec_velocity(impec_ctx* ctx, const double* p_dev, const double* c_dev,
                            double* u_dev, double* v_dev);
/* HyperbolicSolver::MaxStableTimestep (src/HyperbolicSolver.cpp:73-198). */
impec_status impec_max_stable_dt(impec_ctx* ctx, const double* u_dev, const double* v_dev,
                                 double* dt);

/* TRIntegrator::Integrate (src/TRIntegrator.cpp:49-71); *tmo = total_mass_outflux. */
impec_status impec_tr_integrate(impec_ctx* ctx, double* c_dev, double dt, double* tmo);
/* HyperbolicSplitSolver::Advect_X / Advect_Y (src/HyperbolicSplitSolver.cpp:113-159). */
impec_status impec_advect_x(impec_ctx* ctx, double* c_dev, const double* u_dev, double dt);
impec_status impec_advect_y(impec_ctx* ctx, double* c_dev, const double* v_dev, double dt);
/* HyperbolicSplitSolver::AdvectSplit (src/HyperbolicSplitSolver.cpp:51-106).
 * prev_first_sweep: 0 = X_SWEEP, 1 = Y_SWEEP (in/out). */
impec_status impec_advect_split(impec_ctx* ctx, double* c_dev, const double* u_dev,
                                const double* v_dev, double dt, int* prev_first_sweep);
/* HyperbolicSolver::DiffusionSplitCN -> MGSolver::Solve_Parabolic_cc_to_c
 * (src/HyperbolicSolver.cpp:217-223, src/MGSolver.cpp:846-1392). */
impec_status impec_dispersion_cn(impec_ctx* ctx, double* c_dev, const double* u_dev,
                                 const double* v_dev, double dt, double tol, int* its,
                                 double* relres);
/* HyperbolicSplitSolver::Solve (src/HyperbolicSplitSolver.cpp:162-198); *outflux
 * accumulates |total_mass_outflux| of both source half steps. */
impec_status impec_hyperbolic_solve(impec_ctx* ctx, double* c_dev, const double* u_dev,
                                    const double* v_dev, double dt, int* prev_first_sweep,
                                    double* outflux);

/* Reductions of src/Impec2DSolver.cpp:530-620: out[0] total mass, out[1] divergence
 * error, out[2] no-flow boundary error, out[3] max c, out[4] min c. */
impec_status impec_diagnostics(impec_ctx* ctx, const double* c_dev, const double* u_dev,
                               const double* v_dev, double out[5]);

/* ---- resident simulation: one IMPES step per call, state kept in HBM ---- */
typedef struct {
    double t, dt, total_outflux, relres, mass_err;
    int counter, its, para_its, prev_first_sweep;
    int clipped;              /* 1 if dt was shortened to reach t_clip */
} impec_step_info;
/* Device state (c, p, u, v, q) is owned by the context; these return its pointers. */
impec_status impec_state(impec_ctx* ctx, double** c_dev, double** p_dev, double** u_dev,
                         double** v_dev, double** q_dev);
/* Start time of the run (reference: starttime, src/Impec2DSolver.cpp:300); resets the
 * engine clock t and the outflux accumulator used by the mass balance. */
impec_status impec_set_time(impec_ctx* ctx, double t0);
/* One pass of the loop body of Impec2DSolver::Solve (src/Impec2DSolver.cpp:339-415) on the
 * resident state.  With t_clip >= 0, dt is shortened to t_clip - t when t + dt >= t_clip
 * (output-time matching, :375-378); t_clip < 0 disables it. */
impec_status impec_step(impec_ctx* ctx, double t_clip, impec_step_info* info);
/* n steps with no host synchronisation between them (dt stays on the device; info of the
 * last step is returned).  Used by throughput runs. */
impec_status impec_run_steps(impec_ctx* ctx, int n, impec_step_info* info);
/* Binary checkpoint of the resident run, for restarts that continue bit for bit: c, p, u, v,
 * the clock, start time, outflux accumulator, step counter and sweep order.  No counterpart in
 * the reference, which restarts only from an init_file of c (Impec2DSolver::Init,
 * src/Impec2DSolver.cpp:194-220; supported by the .cfg path).  Load checks the grid size, the
 * format and a checksum (IMPEC_ERR_ARG with a message otherwise) and is refused while the
 * context is a member of a live ensemble.  Both wait for the context's stream. */
impec_status impec_checkpoint_save(impec_ctx* ctx, const char* path);
impec_status impec_checkpoint_load(impec_ctx* ctx, const char* path);

/* Pressure solve of the resident state (c -> p) as one CUDA graph (no host round trip per
 * cycle).  With sync = 0 the call only enqueues; cycles/relres are then not written. */
impec_status impec_pressure_solve_resident(impec_ctx* ctx, int sync, int* cycles, double* relres);
/* Cycles, final and initial relative residual of the last pressure solve (waits for the
 * context's stream). */
impec_status impec_last_solve(impec_ctx* ctx, int* cycles, double* relres, double* relres0);
/* Kernel launches executed by this context so far (stream launches + step-graph replays). */
impec_status impec_launch_count(impec_ctx* ctx, long long* n);
/* Engine instrumentation: times `reps` stream launches of one hot kernel on the resident
 * state with CUDA events.  which: 0 fine-level red-black Gauss-Seidel sweep (both colours,
 * FP64), 1 the same in FP32, 2 FP64 fine residual + norm, 3 one x-sweep of the transport,
 * 4 one y-sweep of the transport.  Returns the mean time per launch and the algorithmic
 * bytes one launch moves. */
impec_status impec_time_kernel(impec_ctx* ctx, int which, int reps, double* ms_per_launch,
                               double* bytes_per_launch);

/* Output projection of a parallel-orientation run onto the diagonal grid: Impec2DSolver::Project
 * + ParallelProjector::FillDiagonal (src/Impec2DSolver.cpp:690-716,
 * src/ParallelProjector.cpp:95-199).  field 0 = the resident c, 1 = the resident p; out_dev
 * receives d_N1*d_N2 FP64 values, row-major (the reference uses d_N = round(N / sqrt 2)).  The
 * parallel field's ghost ring is its Neumann mirror.  Enqueued on the context's stream. */
impec_status impec_project_diagonal(impec_ctx* ctx, int field, double* out_dev, int d_N1, int d_N2);
/* The same into a host buffer of d_N1*d_N2 values (d_N1*d_N2 <= N1*N2); returns when it is filled. */
impec_status impec_project_diagonal_download(impec_ctx* ctx, int field, double* out_host, int d_N1, int d_N2);

/* Engine tunables of a context (no counterpart in the reference): "mg_pre", "mg_post" (smoother
 * sweeps before / after the coarse correction, 0..8, sum >= 1), "cluster" (0/1: coarse levels in
 * one thread-block-cluster launch), "cluster_cells", "cluster_cta0", "coarse_cells64",
 * "coarse_cells32" (level-size thresholds).  Defaults come from the IMPEC_MG_* environment at
 * context creation.  Changing a value drops the captured graphs. */
impec_status impec_set_tuning(impec_ctx* ctx, const char* name, long value);
impec_status impec_get_tuning(impec_ctx* ctx, const char* name, long* value);
/* Autotuner: times the resident pressure solve on the context's current state (reps replays
 * per candidate, CUDA events) for several smoother schedules and cluster choices, keeps the
 * fastest and leaves it set.  report (may be NULL) receives one line per candidate. */
impec_status impec_autotune(impec_ctx* ctx, int reps, char* report, int report_len);

/* Tensor-core GEMM of the learned warm start (no counterpart in the reference):
 * C[M x N] (fp32, row stride ldc) = A[M x K] (bf16, row stride lda) * B[N x K]^T (bf16, row
 * stride ldb), device pointers, on `stream`; returns after it completes.  K must be a multiple
 * of 64, lda and ldb multiples of 8, the operands 16-byte aligned. */
impec_status impec_gemm_bf16(const void* A, int lda, const void* B, int ldb, float* C, int ldc, int M, int N, int K,
                             void* stream);

/* 3x3 convolutions of the learned warm start on tcgen05 (no counterpart in the reference).
 * Activations NHWC bf16, channels multiples of 8; weights Wt [cout][Kp] bf16 with
 * k = tap * cin + c, tap = 3 (dy + 1) + (dx + 1), Kp = 9 cin rounded up to 64, zero padded.
 * Forward: v = conv(X) + bias; Z = v (bf16, optional), Y = act(v) (+ skip) (bf16, optional),
 * Yf = the same in fp32 (optional); act 0 = none, 1 = GELU.  Input gradient: the transposed
 * convolution of dZ; with gz given, multiplied by gelu'(gz) after adding `add`.  Weight
 * gradient: dW [cout][Kp] fp32 is accumulated into.  All return after completion. */
impec_status impec_conv3x3_forward(const void* X, int B, int H, int W, int cin, const void* Wt, const float* bias,
                                   int cout, int act, void* Z, void* Y, float* Yf, const void* skip, void* stream);
impec_status impec_conv3x3_input_grad(const void* dZ, int B, int H, int W, int cout, const void* Wt, int cin,
                                      const void* gz, const void* add, void* Y, float* Yf, void* stream);
impec_status impec_conv3x3_weight_grad(const void* dZ, const void* X, int B, int H, int W, int cin, int cout, float* dW,
                                       void* stream);

/* Learned warm start (no counterpart in the reference): a 4-level convolutional encoder-decoder
 * (15 3x3 convolutions, 32..256 channels, GELU, additive skips; BF16 weights and activations,
 * fp32 accumulation on the tensor cores, fp32 AdamW master weights).  Inputs X are
 * [B][H][W][8] bf16 feature maps (channels 5..7 zero), targets T and predictions [B][H][W]
 * fp32; H and W multiples of 8. */
typedef struct impec_net impec_net;
impec_status impec_net_create(unsigned long long seed, impec_net** out);
/* Fails while the network is attached to a context. */
impec_status impec_net_destroy(impec_net* net);
/* One AdamW step (lr, decoupled weight decay) on a batch; *loss = the batch's mean squared error. */
impec_status impec_net_train_batch(impec_net* net, const void* X, const float* T, int B, int H, int W, double lr,
                                   double weight_decay, double* loss, void* stream);
/* Forward and backward only: the parameter gradients are left for impec_net_parameters(which = 1). */
impec_status impec_net_backprop(impec_net* net, const void* X, const float* T, int B, int H, int W, double* loss,
                                void* stream);
impec_status impec_net_forward(impec_net* net, const void* X, int B, int H, int W, float* out, void* stream);
/* *count = number of parameters; which 0: weights (host_out receives, host_in replaces),
 * which 1: gradients (host_out receives).  Order: per layer, weights [cout][Kp] then bias. */
impec_status impec_net_parameters(impec_net* net, float* host_out, const float* host_in, size_t* count, int which);

/* Attaches net to ctx's pressure solves (mode 1: predict, 2: record only), or detaches it (net
 * NULL or mode 0).  Needs warm_start (x0 = the previous pressure) and a well-driven pure-Neumann
 * system.  Each solve then computes r0 = f - A x0 and the features [mean 4 log(1-c+M^(1/4)c),
 * mean log K, sum q dA/I, centred x0 / RMS, r0 / RMS] over factor x factor cells (factor 1, 2,
 * 4, 8 or 16; N1 and N2 multiples of 8 * factor).  Predicting, the network's output d (bilinear to
 * the fine grid) moves the iterate: x0 += alpha d, alpha = (r0, d) / (d, A d); the solve still
 * converges to its tolerance.  The captured step graph is rebuilt at the next step. */
impec_status impec_learned_attach(impec_ctx* ctx, impec_net* net, int factor, int mode);
/* Features of the last solve: X bf16 [N1/factor][N2/factor][8] on the device. */
impec_status impec_learned_features(impec_ctx* ctx, void* X);
/* Training target of the last solve: the mean of (p - x0) over each factor x factor block, p the
 * resident converged pressure, centred and scaled to unit RMS; T fp32 [N1/factor][N2/factor]. */
impec_status impec_learned_target(impec_ctx* ctx, float* T);
/* Step length of the last solve's learned correction (0: rejected). */
impec_status impec_learned_alpha(impec_ctx* ctx, double* alpha);

/* Cold timing of one fine-level smoother sweep (which 0: FP64, 1: FP32; five-point levels):
 * before each of `reps` repetitions `flush_bytes` of the device buffer `flush` are overwritten
 * on the context's stream, so the sweep's data comes from HBM; each repetition is timed with
 * events on that stream.  *ms: mean, *ms_min: fastest, *bytes: the sweep's algorithmic bytes (x
 * read and written, b, the two face planes).  A benchmark probe; no counterpart in the
 * reference. */
impec_status impec_time_kernel_cold(impec_ctx* ctx, int which, int reps, void* flush, size_t flush_bytes,
                                    double* ms, double* ms_min, double* bytes);

/* FP64 fused multiply-adds per second that the current device sustains (eight independent
 * chains per thread on every SM): the denominator of the FP64-pipe fractions reported beside
 * the HBM roofline.  No counterpart in the reference. */
impec_status impec_measure_fp64(double* fma_per_second);

/* Self-test of the bounded waits that guard every tensor-core and TMA wait of the engine (no
 * counterpart in the reference).  A one-thread kernel waits on an mbarrier with the same
 * bounded poll loop: with arrive != 0 it arrives first and the wait completes (*timed_out = 0);
 * with arrive == 0 nothing ever arrives, the wait gives up after max_tries polls
 * (<= 1,048,576, a fraction of a millisecond) and *timed_out = 1.  Either way the kernel returns
 * and the context stays usable: this is how a lost copy surfaces as an error status instead of
 * a hung GPU. */
impec_status impec_selftest_bounded_wait(unsigned max_tries, int arrive, int* timed_out);

/* Allocation-free transport step.  No counterpart in the reference: it exists for callers
 * that may not allocate device memory themselves or through this library -- code running
 * under a host framework that owns every device allocation (a fixed pool or budget), or that
 * must avoid cudaMalloc's implicit device-wide synchronisation -- and so cannot create an
 * impec_ctx.  It performs AdvectSplit's symmetric-parallel update (MUSCL or upwind by
 * P->hmtype, Neumann or periodic by P->bc; P->dim_splitting must be IMPEC_SYMMETRIC_PARALLEL,
 * other values are rejected with IMPEC_ERR_ARG) of c_dev in place, given u_dev, v_dev and dt,
 * enqueued on `stream` (may be NULL), without allocating: its scratch (a copy of dt and the
 * updated field) is a static device array of 1,048,576 cells (8 MiB) that every GPU which
 * loads the library holds until process exit.  Nothing in it has to start at zero: each call
 * writes dt and every cell of the updated field before reading them.  Larger grids
 * (N1*N2 > 1,048,576) are rejected with IMPEC_ERR_ARG.  dt is handed to the GPU as a kernel
 * argument (by value), never copied from the caller's memory.  The first call on a device
 * looks up the array's device address, so make that first call before any stream capture;
 * the address is kept for the life of the process, so after cudaDeviceReset on a device do
 * not call this entry point again in that process.  All calls share the array: calls whose
 * work overlaps on the GPU (different streams, or different host threads) race on it. */
impec_status impec_advect_symmetric_noalloc(const impec_params* P, double* c_dev, const double* u_dev,
                                            const double* v_dev, double dt, void* stream);

/* ---- ensembles of independent realisations ---- */
/* One CUDA graph holding each member's whole IMPES step as a parallel branch, so one launch
 * advances every member (the batched-ensemble mode; no counterpart in the reference,
 * whose driver runs one realisation per process).  Members must not use alternating sweeps and
 * run without output-time clipping.  A member's later changes of tunables are not seen by an
 * existing ensemble: create it again.  While an ensemble lives, calls that would free or move
 * a member's buffers fail with IMPEC_ERR_ARG: impec_ctx_destroy, impec_learned_attach,
 * impec_set_source with new well cells, impec_set_permeability changing between isotropic and
 * anisotropic (new values in the same layout are copied in place and seen by the ensemble). */
typedef struct impec_ensemble impec_ensemble;
impec_status impec_ensemble_create(impec_ctx* const* members, int n, impec_ensemble** out);
/* nsteps graph launches on the ensemble's stream, ordered after work already queued on the
 * members' streams and before work queued on them afterwards; sync != 0 waits for the end. */
impec_status impec_ensemble_step(impec_ensemble* e, int nsteps, int sync);
impec_status impec_ensemble_destroy(impec_ensemble* e);

/* ---- host-buffer entry points (reference Blitz layouts; copies inside the call) ---- */
impec_status impec_state_upload(impec_ctx* ctx, const double* c_host, const double* q_host,
                                int ghost);
impec_status impec_state_download(impec_ctx* ctx, double* c_host, double* p_host,
                                  double* v_host, int ghost);
/* Host velocity (reference layout, v(i,j,k)) -> device u, v of the resident state. */
impec_status impec_velocity_upload(impec_ctx* ctx, const double* v_host, int ghost);
/* Host pressure (reference layout) -> device p of the resident state. */
impec_status impec_pressure_upload(impec_ctx* ctx, const double* p_host, int ghost);
/* Dirichlet-row coefficient kappa of the pinned cell (row = kappa/dA, src/MGSolver.cpp:518-567);
 * 1 in production runs, chosen from the exact solution in the elliptic tests. */
impec_status impec_set_pin_kappa(impec_ctx* ctx, double kappa);

/* ---- configuration files (libconfig .cfg of the reference, src/SimParams.cpp:45-468) ---- */
/* Parse a .cfg into engine parameters (+ start/end time).  Errors: IMPEC_ERR_CONFIG. */
impec_status impec_cfg_load(const char* path, impec_params* P, double* tstart, double* tfinal);
/* Source term q (host, N1*N2) of the .cfg's wells: Impec2DSolver::InitializeSource
 * (src/Impec2DSolver.cpp:241-280). */
impec_status impec_cfg_source(const char* path, double* q_host);
/* Run a whole .cfg like the reference executable: Impec2DSolver(cfg).Run()
 * (src/Driver.cpp:58-87); quiet suppresses the per-step console line. */
impec_status impec_run_cfg(const char* path, int quiet);

#ifdef __cplusplus
}
#endif
#endif
