// Transport: trapezoidal source integrator and dimensionally split MUSCL / upwind advection.
//
// Ghost cells of the reference (two layers, src/Util.cpp:283-438) are replaced by index
// reflection inside the kernels.  The reference's X sweep also updates the ghost rows
// j < 0, j >= N2 (src/HyperbolicSplitSolver.cpp:128-131); those rows are exact mirror images
// of the updated interior rows (mirrored c and mirrored tangential velocity give the same
// fluxes), so the following Y sweep reads them here by reflecting the interior result.
#include <cmath>
#include <mutex>

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
    pdl_enter();
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
    ++ctx->nlaunch, launch_k(ctx->stream, k_tr, 1, RED_THREADS, 0, ctx->nwells, ctx->well_idx, ctx->well_q, c, dt_dev, dt_scale,
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
// Comparisons on the integer pipe.  FP64 compares issue on the FP64 pipe, the bottleneck of
// the transport kernels on GB300; for non-NaN doubles these are exact equivalents (a NaN
// operand still yields a NaN result through the arithmetic around them).
// x > 0: the bit pattern, read as a signed integer, is positive (+0 is 0, negatives are < 0).
__device__ __forceinline__ bool pos(double x) { return __double_as_longlong(x) > 0LL; }
// |a| <= |b|: IEEE magnitudes order like their bit patterns with the sign bit cleared.
__device__ __forceinline__ bool abs_le(double a, double b) {
    return (__double_as_longlong(a) & 0x7fffffffffffffffLL) <= (__double_as_longlong(b) & 0x7fffffffffffffffLL);
}

__device__ __forceinline__ void hancock(double cm, double c0, double cp, double ul, double ur, double kap,
                                        double& sl, double& sr) {
    double a = c0 - cm, b = cp - c0;
    double d = pos(a * b) ? (abs_le(a, b) ? a : b) : 0.0;
    double UR = fma(0.5, d, c0), UL = fma(-0.5, d, c0);
    double df = kap * (ul * UL - ur * UR);
    sl = UL + df;
    sr = UR + df;
}

// WAF intercell flux (times phi) for the split sweeps (hyper_method "waf_split" / "waf"; the
// reference parses these, src/SimParams.cpp:200-208, but ships no source for them).  Toro's
// weighted average flux with the van Leer limiter (Riemann Solvers and Numerical Methods for
// Fluid Dynamics, 3rd ed., ch. 13-14): cr = u dt / (dx phi) = u lam is the Courant number,
// A = 1 - (1 - |cr|) * 2r / (1 + r) for r > 0 (else 1, the upwind flux), r = upwind jump /
// local jump, and F = u ((1 + s A) cL + (1 - s A) cR) / 2 with s = sign(cr).
__device__ __forceinline__ double waf_face(double u, double lam, double cLL, double cL, double cR, double cRR) {
    const double cr = u * lam;
    const double dloc = cR - cL;
    double A = 1.0;
    if (dloc != 0.0) {
        const double dupw = cr >= 0.0 ? cL - cLL : cRR - cR;
        const double r = dupw / dloc;
        if (r > 0.0) A = 1.0 - (1.0 - fabs(cr)) * (2.0 * r / (1.0 + r));
    }
    const double s = cr > 0.0 ? 1.0 : (cr < 0.0 ? -1.0 : 0.0);
    return 0.5 * (1.0 + s * A) * (u * cL) + 0.5 * (1.0 - s * A) * (u * cR);
}

// Reflected (or wrapped) cell index, clamped into [0, n): tile loads may reach further than
// two cells past the boundary on small grids; those values never reach an in-domain output.
template <int BC>
__device__ __forceinline__ int cell_at(int i, int n) {
    int r = BC == IMPEC_BC_PERIODIC ? wrap_cell(i, n) : refl_cell(i, n);
    return r < 0 ? 0 : (r >= n ? n - 1 : r);
}

// Normal face velocity along the sweep direction, ghost faces by odd reflection (Neumann)
// or wrap-around (periodic).
template <int BC>
__device__ __forceinline__ double face_at(const double* __restrict__ u, int f, int n, size_t stride_f, size_t off) {
    if (BC == IMPEC_BC_PERIODIC) {
        int w = wrap_face(f, n);
        w = w < 0 ? 0 : (w > n ? n : w);
        return u[(size_t)w * stride_f + off];
    }
    double s = 1.0;
    int ff = refl_face(f, n, s);
    ff = ff < 0 ? 0 : (ff > n ? n : ff);
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
        Fw = uw * (pos(uw) ? cm : c0);
        Fe = ue * (pos(ue) ? c0 : cp);
        return c0 + lam * (Fw - Fe);
    }
    if (SCHEME == IMPEC_WAFSPLIT) {
        double cmm = C(k - 2), cm = C(k - 1), c0 = C(k), cp = C(k + 1), cpp = C(k + 2);
        Fw = waf_face(uw, lam, cmm, cm, c0, cp);
        Fe = waf_face(ue, lam, cm, c0, cp, cpp);
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
    Fw = uw * (pos(uw) ? srm : sl0);
    Fe = ue * (pos(ue) ? sr0 : slp);
    return c0 + lam * (Fw - Fe);
}

// X sweep: lines along i (stride N2), faces u (N1+1) x N2.
template <int SCHEME, int BC>
__global__ void k_sweep_x(int n1, int n2, const double* __restrict__ cin, const double* __restrict__ cghost,
                          double* __restrict__ cout, const double* __restrict__ u, const double* __restrict__ dt_dev,
                          double dt_scale, double inv_dx_phi) {
    pdl_enter();
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
    pdl_enter();
    int j = blockIdx.x * TBX + threadIdx.x, i = blockIdx.y * TBY + threadIdx.y;
    if (i >= n1 || j >= n2) return;
    const double dt = dt_scale * dt_dev[0];
    const double lam = dt * inv_dy_phi, kap = 0.5 * lam;
    cout[IX(i, j, n2)] = sweep_cell<SCHEME, BC>(cin, nullptr, IX(i, 0, n2), 1, v, IX(i, 0, n2 + 1), 1, j, n2, kap, lam);
}

__global__ void k_average(size_t n, double* __restrict__ c, const double* __restrict__ a, const double* __restrict__ b) {
    pdl_enter();
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        c[k] = 0.5 * (a[k] + b[k]);
}

// ---------------------------------------------------------------- fused symmetric-parallel update
// One CTA owns a TI x TJ tile of the output.  It loads c (2-cell halo), the x-face velocities
// u and the y-face velocities v it needs (ghost values by the reflections above), then
// computes in shared memory  XY = Y(X(c)),  YX = X(Y(c))  and writes (XY + YX)/2, which is
// AdvectSplit's SYMMETRIC_PARALLEL branch (src/HyperbolicSplitSolver.cpp:87-103).  Each
// sweep first computes the two Hancock states of every cell it needs once, then the fluxes
// and updates; the arithmetic per cell is that of sweep_cell, so results are identical.
constexpr int TI = 16, TJ = 32, FUSED_THREADS = 256;
constexpr int CW = TJ + 4;                // row width of c, c1 (j in [j0-2, j0+TJ+2))
constexpr int VW = TJ + 3;                // row width of v faces (fj in [j0-1, j0+TJ+2))
constexpr int HMAX = (TI + 4) * (TJ + 2) > (TI + 2) * (TJ + 4) ? (TI + 4) * (TJ + 2) : (TI + 2) * (TJ + 4);

template <int SCHEME>
__device__ __forceinline__ void states(double cm, double c0, double cp, double ul, double ur, double kap, double& sl,
                                       double& sr) {
    if (SCHEME == IMPEC_UPWINDSPLIT) { sl = sr = c0; return; }
    hancock(cm, c0, cp, ul, ur, kap, sl, sr);
}

template <int SCHEME, int BC>
__global__ void __launch_bounds__(FUSED_THREADS) k_advect_symmetric(int n1, int n2, const double* __restrict__ cin,
                                                                     double* __restrict__ cout,
                                                                     const double* __restrict__ u,
                                                                     const double* __restrict__ v,
                                                                     const double* __restrict__ dt_dev, double inv_dx_phi,
                                                                     double inv_dy_phi) {
    pdl_enter();
    __shared__ double sc[(TI + 4) * CW];   // c, rows i0-2 .. i0+TI+1
    __shared__ double su[(TI + 3) * CW];   // u faces fi in [i0-1, i0+TI+1], cols j0-2 ..
    __shared__ double sv[(TI + 4) * VW];   // v faces, rows i0-2 .., fj in [j0-1, j0+TJ+1]
    __shared__ double s1[TI * CW];         // X(c) on rows i0..i0+TI-1, cols j0-2 ..
    __shared__ double s2[(TI + 4) * TJ];   // Y(c) on rows i0-2 .., cols j0 ..
    __shared__ double sxy[TI * TJ];        // Y(X(c))
    __shared__ double hl[HMAX], hr[HMAX];  // Hancock states at the left / right face of a cell
    const int i0 = blockIdx.y * TI, j0 = blockIdx.x * TJ, t = threadIdx.x;
    const double dt = dt_dev[0];
    const double lx = dt * inv_dx_phi, kx = 0.5 * lx, ly = dt * inv_dy_phi, ky = 0.5 * ly;
    // ---- loads (reflected ghosts) ----
    for (int k = t; k < (TI + 4) * CW; k += FUSED_THREADS) {
        int a = k / CW, b = k % CW;
        sc[k] = cin[IX(cell_at<BC>(i0 - 2 + a, n1), cell_at<BC>(j0 - 2 + b, n2), n2)];
    }
    for (int k = t; k < (TI + 3) * CW; k += FUSED_THREADS) {
        int a = k / CW, b = k % CW;
        su[k] = face_at<BC>(u, i0 - 1 + a, n1, n2, cell_at<BC>(j0 - 2 + b, n2));
    }
    for (int k = t; k < (TI + 4) * VW; k += FUSED_THREADS) {
        int a = k / VW, b = k % VW;
        sv[k] = face_at<BC>(v + IX(cell_at<BC>(i0 - 2 + a, n1), 0, n2 + 1), j0 - 1 + b, n2, 1, 0);
    }
    __syncthreads();
    // ---- XY path, X sweep: cells i in [i0-1, i0+TI], rows b in [0, CW) ----
    for (int k = t; k < (TI + 2) * CW; k += FUSED_THREADS) {
        int a = k / CW, b = k % CW;  // cell i = i0-1+a, c row index a+1
        states<SCHEME>(sc[a * CW + b], sc[(a + 1) * CW + b], sc[(a + 2) * CW + b], su[a * CW + b], su[(a + 1) * CW + b],
                       kx, hl[k], hr[k]);
    }
    __syncthreads();
    for (int k = t; k < TI * CW; k += FUSED_THREADS) {
        int a = k / CW, b = k % CW;  // cell i = i0+a: states at a+1, faces fi = i0+a (su row a+1), i0+a+1
        double uw = su[(a + 1) * CW + b], ue = su[(a + 2) * CW + b];
        double Fw = uw * (pos(uw) ? hr[a * CW + b] : hl[(a + 1) * CW + b]);
        double Fe = ue * (pos(ue) ? hr[(a + 1) * CW + b] : hl[(a + 2) * CW + b]);
        s1[k] = sc[(a + 2) * CW + b] + lx * (Fw - Fe);
    }
    __syncthreads();
    // ---- XY path, Y sweep on s1: cells j in [j0-1, j0+TJ], rows a in [0, TI) ----
    for (int k = t; k < TI * (TJ + 2); k += FUSED_THREADS) {
        int a = k / (TJ + 2), b = k % (TJ + 2);  // cell j = j0-1+b -> s1 col b+1; faces fj = j, j+1 -> sv col b, b+1
        const double* row = s1 + a * CW;
        const double* vr = sv + (a + 2) * VW;
        states<SCHEME>(row[b], row[b + 1], row[b + 2], vr[b], vr[b + 1], ky, hl[k], hr[k]);
    }
    __syncthreads();
    for (int k = t; k < TI * TJ; k += FUSED_THREADS) {
        int a = k / TJ, b = k % TJ;  // cell j = j0+b: states index b+1
        const double* vr = sv + (a + 2) * VW;
        const int h = a * (TJ + 2);
        double vs = vr[b + 1], vn = vr[b + 2];
        double Fs = vs * (pos(vs) ? hr[h + b] : hl[h + b + 1]);
        double Fn = vn * (pos(vn) ? hr[h + b + 1] : hl[h + b + 2]);
        sxy[k] = s1[a * CW + b + 2] + ly * (Fs - Fn);
    }
    __syncthreads();
    // ---- YX path, Y sweep on c: rows a in [0, TI+4) (i = i0-2+a), cells j in [j0-1, j0+TJ] ----
    for (int k = t; k < (TI + 4) * (TJ + 2); k += FUSED_THREADS) {
        int a = k / (TJ + 2), b = k % (TJ + 2);
        const double* row = sc + a * CW;
        const double* vr = sv + a * VW;
        states<SCHEME>(row[b], row[b + 1], row[b + 2], vr[b], vr[b + 1], ky, hl[k], hr[k]);
    }
    __syncthreads();
    for (int k = t; k < (TI + 4) * TJ; k += FUSED_THREADS) {
        int a = k / TJ, b = k % TJ;
        const double* vr = sv + a * VW;
        const int h = a * (TJ + 2);
        double vs = vr[b + 1], vn = vr[b + 2];
        double Fs = vs * (pos(vs) ? hr[h + b] : hl[h + b + 1]);
        double Fn = vn * (pos(vn) ? hr[h + b + 1] : hl[h + b + 2]);
        s2[k] = sc[a * CW + b + 2] + ly * (Fs - Fn);
    }
    __syncthreads();
    // ---- YX path, X sweep on s2: cells i in [i0-1, i0+TI] (s2 rows a+1), cols b in [0, TJ) ----
    for (int k = t; k < (TI + 2) * TJ; k += FUSED_THREADS) {
        int a = k / TJ, b = k % TJ;
        states<SCHEME>(s2[a * TJ + b], s2[(a + 1) * TJ + b], s2[(a + 2) * TJ + b], su[a * CW + b + 2],
                       su[(a + 1) * CW + b + 2], kx, hl[k], hr[k]);
    }
    __syncthreads();
    for (int k = t; k < TI * TJ; k += FUSED_THREADS) {
        int a = k / TJ, b = k % TJ;
        const int gi = i0 + a, gj = j0 + b;
        if (gi >= n1 || gj >= n2) continue;
        double uw = su[(a + 1) * CW + b + 2], ue = su[(a + 2) * CW + b + 2];
        double Fw = uw * (pos(uw) ? hr[a * TJ + b] : hl[(a + 1) * TJ + b]);
        double Fe = ue * (pos(ue) ? hr[(a + 1) * TJ + b] : hl[(a + 2) * TJ + b]);
        double yx = s2[(a + 2) * TJ + b] + lx * (Fw - Fe);
        cout[IX(gi, gj, n2)] = 0.5 * (sxy[k] + yx);
    }
}

// ---------------------------------------------------------------- corner transport upwind
// hyper_method "ctu" (parsed by the reference, src/SimParams.cpp:200-208, no source shipped):
// Colella's unsplit second-order CTU (J. Comput. Phys. 87 (1990) 171-200) on face velocities.
// Each face takes its upwind cell's value extrapolated to the face and the half time level --
// the central slope (unlimited, the recorded order is "2nd order"), the normal Courant
// correction, and half the transverse upwind advection of that cell -- and the interior is
// updated conservatively in one pass.  lx = dt/(dx phi), ly = dt/(dy phi) per unit velocity.
template <int BC>
__global__ void k_ctu(int n1, int n2, const double* __restrict__ cin, double* __restrict__ cout,
                      const double* __restrict__ u, const double* __restrict__ v, const double* __restrict__ dt_dev,
                      double inv_dx_phi, double inv_dy_phi) {
    pdl_enter();
    const int j = blockIdx.x * TBX + threadIdx.x, i = blockIdx.y * TBY + threadIdx.y;
    if (i >= n1 || j >= n2) return;
    const double dt = dt_dev[0], lx = dt * inv_dx_phi, ly = dt * inv_dy_phi;
    auto C = [&](int a, int b) { return cin[IX(cell_at<BC>(a, n1), cell_at<BC>(b, n2), n2)]; };
    // x-face f of row b (normal: odd reflection across x walls; row b: even reflection)
    auto U = [&](int f, int b) { return face_at<BC>(u, f, n1, n2, cell_at<BC>(b, n2)); };
    // y-face f of row a
    auto V = [&](int a, int f) { return face_at<BC>(v + IX(cell_at<BC>(a, n1), 0, n2 + 1), f, n2, 1, 0); };
    auto ty = [&](int a, int b) {  // cell-centred v times its upwind y difference, cell (a, b)
        const double bc = 0.5 * (V(a, b) + V(a, b + 1));
        return bc * (bc >= 0.0 ? C(a, b) - C(a, b - 1) : C(a, b + 1) - C(a, b));
    };
    auto tx = [&](int a, int b) {
        const double ac = 0.5 * (U(a, b) + U(a + 1, b));
        return ac * (ac >= 0.0 ? C(a, b) - C(a - 1, b) : C(a + 1, b) - C(a, b));
    };
    auto Fx = [&](int f) {  // x-face f of row j
        const double vel = U(f, j);
        const int m = vel >= 0.0 ? f - 1 : f;
        const double sx = 0.5 * (C(m + 1, j) - C(m - 1, j));
        const double st = vel >= 0.0 ? C(m, j) + 0.5 * (1.0 - vel * lx) * sx - 0.5 * ly * ty(m, j)
                                     : C(m, j) - 0.5 * (1.0 + vel * lx) * sx - 0.5 * ly * ty(m, j);
        return vel * st;
    };
    auto Fy = [&](int f) {  // y-face f of row i
        const double vel = V(i, f);
        const int m = vel >= 0.0 ? f - 1 : f;
        const double sy = 0.5 * (C(i, m + 1) - C(i, m - 1));
        const double st = vel >= 0.0 ? C(i, m) + 0.5 * (1.0 - vel * ly) * sy - 0.5 * lx * tx(i, m)
                                     : C(i, m) - 0.5 * (1.0 + vel * ly) * sy - 0.5 * lx * tx(i, m);
        return vel * st;
    };
    cout[IX(i, j, n2)] = C(i, j) + lx * (Fx(i) - Fx(i + 1)) + ly * (Fy(j) - Fy(j + 1));
}

static dim3 tgrid(int n1, int n2) { return dim3((n2 + TBX - 1) / TBX, (n1 + TBY - 1) / TBY); }

impec_status advect_x_dev(impec_ctx* ctx, const double* cin, double* cout, const double* u, double dt_scale,
                          const double* dt_dev, const double* cghost) {
    const impec_params& P = ctx->P;
    const double f = 1.0 / (ctx->G.dx * P.porosity);
    dim3 g = tgrid(P.N1, P.N2), b(TBX, TBY);
    ++ctx->nlaunch;
    const bool per = P.bc == IMPEC_BC_PERIODIC;
    if (P.hmtype == IMPEC_MUSCL) {
        if (per) launch_k(ctx->stream, k_sweep_x<IMPEC_MUSCL, IMPEC_BC_PERIODIC>, g, b, 0, P.N1, P.N2, cin, cghost, cout, u, dt_dev, dt_scale, f);
        else launch_k(ctx->stream, k_sweep_x<IMPEC_MUSCL, IMPEC_BC_NEUMANN>, g, b, 0, P.N1, P.N2, cin, cghost, cout, u, dt_dev, dt_scale, f);
    } else if (P.hmtype == IMPEC_WAFSPLIT || P.hmtype == IMPEC_WAF) {
        if (per) launch_k(ctx->stream, k_sweep_x<IMPEC_WAFSPLIT, IMPEC_BC_PERIODIC>, g, b, 0, P.N1, P.N2, cin, cghost, cout, u, dt_dev, dt_scale, f);
        else launch_k(ctx->stream, k_sweep_x<IMPEC_WAFSPLIT, IMPEC_BC_NEUMANN>, g, b, 0, P.N1, P.N2, cin, cghost, cout, u, dt_dev, dt_scale, f);
    } else {
        if (per) launch_k(ctx->stream, k_sweep_x<IMPEC_UPWINDSPLIT, IMPEC_BC_PERIODIC>, g, b, 0, P.N1, P.N2, cin, cghost, cout, u, dt_dev, dt_scale, f);
        else launch_k(ctx->stream, k_sweep_x<IMPEC_UPWINDSPLIT, IMPEC_BC_NEUMANN>, g, b, 0, P.N1, P.N2, cin, cghost, cout, u, dt_dev, dt_scale, f);
    }
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

impec_status advect_y_dev(impec_ctx* ctx, const double* cin, double* cout, const double* v, double dt_scale,
                          const double* dt_dev) {
    const impec_params& P = ctx->P;
    const double f = 1.0 / (ctx->G.dy * P.porosity);
    dim3 g = tgrid(P.N1, P.N2), b(TBX, TBY);
    ++ctx->nlaunch;
    const bool per = P.bc == IMPEC_BC_PERIODIC;
    if (P.hmtype == IMPEC_MUSCL) {
        if (per) launch_k(ctx->stream, k_sweep_y<IMPEC_MUSCL, IMPEC_BC_PERIODIC>, g, b, 0, P.N1, P.N2, cin, cout, v, dt_dev, dt_scale, f);
        else launch_k(ctx->stream, k_sweep_y<IMPEC_MUSCL, IMPEC_BC_NEUMANN>, g, b, 0, P.N1, P.N2, cin, cout, v, dt_dev, dt_scale, f);
    } else if (P.hmtype == IMPEC_WAFSPLIT || P.hmtype == IMPEC_WAF) {
        if (per) launch_k(ctx->stream, k_sweep_y<IMPEC_WAFSPLIT, IMPEC_BC_PERIODIC>, g, b, 0, P.N1, P.N2, cin, cout, v, dt_dev, dt_scale, f);
        else launch_k(ctx->stream, k_sweep_y<IMPEC_WAFSPLIT, IMPEC_BC_NEUMANN>, g, b, 0, P.N1, P.N2, cin, cout, v, dt_dev, dt_scale, f);
    } else {
        if (per) launch_k(ctx->stream, k_sweep_y<IMPEC_UPWINDSPLIT, IMPEC_BC_PERIODIC>, g, b, 0, P.N1, P.N2, cin, cout, v, dt_dev, dt_scale, f);
        else launch_k(ctx->stream, k_sweep_y<IMPEC_UPWINDSPLIT, IMPEC_BC_NEUMANN>, g, b, 0, P.N1, P.N2, cin, cout, v, dt_dev, dt_scale, f);
    }
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

impec_status average_dev(impec_ctx* ctx, double* c, const double* a, const double* b) {
    const size_t n = (size_t)ctx->P.N1 * ctx->P.N2;
    ++ctx->nlaunch, launch_k(ctx->stream, k_average, ctx->num_sms * 4, 256, 0, n, c, a, b);
    IMPEC_LAUNCH_CHECK();
    return IMPEC_OK;
}

// AdvectSplit (src/HyperbolicSplitSolver.cpp:51-106); pfs 0 = X_SWEEP, 1 = Y_SWEEP.
impec_status advect_split_dev(impec_ctx* ctx, double* c, const double* u, const double* v, const double* dt_dev,
                              int* pfs) {
    const impec_params& P = ctx->P;
    const size_t bytes = (size_t)P.N1 * P.N2 * 8;
    double *t1 = ctx->t1, *t2 = ctx->t2, *t3 = ctx->t3;
    if (P.hmtype == IMPEC_CTU) {  // unsplit: one CTU update, c -> t1, then back into c; pfs untouched
        const double fx = 1.0 / (ctx->G.dx * P.porosity), fy = 1.0 / (ctx->G.dy * P.porosity);
        ++ctx->nlaunch;
        if (P.bc == IMPEC_BC_PERIODIC) launch_k(ctx->stream, k_ctu<IMPEC_BC_PERIODIC>, tgrid(P.N1, P.N2), dim3(TBX, TBY), 0, P.N1, P.N2, c, t1, u, v, dt_dev, fx, fy);
        else launch_k(ctx->stream, k_ctu<IMPEC_BC_NEUMANN>, tgrid(P.N1, P.N2), dim3(TBX, TBY), 0, P.N1, P.N2, c, t1, u, v, dt_dev, fx, fy);
        IMPEC_LAUNCH_CHECK();
        IMPEC_CUDA_TRY(cudaMemcpyAsync(c, t1, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        return IMPEC_OK;  // unsplit: the alternating-sweep state stays as it was
    }
    if (P.dim_splitting == IMPEC_SYMMETRIC_PARALLEL && (P.hmtype == IMPEC_WAFSPLIT || P.hmtype == IMPEC_WAF)) {
        // the average of XY and YX through the per-sweep kernels (the fused tile kernel has
        // MUSCL and upwind states only): t2 = Y(X(c)), t1 = X(Y(c)), c = (t2 + t1) / 2
        IMPEC_TRY(advect_x_dev(ctx, c, t1, u, 1.0, dt_dev));
        IMPEC_TRY(advect_y_dev(ctx, t1, t2, v, 1.0, dt_dev));
        IMPEC_TRY(advect_y_dev(ctx, c, t3, v, 1.0, dt_dev));
        IMPEC_TRY(advect_x_dev(ctx, t3, t1, u, 1.0, dt_dev));
        IMPEC_TRY(average_dev(ctx, c, t2, t1));
        *pfs = 0;
        return IMPEC_OK;
    }
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
        default: {  // SYMMETRIC_PARALLEL: one fused pass, c -> t1, then swap into c
            const double fx = 1.0 / (ctx->G.dx * P.porosity), fy = 1.0 / (ctx->G.dy * P.porosity);
            dim3 g((P.N2 + TJ - 1) / TJ, (P.N1 + TI - 1) / TI);
            const bool per = P.bc == IMPEC_BC_PERIODIC;
            ++ctx->nlaunch;
            if (P.hmtype == IMPEC_MUSCL) {
                if (per) launch_k(ctx->stream, k_advect_symmetric<IMPEC_MUSCL, IMPEC_BC_PERIODIC>, g, FUSED_THREADS, 0, P.N1, P.N2, c, t1, u, v, dt_dev, fx, fy);
                else launch_k(ctx->stream, k_advect_symmetric<IMPEC_MUSCL, IMPEC_BC_NEUMANN>, g, FUSED_THREADS, 0, P.N1, P.N2, c, t1, u, v, dt_dev, fx, fy);
            } else {
                if (per) launch_k(ctx->stream, k_advect_symmetric<IMPEC_UPWINDSPLIT, IMPEC_BC_PERIODIC>, g, FUSED_THREADS, 0, P.N1, P.N2, c, t1, u, v, dt_dev, fx, fy);
                else launch_k(ctx->stream, k_advect_symmetric<IMPEC_UPWINDSPLIT, IMPEC_BC_NEUMANN>, g, FUSED_THREADS, 0, P.N1, P.N2, c, t1, u, v, dt_dev, fx, fy);
            }
            IMPEC_LAUNCH_CHECK();
            IMPEC_CUDA_TRY(cudaMemcpyAsync(c, t1, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
            *pfs = 0;
        }
    }
    (void)bytes;
    return IMPEC_OK;
}

}  // namespace impec

// ---------------------------------------------------------------- allocation-free transport step
// For callers that cannot allocate device memory: code running under a host framework that
// owns every device allocation (a fixed memory pool or budget), or a caller that must not
// trigger cudaMalloc's implicit device synchronisation in the middle of its own work.  The
// symmetric-parallel update above needs one field-sized buffer (it cannot update c in place,
// since neighbouring tiles read the old c) and a device copy of dt; here both live in a
// file-scope device array that every GPU loading this library holds until the process exits.
// Nothing in the array has to start at zero: each call writes dt and every cell of the
// updated field before any kernel reads them.
namespace impec {

constexpr size_t NOALLOC_MAX_CELLS = size_t(1) << 20;  // 1,048,576 cells: 8 MiB of FP64
constexpr size_t NOALLOC_FIELD_OFFSET = 32;            // doubles before the field (dt at [0]); 256-byte aligned
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_FIELD_OFFSET + NOALLOC_MAX_CELLS];

// Stores dt in the scratch.  dt travels as a kernel argument, so the value itself is what a
// launch (or a captured launch node) carries; a host-to-device copy would instead carry the
// address of the caller's stack variable.
__global__ void k_noalloc_store_dt(double* __restrict__ dst, double dt) { dst[0] = dt; }

// Device address of g_noalloc_scratch on the current device, looked up once per device (the
// host-side name of the array is only a stand-in, not a device address).  The address is kept
// for the life of the process: after cudaDeviceReset on that device this entry point must not
// be called again.
static impec_status noalloc_scratch(double** out) {
    static std::mutex mu;
    static double* addr[64] = {nullptr};
    int dev = 0;
    IMPEC_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("device ordinal out of range"); return IMPEC_ERR_ARG; }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        IMPEC_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        addr[dev] = static_cast<double*>(p);
    }
    *out = addr[dev];
    return IMPEC_OK;
}

}  // namespace impec

extern "C" impec_status impec_advect_symmetric_noalloc(const impec_params* P, double* c_dev, const double* u_dev,
                                                       const double* v_dev, double dt, void* stream) {
    using namespace impec;
    if (!P || !c_dev || !u_dev || !v_dev) { set_error("null argument"); return IMPEC_ERR_ARG; }
    if (P->N1 < 2 || P->N2 < 2) { set_error("N1 and N2 must be >= 2"); return IMPEC_ERR_ARG; }
    if ((size_t)P->N1 * (size_t)P->N2 > NOALLOC_MAX_CELLS) {
        set_error("impec_advect_symmetric_noalloc: N1*N2 exceeds its static scratch of 1048576 cells; "
                  "use impec_advect_split with a context instead");
        return IMPEC_ERR_ARG;
    }
    if (P->hmtype != IMPEC_MUSCL && P->hmtype != IMPEC_UPWINDSPLIT) { set_error("unknown hmtype"); return IMPEC_ERR_ARG; }
    if (P->bc != IMPEC_BC_NEUMANN && P->bc != IMPEC_BC_PERIODIC) { set_error("unknown bc"); return IMPEC_ERR_ARG; }
    if (P->dim_splitting != IMPEC_SYMMETRIC_PARALLEL) {
        set_error("impec_advect_symmetric_noalloc performs only the symmetric-parallel splitting; "
                  "set dim_splitting to IMPEC_SYMMETRIC_PARALLEL");
        return IMPEC_ERR_ARG;
    }
    if (!(P->porosity > 0) || !(P->x_ub > P->x_lb) || !(P->y_ub > P->y_lb) || !(dt >= 0) || isinf(dt)) {
        set_error("invalid porosity, domain or dt");
        return IMPEC_ERR_ARG;
    }
    double* scratch = nullptr;
    IMPEC_TRY(noalloc_scratch(&scratch));
    cudaStream_t s = (cudaStream_t)stream;
    const int N1 = P->N1, N2 = P->N2;
    const double dx = (P->x_ub - P->x_lb) / N1, dy = (P->y_ub - P->y_lb) / N2;
    const double fx = 1.0 / (dx * P->porosity), fy = 1.0 / (dy * P->porosity);
    double* cnew = scratch + NOALLOC_FIELD_OFFSET;
    launch_k(s, k_noalloc_store_dt, 1, 1, 0, scratch, dt);
    dim3 g((N2 + TJ - 1) / TJ, (N1 + TI - 1) / TI);
    const bool per = P->bc == IMPEC_BC_PERIODIC;
    if (P->hmtype == IMPEC_MUSCL) {
        if (per) launch_k(s, k_advect_symmetric<IMPEC_MUSCL, IMPEC_BC_PERIODIC>, g, FUSED_THREADS, 0, N1, N2, c_dev, cnew, u_dev, v_dev, scratch, fx, fy);
        else launch_k(s, k_advect_symmetric<IMPEC_MUSCL, IMPEC_BC_NEUMANN>, g, FUSED_THREADS, 0, N1, N2, c_dev, cnew, u_dev, v_dev, scratch, fx, fy);
    } else {
        if (per) launch_k(s, k_advect_symmetric<IMPEC_UPWINDSPLIT, IMPEC_BC_PERIODIC>, g, FUSED_THREADS, 0, N1, N2, c_dev, cnew, u_dev, v_dev, scratch, fx, fy);
        else launch_k(s, k_advect_symmetric<IMPEC_UPWINDSPLIT, IMPEC_BC_NEUMANN>, g, FUSED_THREADS, 0, N1, N2, c_dev, cnew, u_dev, v_dev, scratch, fx, fy);
    }
    IMPEC_LAUNCH_CHECK();
    IMPEC_CUDA_TRY(cudaMemcpyAsync(c_dev, cnew, (size_t)N1 * N2 * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return IMPEC_OK;
}
