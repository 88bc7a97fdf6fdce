// Projection of a parallel-orientation field onto the diagonal grid, for output:
// Impec2DSolver::Project + ParallelProjector (src/Impec2DSolver.cpp:690-716,
// src/ParallelProjector.cpp:51-199).
//
// The diagonal grid has d_N1 x d_N2 cells of size (x_ub-x_lb)/(sqrt 2 d_N1) x
// (y_ub-y_lb)/(sqrt 2 d_N2).  Each cell centre is rotated by -45 degrees into the parallel
// grid's frame (|y| by the configuration's mirror symmetry) and the parallel field is
// interpolated bilinearly from the four cells around floor(x / L * N).  The reference reads
// one ghost ring of the parallel array there; the ghosts are the Neumann mirror of the
// interior (index reflection).  Every operation is the reference's, in its order, with
// correctly rounded intrinsics and no contraction, so the values are bit-identical to the
// oracle's restatement.
#include <cmath>

#include "internal.cuh"

namespace impec {

struct ProjArgs {
    int pN1, pN2, dN1, dN2;
    double x_lb, y_lb, Lx, Ly;  // Lx = x_ub - x_lb, Ly = y_ub - y_lb
    double p_dx, p_dy, d_dx, d_dy;
    double ca, sa;  // cos and sin of the rotation angle -pi/4, as the host's libm gives them
};

__device__ __forceinline__ double proj_centred(double lb, double dx, int idx) {
    return __dadd_rn(lb, __dmul_rn(__dadd_rn((double)idx, 0.5), dx));
}

// Value at parallel cell (i, j), ghost ring by reflection.  Indices beyond one mirror (only
// possible for domains not starting at the origin) are clamped into the array.
__device__ __forceinline__ double proj_at(const ProjArgs& A, const double* __restrict__ f, int i, int j) {
    i = min(max(refl_cell(i, A.pN1), 0), A.pN1 - 1);
    j = min(max(refl_cell(j, A.pN2), 0), A.pN2 - 1);
    return f[(size_t)i * A.pN2 + j];
}

__global__ void k_project_diagonal(ProjArgs A, const double* __restrict__ f, double* __restrict__ out) {
    pdl_enter();
    const int j = blockIdx.x * 32 + threadIdx.x, i = blockIdx.y * 8 + threadIdx.y;
    if (i >= A.dN1 || j >= A.dN2) return;
    // FillDiagonal: cell centre of the diagonal grid, DiagonalToParallel
    const double x = proj_centred(A.x_lb, A.d_dx, i), y = proj_centred(A.y_lb, A.d_dy, j);
    const double px = __dsub_rn(__dmul_rn(A.ca, x), __dmul_rn(A.sa, y));
    const double py = __dadd_rn(__dmul_rn(A.sa, x), __dmul_rn(A.ca, y));
    // GetFromParallel
    const double X = px, Y = fabs(py);
    const int x00 = (int)fmin(fmax(floor(__dmul_rn(__ddiv_rn(X, A.Lx), (double)A.pN1)), -2.0 * A.pN1), 2.0 * A.pN1);
    const int y00 = (int)fmin(fmax(floor(__dmul_rn(__ddiv_rn(Y, A.Ly), (double)A.pN2)), -2.0 * A.pN2), 2.0 * A.pN2);
    const int x11 = x00 + 1, y11 = y00 + 1;
    const double cx0 = proj_centred(A.x_lb, A.p_dx, x00), cx1 = proj_centred(A.x_lb, A.p_dx, x11);
    const double cy0 = proj_centred(A.y_lb, A.p_dy, y00), cy1 = proj_centred(A.y_lb, A.p_dy, y11);
    const double w = __ddiv_rn(1.0, __dmul_rn(__dsub_rn(cx1, cx0), __dsub_rn(cy1, cy0)));
    const double t00 = __dmul_rn(__dmul_rn(__dmul_rn(w, __dsub_rn(cx1, X)), __dsub_rn(cy1, Y)), proj_at(A, f, x00, y00));
    const double t10 = __dmul_rn(__dmul_rn(__dmul_rn(w, __dsub_rn(X, cx0)), __dsub_rn(cy1, Y)), proj_at(A, f, x11, y00));
    const double t01 = __dmul_rn(__dmul_rn(__dmul_rn(w, __dsub_rn(cx1, X)), __dsub_rn(Y, cy0)), proj_at(A, f, x00, y11));
    const double t11 = __dmul_rn(__dmul_rn(__dmul_rn(w, __dsub_rn(X, cx0)), __dsub_rn(Y, cy0)), proj_at(A, f, x11, y11));
    out[(size_t)i * A.dN2 + j] = __dadd_rn(__dadd_rn(__dadd_rn(t00, t10), t01), t11);
}

}  // namespace impec

using namespace impec;

extern "C" impec_status impec_project_diagonal(impec_ctx* ctx, int field, double* out_dev, int d_N1, int d_N2) {
    if (!ctx || !out_dev || d_N1 < 1 || d_N2 < 1 || (field != 0 && field != 1)) {
        set_error("impec_project_diagonal: bad argument");
        return IMPEC_ERR_ARG;
    }
    const impec_params& P = ctx->P;
    ProjArgs A;
    A.pN1 = P.N1;
    A.pN2 = P.N2;
    A.dN1 = d_N1;
    A.dN2 = d_N2;
    A.x_lb = P.x_lb;
    A.y_lb = P.y_lb;
    A.Lx = P.x_ub - P.x_lb;
    A.Ly = P.y_ub - P.y_lb;
    A.p_dx = (P.x_ub - P.x_lb) / (double)P.N1;
    A.p_dy = (P.y_ub - P.y_lb) / (double)P.N2;
    A.d_dx = (P.x_ub - P.x_lb) / (std::sqrt(2.) * d_N1);
    A.d_dy = (P.y_ub - P.y_lb) / (std::sqrt(2.) * d_N2);
    const double angle = -M_PI / 4.;
    A.ca = std::cos(angle);
    A.sa = std::sin(angle);
    dim3 g((d_N2 + 31) / 32, (d_N1 + 7) / 8);
    ++ctx->nlaunch;
    IMPEC_CUDA_TRY(launch_k(ctx->stream, k_project_diagonal, g, dim3(32, 8), 0, A, field == 0 ? ctx->c : ctx->p, out_dev));
    return IMPEC_OK;
}

extern "C" impec_status impec_project_diagonal_download(impec_ctx* ctx, int field, double* out_host, int d_N1,
                                                        int d_N2) {
    if (!ctx || !out_host) {
        set_error("impec_project_diagonal_download: null argument");
        return IMPEC_ERR_ARG;
    }
    if ((size_t)d_N1 * d_N2 > (size_t)ctx->P.N1 * ctx->P.N2) {
        set_error("impec_project_diagonal_download: the diagonal grid is larger than the parallel grid");
        return IMPEC_ERR_ARG;
    }
    IMPEC_TRY(impec_project_diagonal(ctx, field, ctx->t1, d_N1, d_N2));  // t1: transport scratch, free between steps
    IMPEC_CUDA_TRY(cudaMemcpyAsync(out_host, ctx->t1, sizeof(double) * d_N1 * d_N2, cudaMemcpyDeviceToHost, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}
