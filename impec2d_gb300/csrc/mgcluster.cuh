// Cluster V-cycle (included by pressure.cu inside namespace impec).
//
// The coarse levels of one V-cycle (<= 128^2 cells by default) in a single launch of one
// thread-block cluster of up to 16 CTAs.  Each CTA keeps a band of rows of every level in its
// shared memory: for five-point operators the faces, 1/diagonal, diagonal, iterate and
// right-hand side; for nine-point ones (nu < 1) the nine coefficient planes, 1/diagonal,
// iterate and right-hand side, smoothed by four-colour Gauss-Seidel (the arithmetic of
// k_gs4_exp9).  A stencil reads the row above or below its band from the neighbouring CTA's shared
// memory (distributed shared memory), and the phases of the cycle (one colour of a sweep, the
// restriction, the prolongation) are separated by cluster barriers.  The smallest levels
// (<= 256 cells by default) and the dense coarsest solve run on CTA 0 alone, with block
// barriers.  Each cell is updated with the arithmetic of the per-level kernels (k_rb_face5,
// resid / k_restrict, k_prolong, the dense solve of k_coarse_vcycle) in the same order, so the
// cycle gives the same bits as those launches.
//
// Row ownership: level l's rows are cut into bands of rows[l] rows (an even number, so a 2x2
// restriction aggregate never straddles two CTAs); CTA r owns rows [r*rows[l], (r+1)*rows[l]).
// Levels nd .. nl-1 have rows[l] = n1[l]: CTA 0 owns all of them.
//
// Staging: every CTA copies its bands (and CTA 0 the coarsest inverse) with asynchronous
// element copies (cp.async), all in flight at once, and waits for them once.
//
// Every barrier is reached by all threads of all CTAs the same number of times (the counts
// depend only on nd), and no CTA reads another's shared memory after the last barrier.
#pragma once
// Needs <cooperative_groups.h>, included at the top of pressure.cu.

constexpr int CL_MAXL = 10;
constexpr int CL_THREADS = 512;
constexpr int CL_MAX_CTAS = 16;
// shared arrays of a level; a nine-point level keeps its nine planes at CL_TX (plane stride
// rows * n2) and has no CL_TY / CL_DG (the diagonal is plane 0)
enum { CL_TX = 0, CL_TY, CL_ID, CL_DG, CL_X, CL_B };

template <class T>
struct ClusterArgs {
    int kind;  // FACE5 or EXP9 (every level of the cycle)
    int nl;    // levels handled: 0 .. nl-1 (nl-1 is the dense coarsest level)
    int nd;  // levels 0 .. nd-1 are spread over the cluster; nd .. nl-1 live on CTA 0
    int singular, dn;
    int pre, post;  // smoother sweeps before / after the coarse correction
    int zero_color;  // restriction skips cells of this colour (their residual is ~0), or -1
    int rb_skip;     // first pre-smoothing colour from x = 0 (no neighbours); red-only prolongation
    int n1[CL_MAXL], n2[CL_MAXL], rows[CL_MAXL];
    unsigned off[CL_MAXL][6];  // shared-memory offsets (elements of T) of tx, ty, id, dg, x, b
    const T* tx[CL_MAXL];
    const T* ty[CL_MAXL];
    const T* id[CL_MAXL];
    const T* dg[CL_MAXL];
    const T* a9[CL_MAXL];  // nine-point planes (EXP9)
    T* x0;        // iterate of level 0 (global), read at the start and written at the end
    const T* b0;  // right-hand side of level 0 (global)
    const double* dinv;
    unsigned dinv_off;  // byte offset in shared memory of CTA 0's copy of dinv
};

// Pointer to row i of array `arr` of level l, in the shared memory of the CTA that owns it.
template <class T>
__device__ __forceinline__ T* cl_row(const cooperative_groups::cluster_group& cl, T* sm, int rank,
                                     const ClusterArgs<T>& A, int l, int arr, int i, int stride) {
    const int R = A.rows[l];
    const int o = i / R;
    T* p = sm + A.off[l][arr] + (size_t)(i - o * R) * stride;
    return o == rank ? p : cl.map_shared_rank(p, (unsigned)o);
}

// Band of level l owned by `rank`: rows [lo, lo + cnt).
template <class T>
__device__ __forceinline__ void cl_band(const ClusterArgs<T>& A, int l, int rank, int& lo, int& cnt) {
    lo = rank * A.rows[l];
    const int hi = lo + A.rows[l] < A.n1[l] ? lo + A.rows[l] : A.n1[l];
    cnt = hi > lo ? hi - lo : 0;
}

// One colour of a red-black sweep on the band (the arithmetic of k_rb_face5; with zero, the
// first colour of a sweep from x = 0, that of k_rb_zero: x = b * idiag, no neighbour read).
template <class T>
__device__ void cl_sweep(const cooperative_groups::cluster_group& cl, T* sm, int rank, const ClusterArgs<T>& A,
                         int l, int col, bool zero = false) {
    int lo, cnt;
    cl_band(A, l, rank, lo, cnt);
    if (cnt == 0) return;
    const int n1 = A.n1[l], n2 = A.n2[l], half = (n2 + 1) / 2;
    T* x = sm + A.off[l][CL_X];
    const T* b = sm + A.off[l][CL_B];
    const T* tx = sm + A.off[l][CL_TX];
    const T* ty = sm + A.off[l][CL_TY];
    const T* id = sm + A.off[l][CL_ID];
    if (zero) {
        for (int k = threadIdx.x; k < cnt * half; k += blockDim.x) {
            const int li = k / half, i = lo + li, j = 2 * (k - li * half) + ((i + col) & 1);
            if (j < n2) x[li * n2 + j] = b[li * n2 + j] * id[li * n2 + j];
        }
        return;
    }
    const T* xup = lo > 0 ? cl_row(cl, sm, rank, A, l, CL_X, lo - 1, n2) : nullptr;
    const T* xdn = lo + cnt < n1 ? cl_row(cl, sm, rank, A, l, CL_X, lo + cnt, n2) : nullptr;
    for (int k = threadIdx.x; k < cnt * half; k += blockDim.x) {
        const int li = k / half, i = lo + li, j = 2 * (k - li * half) + ((i + col) & 1);
        if (j >= n2) continue;
        const int c = li * n2 + j;
        T s = b[c];
        if (i > 0) s += tx[c] * (li > 0 ? x[c - n2] : xup[j]);
        if (i < n1 - 1) s += tx[c + n2] * (li + 1 < cnt ? x[c + n2] : xdn[j]);
        if (j > 0) s += ty[li * (n2 + 1) + j] * x[c - 1];
        if (j < n2 - 1) s += ty[li * (n2 + 1) + j + 1] * x[c + 1];
        x[c] = s * id[c];
    }
}

// One colour (ci, cj) = (col >> 1, col & 1) of a four-colour Gauss-Seidel sweep of a
// nine-point level on the band: s = b - sum_e a_e x_e over the neighbours in c_off order,
// x = s * idiag (the arithmetic of k_gs4_exp9).  Bands start on even rows, so a band row's
// parity is its global row's.
template <class T>
__device__ void cl_sweep9(const cooperative_groups::cluster_group& cl, T* sm, int rank, const ClusterArgs<T>& A,
                          int l, int col) {
    int lo, cnt;
    cl_band(A, l, rank, lo, cnt);
    if (cnt == 0) return;
    const int n1 = A.n1[l], n2 = A.n2[l], ci = col >> 1, cj = col & 1;
    const size_t ps = (size_t)A.rows[l] * n2;  // plane stride of the staged band
    T* x = sm + A.off[l][CL_X];
    const T* b = sm + A.off[l][CL_B];
    const T* id = sm + A.off[l][CL_ID];
    const T* a9 = sm + A.off[l][CL_TX];
    const T* xup = lo > 0 ? cl_row(cl, sm, rank, A, l, CL_X, lo - 1, n2) : nullptr;
    const T* xdn = lo + cnt < n1 ? cl_row(cl, sm, rank, A, l, CL_X, lo + cnt, n2) : nullptr;
    const int nr = (cnt - ci + 1) / 2, nc = (n2 - cj + 1) / 2;
    for (int k = threadIdx.x; k < nr * nc; k += blockDim.x) {
        const int li = ci + 2 * (k / nc), j = cj + 2 * (k % nc), i = lo + li, c = li * n2 + j;
        T o = 0;
#pragma unroll
        for (int e = 1; e < 9; ++e) {
            const int ii = i + c_off[e][0], jj = j + c_off[e][1];
            if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
            const T xv = ii < lo ? xup[jj] : (ii >= lo + cnt ? xdn[jj] : x[(ii - lo) * n2 + jj]);
            o += a9[e * ps + c] * xv;
        }
        x[c] = (b[c] - o) * id[c];
    }
}

// The s-th colour launch of a smoothing pass (s counts colours over all its sweeps): five-point
// colours alternate 0, 1 (post: 1, 0); nine-point ones run 0..3 (post: 3..0).  zero: the first
// colour of a five-point pass from x = 0.
template <class T>
__device__ void cl_colour(const cooperative_groups::cluster_group& cl, T* sm, int rank, const ClusterArgs<T>& A,
                          int l, int s, bool post, bool zero) {
    if (A.kind == FACE5) cl_sweep(cl, sm, rank, A, l, post ? 1 - (s & 1) : (s & 1), zero);
    else cl_sweep9(cl, sm, rank, A, l, post ? 3 - (s & 3) : (s & 3));
}

// Residual of the band summed over 2x2 aggregates into the coarse right-hand side (owned by
// whichever CTA holds the coarse row); coarse iterate := 0.  The arithmetic of k_restrict.
template <class T>
__device__ void cl_restrict(const cooperative_groups::cluster_group& cl, T* sm, int rank, const ClusterArgs<T>& A,
                            int l) {
    int lo, cnt;
    cl_band(A, l, rank, lo, cnt);
    if (cnt == 0) return;
    const int n1 = A.n1[l], n2 = A.n2[l], c2 = A.n2[l + 1];
    const T* x = sm + A.off[l][CL_X];
    const T* b = sm + A.off[l][CL_B];
    const T* tx = sm + A.off[l][CL_TX];
    const T* ty = sm + A.off[l][CL_TY];
    const T* dg = sm + A.off[l][CL_DG];
    const size_t ps = (size_t)A.rows[l] * n2;  // nine-point plane stride
    const T* xup = lo > 0 ? cl_row(cl, sm, rank, A, l, CL_X, lo - 1, n2) : nullptr;
    const T* xdn = lo + cnt < n1 ? cl_row(cl, sm, rank, A, l, CL_X, lo + cnt, n2) : nullptr;
    const int I0 = lo >> 1, I1 = (lo + cnt + 1) >> 1;
    for (int k = threadIdx.x; k < (I1 - I0) * c2; k += blockDim.x) {
        const int I = I0 + k / c2, J = k % c2;
        T s = 0;
        for (int a = 0; a < 2; ++a)
            for (int bb = 0; bb < 2; ++bb) {
                const int i = 2 * I + a, j = 2 * J + bb;
                if (i >= n1 || j >= n2 || ((i + j) & 1) == A.zero_color) continue;  // as k_restrict
                const int li = i - lo, c = li * n2 + j;
                T r = b[c];
                if (A.kind == FACE5) {
                    if (i > 0) r += tx[c] * (li > 0 ? x[c - n2] : xup[j]);
                    if (i < n1 - 1) r += tx[c + n2] * (li + 1 < cnt ? x[c + n2] : xdn[j]);
                    if (j > 0) r += ty[li * (n2 + 1) + j] * x[c - 1];
                    if (j < n2 - 1) r += ty[li * (n2 + 1) + j + 1] * x[c + 1];
                    s += r - dg[c] * x[c];
                } else {  // as resid() for nine-point operators: r = b - sum a_e x_e - a_0 x
                    for (int e = 1; e < 9; ++e) {
                        const int ii = i + c_off[e][0], jj = j + c_off[e][1];
                        if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
                        const T xv = ii < lo ? xup[jj] : (ii >= lo + cnt ? xdn[jj] : x[(ii - lo) * n2 + jj]);
                        r -= tx[e * ps + c] * xv;
                    }
                    s += r - tx[c] * x[c];
                }
            }
        cl_row(cl, sm, rank, A, l + 1, CL_B, I, c2)[J] = s;
        cl_row(cl, sm, rank, A, l + 1, CL_X, I, c2)[J] = T(0);
    }
}

// Bilinear prolongation of the coarse iterate added to the band (the arithmetic of k_prolong;
// with A.rb_skip on the red cells only, as k_prolong_rb: the post-smoothing that follows
// starts with the black colour and overwrites every black cell unread).
template <class T>
__device__ void cl_prolong(const cooperative_groups::cluster_group& cl, T* sm, int rank, const ClusterArgs<T>& A,
                           int l) {
    int lo, cnt;
    cl_band(A, l, rank, lo, cnt);
    if (cnt == 0) return;
    const int n2 = A.n2[l], c1 = A.n1[l + 1], c2 = A.n2[l + 1];
    T* x = sm + A.off[l][CL_X];
    for (int k = threadIdx.x; k < cnt * n2; k += blockDim.x) {
        const int li = k / n2, j = k - li * n2, i = lo + li;
        if (A.rb_skip && ((i + j) & 1)) continue;
        const int I = i >> 1, J = j >> 1;
        int I2 = (i & 1) ? I + 1 : I - 1, J2 = (j & 1) ? J + 1 : J - 1;
        if (I2 < 0 || I2 >= c1) I2 = I;
        if (J2 < 0 || J2 >= c2) J2 = J;
        const T* r1 = cl_row(cl, sm, rank, A, l + 1, CL_X, I, c2);
        const T* r2 = cl_row(cl, sm, rank, A, l + 1, CL_X, I2, c2);
        T v = x[k];
        v += T(0.5625) * r1[J];
        v += T(0.1875) * r2[J];
        v += T(0.1875) * r1[J2];
        v += T(0.0625) * r2[J2];
        x[k] = v;
    }
}

template <class T>
__global__ void __launch_bounds__(CL_THREADS) k_cluster_vcycle(const __grid_constant__ ClusterArgs<T> A) {
    pdl_enter();
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char cl_raw[];
    T* sm = reinterpret_cast<T*>(cl_raw);
    const int rank = (int)cl.block_rank();

    // stage this CTA's bands (operators of every level; iterate and rhs of level 0)
    for (int l = 0; l < A.nl; ++l) {
        int lo, cnt;
        cl_band(A, l, rank, lo, cnt);
        if (cnt == 0) continue;
        const int n2 = A.n2[l];
        T* tx = sm + A.off[l][CL_TX];
        T* ty = sm + A.off[l][CL_TY];
        T* id = sm + A.off[l][CL_ID];
        T* dg = sm + A.off[l][CL_DG];
        if (A.kind == FACE5) {
            for (int k = threadIdx.x; k < (cnt + 1) * n2; k += blockDim.x)
                stage_async(tx + k, A.tx[l] + (size_t)lo * n2 + k);
            for (int k = threadIdx.x; k < cnt * (n2 + 1); k += blockDim.x)
                stage_async(ty + k, A.ty[l] + (size_t)lo * (n2 + 1) + k);
            for (int k = threadIdx.x; k < cnt * n2; k += blockDim.x) {
                stage_async(id + k, A.id[l] + (size_t)lo * n2 + k);
                stage_async(dg + k, A.dg[l] + (size_t)lo * n2 + k);
            }
        } else if (l + 1 < A.nl) {  // nine planes and 1/diagonal (the dense level needs neither)
            const size_t ps = (size_t)A.rows[l] * n2, n = (size_t)A.n1[l] * n2;
            for (int e = 0; e < 9; ++e)
                for (int k = threadIdx.x; k < cnt * n2; k += blockDim.x)
                    stage_async(tx + e * ps + k, A.a9[l] + e * n + (size_t)lo * n2 + k);
            for (int k = threadIdx.x; k < cnt * n2; k += blockDim.x) stage_async(id + k, A.id[l] + (size_t)lo * n2 + k);
        }
        if (l == 0) {
            T* x = sm + A.off[0][CL_X];
            T* b = sm + A.off[0][CL_B];
            for (int k = threadIdx.x; k < cnt * n2; k += blockDim.x) {
                stage_async(x + k, A.x0 + (size_t)lo * n2 + k);
                stage_async(b + k, A.b0 + (size_t)lo * n2 + k);
            }
        }
    }
    if (rank == 0) {  // the dense inverse of the coarsest level
        double* dinv = reinterpret_cast<double*>(cl_raw + A.dinv_off);
        for (int k = threadIdx.x; k < A.dn * A.dn; k += blockDim.x) stage_async(dinv + k, A.dinv + k);
    }
    stage_wait();
    cl.sync();
    // down: levels spread over the cluster
    const int ncol = A.kind == FACE5 ? 2 : 4;
    for (int l = 0; l < A.nd; ++l) {
        for (int s = 0; s < ncol * A.pre; ++s) {
            cl_colour(cl, sm, rank, A, l, s, false, A.rb_skip && s == 0 && l > 0);
            cl.sync();
        }
        cl_restrict(cl, sm, rank, A, l);
        cl.sync();
    }
    // the small levels and the dense solve on CTA 0
    if (rank == 0) {
        for (int l = A.nd; l < A.nl - 1; ++l) {
            for (int s = 0; s < ncol * A.pre; ++s) {
                cl_colour(cl, sm, 0, A, l, s, false, A.rb_skip && s == 0 && l > 0);
                __syncthreads();
            }
            cl_restrict(cl, sm, 0, A, l);
            __syncthreads();
        }
        const double* dinv = reinterpret_cast<const double*>(cl_raw + A.dinv_off);
        const int L = A.nl - 1;
        dense_coarse_apply<T>(A.dn, dinv, sm + A.off[L][CL_B], sm + A.off[L][CL_X], A.singular);
        for (int l = A.nl - 2; l >= A.nd; --l) {
            cl_prolong(cl, sm, 0, A, l);
            __syncthreads();
            for (int s = 0; s < ncol * A.post; ++s) {
                cl_colour(cl, sm, 0, A, l, s, true, false);
                __syncthreads();
            }
        }
    }
    cl.sync();
    // up: levels spread over the cluster
    for (int l = A.nd - 1; l >= 0; --l) {
        cl_prolong(cl, sm, rank, A, l);
        cl.sync();
        for (int s = 0; s < ncol * A.post; ++s) {
            cl_colour(cl, sm, rank, A, l, s, true, false);
            cl.sync();
        }
    }
    // level-0 band back to global (local shared memory only: no CTA reads a peer after the
    // last barrier)
    int lo, cnt;
    cl_band(A, 0, rank, lo, cnt);
    const T* x = sm + A.off[0][CL_X];
    for (int k = threadIdx.x; k < cnt * A.n2[0]; k += blockDim.x) A.x0[(size_t)lo * A.n2[0] + k] = x[k];
}
