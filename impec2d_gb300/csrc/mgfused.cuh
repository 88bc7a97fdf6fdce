// Fused multigrid kernels (included by pressure.cu).
//
// 1. k_coarse_vcycle: the whole V-cycle of the coarse levels (<= 32^2 cells in FP64, <= 64^2 in
//    FP32) in one CTA, operators and iterates in shared memory, coarsest level by the dense
//    FP64 inverse.  Replaces ~10 launches per coarse level.
// 2. k_level_pre / k_level_post: on an intermediate five-point level, two red-black
//    Gauss-Seidel sweeps fused with the residual and the 2x2 restriction (pre), and the
//    bilinear prolongation fused with two sweeps (post).  Each CTA updates its tile plus a
//    shrinking halo (temporal blocking): red/black colours follow the global indices and
//    faces outside the grid are zero, so the result equals the unfused kernels bit for bit.
#pragma once
// Included inside namespace impec of pressure.cu (uses its IX, c_off and Level definitions).

constexpr int MGC_MAXL = 8;

template <class T>
struct CoarseArgs {
    int nl, singular, dn;
    int pre, post;  // smoother sweeps before / after the coarse correction
    int n1[MGC_MAXL], n2[MGC_MAXL];
    const T* tx[MGC_MAXL];
    const T* ty[MGC_MAXL];
    const T* a9[MGC_MAXL];
    const T* id[MGC_MAXL];
    const T* dg[MGC_MAXL];  // diagonals (FACE5; EXP9 uses plane 0 of a9)
    T* x0;           // iterate of the first handled level (global)
    const T* b0;     // its right-hand side (global)
    const double* dinv;
};

template <class T, int KIND>
__device__ void cv_smooth(int n1, int n2, const T* tx, const T* ty, const T* a9, const T* id, const T* b, T* x,
                          bool reverse, int sweeps) {
    const int n = n1 * n2;
    for (int s = 0; s < sweeps; ++s) {
        const int ncol = KIND == FACE5 ? 2 : 4;
        for (int cc = 0; cc < ncol; ++cc) {
            const int col = reverse ? ncol - 1 - cc : cc;
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                const int i = k / n2, j = k % n2;
                if (KIND == FACE5) {
                    if (((i + j) & 1) != col) continue;
                    T sm = b[k];
                    if (i > 0) sm += tx[IX(i, j, n2)] * x[k - n2];
                    if (i < n1 - 1) sm += tx[IX(i + 1, j, n2)] * x[k + n2];
                    if (j > 0) sm += ty[IX(i, j, n2 + 1)] * x[k - 1];
                    if (j < n2 - 1) sm += ty[IX(i, j + 1, n2 + 1)] * x[k + 1];
                    x[k] = sm * id[k];
                } else {
                    if ((((i & 1) << 1) | (j & 1)) != col) continue;
                    T sm = b[k];
                    for (int e = 1; e < 9; ++e) {
                        int ii = i + c_off[e][0], jj = j + c_off[e][1];
                        if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
                        sm -= a9[e * n + k] * x[IX(ii, jj, n2)];
                    }
                    x[k] = sm * id[k];
                }
            }
            __syncthreads();
        }
    }
}

// Same arithmetic as resid() of the level kernels: s = b + sum t * x_nb (or b - sum a_e * x_nb),
// r = s - diag * x.
template <class T, int KIND>
__device__ __forceinline__ T cv_resid(int i, int j, int n1, int n2, const T* tx, const T* ty, const T* a9, const T* dg,
                                      const T* b, const T* x) {
    const int k = IX(i, j, n2);
    T s = b[k];
    if (KIND == FACE5) {
        if (i > 0) s += tx[k] * x[k - n2];
        if (i < n1 - 1) s += tx[k + n2] * x[k + n2];
        if (j > 0) s += ty[IX(i, j, n2 + 1)] * x[k - 1];
        if (j < n2 - 1) s += ty[IX(i, j + 1, n2 + 1)] * x[k + 1];
        return s - dg[k] * x[k];
    }
    const int n = n1 * n2;
    for (int e = 1; e < 9; ++e) {
        int ii = i + c_off[e][0], jj = j + c_off[e][1];
        if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
        s -= a9[e * n + k] * x[IX(ii, jj, n2)];
    }
    return s - a9[k] * x[k];
}

template <class T, int KIND>
__global__ void __launch_bounds__(1024) k_coarse_vcycle(CoarseArgs<T> A) {
    pdl_enter();
    extern __shared__ __align__(16) unsigned char cv_raw[];
    T* sm = reinterpret_cast<T*>(cv_raw);
    T *tx[MGC_MAXL], *ty[MGC_MAXL], *a9[MGC_MAXL], *id[MGC_MAXL], *dg[MGC_MAXL], *x[MGC_MAXL], *b[MGC_MAXL];
    size_t off = 0;
    for (int l = 0; l < A.nl; ++l) {
        const int n1 = A.n1[l], n2 = A.n2[l], n = n1 * n2;
        tx[l] = ty[l] = a9[l] = dg[l] = nullptr;
        if (KIND == FACE5) {
            tx[l] = sm + off; off += (size_t)(n1 + 1) * n2;
            ty[l] = sm + off; off += (size_t)n1 * (n2 + 1);
            dg[l] = sm + off; off += n;
        } else {
            a9[l] = sm + off; off += (size_t)9 * n;
        }
        id[l] = sm + off; off += n;
        x[l] = sm + off; off += n;
        b[l] = sm + off; off += n;
    }
    for (int l = 0; l < A.nl; ++l) {
        const int n1 = A.n1[l], n2 = A.n2[l], n = n1 * n2;
        if (KIND == FACE5) {
            for (int k = threadIdx.x; k < (n1 + 1) * n2; k += blockDim.x) tx[l][k] = A.tx[l][k];
            for (int k = threadIdx.x; k < n1 * (n2 + 1); k += blockDim.x) ty[l][k] = A.ty[l][k];
            for (int k = threadIdx.x; k < n; k += blockDim.x) dg[l][k] = A.dg[l][k];
        } else {
            for (int k = threadIdx.x; k < 9 * n; k += blockDim.x) a9[l][k] = A.a9[l][k];
        }
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            id[l][k] = A.id[l][k];
            x[l][k] = l == 0 ? A.x0[k] : T(0);
            b[l][k] = l == 0 ? A.b0[k] : T(0);
        }
    }
    __syncthreads();
    const int L = A.nl - 1;  // dense level
    for (int l = 0; l < L; ++l) {
        const int n1 = A.n1[l], n2 = A.n2[l], c1 = A.n1[l + 1], c2 = A.n2[l + 1];
        cv_smooth<T, KIND>(n1, n2, tx[l], ty[l], a9[l], id[l], b[l], x[l], false, A.pre);
        for (int K = threadIdx.x; K < c1 * c2; K += blockDim.x) {
            const int I = K / c2, J = K % c2;
            T s = 0;
            for (int a = 0; a < 2; ++a)
                for (int bb = 0; bb < 2; ++bb) {
                    int i = 2 * I + a, j = 2 * J + bb;
                    if (i < n1 && j < n2) s += cv_resid<T, KIND>(i, j, n1, n2, tx[l], ty[l], a9[l], dg[l], b[l], x[l]);
                }
            b[l + 1][K] = s;
            x[l + 1][K] = 0;
        }
        __syncthreads();
    }
    {  // coarsest: x = Dinv b (FP64), b(0) := 0 and mean removal for the singular system
        __shared__ double red[32];
        const int n = A.dn;
        double v = 0;
        if ((int)threadIdx.x < n) {
            double s = 0;
            for (int c = 0; c < n; ++c) {
                double bc = (A.singular && c == 0) ? 0.0 : (double)b[L][c];
                s += A.dinv[(size_t)threadIdx.x * n + c] * bc;
            }
            v = s;
        }
        double m = 0;
        if (A.singular) {
            double w = v;
            for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = w;
            __syncthreads();
            if (threadIdx.x == 0) {
                double t = 0;
                for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
                red[0] = t / n;
            }
            __syncthreads();
            m = red[0];
        }
        if ((int)threadIdx.x < n) x[L][threadIdx.x] = (T)(v - m);
        __syncthreads();
    }
    for (int l = L - 1; l >= 0; --l) {
        const int n1 = A.n1[l], n2 = A.n2[l], c1 = A.n1[l + 1], c2 = A.n2[l + 1];
        for (int k = threadIdx.x; k < n1 * n2; k += blockDim.x) {
            const int i = k / n2, j = k % n2;
            int I = i >> 1, J = j >> 1;
            int I2 = (i & 1) ? I + 1 : I - 1, J2 = (j & 1) ? J + 1 : J - 1;
            if (I2 < 0 || I2 >= c1) I2 = I;
            if (J2 < 0 || J2 >= c2) J2 = J;
            const T* xc = x[l + 1];
            T v = x[l][k];
            v += T(0.5625) * xc[IX(I, J, c2)];
            v += T(0.1875) * xc[IX(I2, J, c2)];
            v += T(0.1875) * xc[IX(I, J2, c2)];
            v += T(0.0625) * xc[IX(I2, J2, c2)];
            x[l][k] = v;
        }
        __syncthreads();
        cv_smooth<T, KIND>(n1, n2, tx[l], ty[l], a9[l], id[l], b[l], x[l], true, A.post);
    }
    const int n0 = A.n1[0] * A.n2[0];
    for (int k = threadIdx.x; k < n0; k += blockDim.x) A.x0[k] = x[0][k];
}

// ---------------------------------------------------------------- temporally blocked levels
constexpr int TB = 32;           // output tile edge
constexpr int TBH_PRE = 5;       // 4 half sweeps + residual
constexpr int TBH_POST = 4;      // 4 half sweeps
constexpr int TBT = 256;         // threads

// Loads x, b, idiag over the region [i0-H, i0+TB+H) x [j0-H, j0+TB+H) and the faces around it;
// cells and faces outside the grid become zero.
template <class T, int H>
__device__ __forceinline__ void tb_load(int n1, int n2, int i0, int j0, const T* __restrict__ gtx,
                                        const T* __restrict__ gty, const T* __restrict__ gid,
                                        const T* __restrict__ gb, const T* __restrict__ gx, T* x, T* b, T* id, T* tx,
                                        T* ty) {
    constexpr int R = TB + 2 * H;
    for (int k = threadIdx.x; k < R * R; k += TBT) {
        const int a = k / R, c = k % R, gi = i0 - H + a, gj = j0 - H + c;
        const bool in = gi >= 0 && gi < n1 && gj >= 0 && gj < n2;
        x[k] = in ? gx[IX(gi, gj, n2)] : T(0);
        b[k] = in ? gb[IX(gi, gj, n2)] : T(0);
        id[k] = in ? gid[IX(gi, gj, n2)] : T(0);
    }
    for (int k = threadIdx.x; k < (R + 1) * R; k += TBT) {  // tx: faces fi in [i0-H, i0+TB+H], cols
        const int a = k / R, c = k % R, fi = i0 - H + a, gj = j0 - H + c;
        tx[k] = (fi >= 0 && fi <= n1 && gj >= 0 && gj < n2) ? gtx[IX(fi, gj, n2)] : T(0);
    }
    for (int k = threadIdx.x; k < R * (R + 1); k += TBT) {  // ty: rows, faces fj in [j0-H, j0+TB+H]
        const int a = k / (R + 1), c = k % (R + 1), gi = i0 - H + a, fj = j0 - H + c;
        ty[k] = (gi >= 0 && gi < n1 && fj >= 0 && fj <= n2) ? gty[IX(gi, fj, n2 + 1)] : T(0);
    }
}

// Half sweep of colour col on local cells [lo, hi)^2 of a region of edge R.
template <class T, int R>
__device__ __forceinline__ void tb_half(int n1, int n2, int i0, int j0, int H, int lo, int hi, int col, const T* b,
                                        const T* id, const T* tx, const T* ty, T* x) {
    const int w = hi - lo;
    for (int k = threadIdx.x; k < w * w; k += TBT) {
        const int a = lo + k / w, c = lo + k % w, gi = i0 - H + a, gj = j0 - H + c;
        if (((gi + gj) & 1) != col) continue;
        if (gi < 0 || gi >= n1 || gj < 0 || gj >= n2) continue;
        const int q = a * R + c;
        T s = b[q];
        if (gi > 0) s += tx[a * R + c] * x[q - R];
        if (gi < n1 - 1) s += tx[(a + 1) * R + c] * x[q + R];
        if (gj > 0) s += ty[a * (R + 1) + c] * x[q - 1];
        if (gj < n2 - 1) s += ty[a * (R + 1) + c + 1] * x[q + 1];
        x[q] = s * id[q];
    }
    __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(TBT) k_level_pre(int n1, int n2, const T* __restrict__ gtx, const T* __restrict__ gty,
                                                   const T* __restrict__ gid, const T* __restrict__ gb,
                                                   T* __restrict__ gx, int c2, T* __restrict__ bc,
                                                   T* __restrict__ xc, int nc1) {
    pdl_enter();
    constexpr int H = TBH_PRE, R = TB + 2 * H;
    extern __shared__ __align__(16) unsigned char tb_raw[];
    T* x = reinterpret_cast<T*>(tb_raw);
    T* b = x + R * R;
    T* id = b + R * R;
    T* tx = id + R * R;
    T* ty = tx + (R + 1) * R;
    const int i0 = blockIdx.y * TB, j0 = blockIdx.x * TB;
    tb_load<T, H>(n1, n2, i0, j0, gtx, gty, gid, gb, gx, x, b, id, tx, ty);
    __syncthreads();
    for (int s = 0; s < 4; ++s) tb_half<T, R>(n1, n2, i0, j0, H, s + 1, R - s - 1, s & 1, b, id, tx, ty, x);
    // residual on the tile (local [H, H+TB)), summed over 2x2 aggregates
    for (int K = threadIdx.x; K < (TB / 2) * (TB / 2); K += TBT) {
        const int I = (i0 >> 1) + K / (TB / 2), J = (j0 >> 1) + K % (TB / 2);
        if (I >= nc1 || J >= c2) continue;
        T s = 0;
        for (int a = 0; a < 2; ++a)
            for (int bb = 0; bb < 2; ++bb) {
                const int gi = 2 * I + a, gj = 2 * J + bb;
                if (gi >= n1 || gj >= n2) continue;
                const int la = gi - i0 + H, lc = gj - j0 + H, q = la * R + lc;
                T tw = tx[la * R + lc], te = tx[(la + 1) * R + lc], ts = ty[la * (R + 1) + lc], tn = ty[la * (R + 1) + lc + 1];
                T o = 0;
                if (gi > 0) o += tw * x[q - R];
                if (gi < n1 - 1) o += te * x[q + R];
                if (gj > 0) o += ts * x[q - 1];
                if (gj < n2 - 1) o += tn * x[q + 1];
                T diag = tw + te + ts + tn;
                s += b[q] - (diag * x[q] - o);
            }
        bc[IX(I, J, c2)] = s;
        xc[IX(I, J, c2)] = 0;
    }
    for (int k = threadIdx.x; k < TB * TB; k += TBT) {
        const int gi = i0 + k / TB, gj = j0 + k % TB;
        if (gi < n1 && gj < n2) gx[IX(gi, gj, n2)] = x[(k / TB + H) * R + (k % TB + H)];
    }
}

template <class T>
__global__ void __launch_bounds__(TBT) k_level_post(int n1, int n2, const T* __restrict__ gtx,
                                                    const T* __restrict__ gty, const T* __restrict__ gid,
                                                    const T* __restrict__ gb, T* __restrict__ gx, int c1, int c2,
                                                    const T* __restrict__ xc) {
    pdl_enter();
    constexpr int H = TBH_POST, R = TB + 2 * H;
    extern __shared__ __align__(16) unsigned char tb_raw[];
    T* x = reinterpret_cast<T*>(tb_raw);
    T* b = x + R * R;
    T* id = b + R * R;
    T* tx = id + R * R;
    T* ty = tx + (R + 1) * R;
    const int i0 = blockIdx.y * TB, j0 = blockIdx.x * TB;
    tb_load<T, H>(n1, n2, i0, j0, gtx, gty, gid, gb, gx, x, b, id, tx, ty);
    __syncthreads();
    for (int k = threadIdx.x; k < R * R; k += TBT) {  // bilinear prolongation on the region
        const int gi = i0 - H + k / R, gj = j0 - H + k % R;
        if (gi < 0 || gi >= n1 || gj < 0 || gj >= n2) continue;
        int I = gi >> 1, J = gj >> 1;
        int I2 = (gi & 1) ? I + 1 : I - 1, J2 = (gj & 1) ? J + 1 : J - 1;
        if (I2 < 0 || I2 >= c1) I2 = I;
        if (J2 < 0 || J2 >= c2) J2 = J;
        T e = T(0.5625) * xc[IX(I, J, c2)] + T(0.1875) * xc[IX(I2, J, c2)] + T(0.1875) * xc[IX(I, J2, c2)] +
              T(0.0625) * xc[IX(I2, J2, c2)];
        x[k] += e;
    }
    __syncthreads();
    for (int s = 0; s < 4; ++s) tb_half<T, R>(n1, n2, i0, j0, H, s + 1, R - s - 1, 1 - (s & 1), b, id, tx, ty, x);
    for (int k = threadIdx.x; k < TB * TB; k += TBT) {
        const int gi = i0 + k / TB, gj = j0 + k % TB;
        if (gi < n1 && gj < n2) gx[IX(gi, gj, n2)] = x[(k / TB + H) * R + (k % TB + H)];
    }
}

template <class T, int H>
constexpr size_t tb_smem() {
    return sizeof(T) * (size_t)(3 * (TB + 2 * H) * (TB + 2 * H) + 2 * (TB + 2 * H + 1) * (TB + 2 * H));
}

