// Single-CTA coarse V-cycle (included by pressure.cu).
//
// k_coarse_vcycle: the whole V-cycle of the coarse levels (<= 32^2 cells in FP64, <= 64^2 in
// FP32) in one CTA, operators and iterates in shared memory, coarsest level by the dense FP64
// inverse.  Replaces ~10 launches per coarse level.
#pragma once
// Included inside namespace impec of pressure.cu (uses its IX, c_off and Level definitions).

constexpr int MGC_MAXL = 8;

// Coarsest-level solve x = Dinv b' in FP64 (n <= 64), b' = b with b(0) := 0 for the singular
// system (whose Dinv, from k_dense_invert, already removes the mean of the result).  Every
// thread of the block takes part (the count of loop trips and shuffles is the same for all):
// row r is summed by the 8 lanes of one lane group, lane g over the columns g, g + 8, g + 16,
// ... in ascending order; an xor butterfly then adds the 8 partials as
// ((p0+p1)+(p2+p3))+((p4+p5)+(p6+p7)) on every lane.  On this FP64 pipe the latency of the
// dependent chain sets the time, so it is kept short: 8 multiply-adds and 3 additions.  The
// coarse V-cycle kernels all solve the coarsest level here, so they give the same bits.
// dinv: row-major, row stride n, in global or shared memory.
template <class T>
__device__ void dense_coarse_apply(int n, const double* dinv, const T* b, T* x, int singular) {
    const int t = threadIdx.x, g = t & 7, rows = blockDim.x >> 3;
    for (int base = 0; base < n; base += rows) {
        const int r = base + (t >> 3);
        double s = 0.0;
        if (r < n)
            for (int c = g; c < n; c += 8) {
                const double bc = (singular && c == 0) ? 0.0 : (double)b[c];
                s += dinv[r * n + c] * bc;
            }
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        s += __shfl_xor_sync(0xffffffffu, s, 4);
        if (r < n && g == 0) x[r] = (T)s;
    }
    __syncthreads();
}

template <class T>
struct CoarseArgs {
    int nl, singular, dn;
    int pre, post;  // smoother sweeps before / after the coarse correction
    int zero_color;  // restriction skips cells of this colour (their residual is ~0), or -1
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
                } else {  // as k_gs4_exp9: s = b - sum_e a_e x_e, x = s * idiag
                    if ((((i & 1) << 1) | (j & 1)) != col) continue;
                    T o = 0;
                    for (int e = 1; e < 9; ++e) {
                        int ii = i + c_off[e][0], jj = j + c_off[e][1];
                        if (ii < 0 || ii >= n1 || jj < 0 || jj >= n2) continue;
                        o += a9[e * n + k] * x[IX(ii, jj, n2)];
                    }
                    x[k] = (b[k] - o) * id[k];
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
            for (int k = threadIdx.x; k < (n1 + 1) * n2; k += blockDim.x) stage_async(tx[l] + k, A.tx[l] + k);
            for (int k = threadIdx.x; k < n1 * (n2 + 1); k += blockDim.x) stage_async(ty[l] + k, A.ty[l] + k);
            for (int k = threadIdx.x; k < n; k += blockDim.x) stage_async(dg[l] + k, A.dg[l] + k);
        } else {
            for (int k = threadIdx.x; k < 9 * n; k += blockDim.x) stage_async(a9[l] + k, A.a9[l] + k);
        }
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            stage_async(id[l] + k, A.id[l] + k);
            if (l == 0) {
                stage_async(x[l] + k, A.x0 + k);
                stage_async(b[l] + k, A.b0 + k);
            } else {
                x[l][k] = T(0);
                b[l][k] = T(0);
            }
        }
    }
    stage_wait();
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
                    if (((i + j) & 1) == A.zero_color) continue;  // as k_restrict
                    if (i < n1 && j < n2) s += cv_resid<T, KIND>(i, j, n1, n2, tx[l], ty[l], a9[l], dg[l], b[l], x[l]);
                }
            b[l + 1][K] = s;
            x[l + 1][K] = 0;
        }
        __syncthreads();
    }
    dense_coarse_apply<T>(A.dn, A.dinv, b[L], x[L], A.singular);  // coarsest level
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
