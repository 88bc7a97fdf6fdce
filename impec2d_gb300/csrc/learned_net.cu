// Learned pressure warm start: a 4-level convolutional encoder-decoder that predicts, from
// the state at the start of a pressure solve, the error of the previous step's pressure as an
// initial guess.  It is used only to move the initial iterate (the solve still converges to
// its tolerance).  No counterpart in the reference.
//
// Layers (3x3 convolutions, GELU, BF16 weights and activations, fp32 accumulation on tcgen05):
//   level 0 (H x W):     0: 8 -> 32,   1: 32 -> 32                      (e0)
//   level 1 (H/2):       2: 32 -> 64,  3: 64 -> 64   after 2x2 pooling  (e1)
//   level 2 (H/4):       4: 64 -> 128, 5: 128 -> 128                    (e2)
//   level 3 (H/8):       6: 128 -> 256, 7: 256 -> 256
//   decoder:  8: 256 -> 128 (+ e2),  9: 128 -> 128  after nearest 2x upsampling (H/4)
//            10: 128 -> 64  (+ e1), 11: 64 -> 64                              (H/2)
//            12: 64 -> 32   (+ e0), 13: 32 -> 32                              (H)
//   head:    14: 32 -> 8, linear; channel 0 is the prediction.
// Skips add the encoder output after the decoder convolution's activation.  Training: MSE
// loss, AdamW on fp32 master weights (the bf16 copies feed the tensor cores).
//
// Use inside the pressure solve (impec_learned_attach): with the operator of the new
// mobility built and x0 = the previous pressure, the solve computes r0 = f - A x0, the
// features below averaged over factor x factor cells, the network's prediction d (bilinear
// back to the fine grid), and steps x0 += alpha d with alpha = (r0, d) / (d, A d), the step
// that minimises the A-norm error along d.  Features per coarse cell:
//   0: mean of 4 log(1 - c + M^(1/4) c)   (log of the mobility ratio to the resident fluid)
//   1: mean of log K
//   2: sum of q dA / I                    (+1 at the injector, -1 at a producer)
//   3: mean of x0, centred and divided by its RMS over the coarse cells
//   4: mean of r0, divided by its RMS over the coarse cells
// The training target of a recorded solve is the mean over each coarse cell of (p - x0), p
// the converged pressure, centred and scaled to unit RMS (alpha makes the scale irrelevant).
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "learned.cuh"

namespace impec {

constexpr int NET_LAYERS = 15, NET_IN = 8, NET_OUT = 8;

struct NetLayer {
    int cin, cout, level, act, skip_from;  // skip_from: layer whose output is added, or -1
    int Kp;
    __nv_bfloat16* w = nullptr;            // [cout][Kp] bf16
    float *wm = nullptr, *b = nullptr;     // master weights [cout][Kp], bias [cout]
    float *gw = nullptr, *gb = nullptr;    // gradients
    float *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;  // AdamW moments
    __nv_bfloat16* wd = nullptr;           // transposed weights for the input gradient
};

// Per-layer activation and gradient buffers for a given batch shape.
struct NetBuffers {
    int B = 0, H = 0, W = 0;
    __nv_bfloat16 *z[NET_LAYERS] = {}, *y[NET_LAYERS] = {}, *dz[NET_LAYERS] = {};
    __nv_bfloat16 *d1 = nullptr, *d2 = nullptr, *d3 = nullptr, *u2 = nullptr, *u1 = nullptr, *u0 = nullptr;
    __nv_bfloat16 *graw = nullptr, *ds0 = nullptr, *ds1 = nullptr, *ds2 = nullptr;
    float* out = nullptr;
    double* loss = nullptr;
    std::vector<void*> all;
};

// State of a network attached to a context as the initial guess of its pressure solves.
struct LearnedHook {
    impec_net* net = nullptr;
    int factor = 1, mode = 0, h = 0, w = 0;
    NetBuffers nb;                  // inference buffers at (1, h, w), separate from the training ones
    __nv_bfloat16* X = nullptr;     // features [h][w][8]
    float* raw = nullptr;           // pooled raw channels [h][w][5]
    float* T = nullptr;             // target scratch [h][w]
    double* x0 = nullptr;           // initial iterate of the last solve
    double* sums = nullptr;         // [0] sum x, [1] sum x^2, [2] sum r^2 over coarse cells; [3], [4] target sums
};

}  // namespace impec

struct impec_net {
    impec::NetLayer L[impec::NET_LAYERS];
    impec::NetBuffers buf;
    long long step = 0;
    int num_sms = 148;
    int attached = 0;  // contexts whose pressure solves use this network
    int* err = nullptr;
};

namespace impec {

static const int kLayerSpec[NET_LAYERS][5] = {
    // cin, cout, level, act, skip_from
    {NET_IN, 32, 0, 1, -1}, {32, 32, 0, 1, -1},  {32, 64, 1, 1, -1},  {64, 64, 1, 1, -1},    {64, 128, 2, 1, -1},
    {128, 128, 2, 1, -1},   {128, 256, 3, 1, -1}, {256, 256, 3, 1, -1}, {256, 128, 2, 1, 5},    {128, 128, 2, 1, -1},
    {128, 64, 1, 1, 3},     {64, 64, 1, 1, -1},   {64, 32, 0, 1, 1},    {32, 32, 0, 1, -1},     {32, NET_OUT, 0, 0, -1}};

// ---------------------------------------------------------------- elementwise kernels
__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float gelu_d(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// 2x2 average pooling and nearest 2x upsampling, 8 channels (16 bytes) per thread; C is a
// multiple of 8.
__global__ void k_pool2(const __nv_bfloat16* __restrict__ in, int B, int h, int w, int C, __nv_bfloat16* __restrict__ out) {
    const int C8 = C >> 3;
    const size_t n = (size_t)B * h * w * C8;  // output vectors, h x w = the pooled size
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int c8 = (int)(i % C8);
        size_t t = i / C8;
        const int x = (int)(t % w);
        t /= w;
        const int y = (int)(t % h), b = (int)(t / h);
        const size_t W2 = 2 * (size_t)w, r0 = ((size_t)b * 2 * h + 2 * y) * W2 + 2 * x;
        const size_t src[4] = {r0, r0 + 1, r0 + W2, r0 + W2 + 1};
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            __align__(16) __nv_bfloat16 v[8];
            *reinterpret_cast<uint4*>(v) = *reinterpret_cast<const uint4*>(in + src[q] * C + 8 * c8);
#pragma unroll
            for (int k = 0; k < 8; ++k) acc[k] += bf(v[k]);
        }
        __align__(16) __nv_bfloat16 o[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) o[k] = __float2bfloat16(0.25f * acc[k]);
        *reinterpret_cast<uint4*>(out + i * 8) = *reinterpret_cast<const uint4*>(o);
    }
}

__global__ void k_up2(const __nv_bfloat16* __restrict__ in, int B, int h, int w, int C, __nv_bfloat16* __restrict__ out) {
    const int C8 = C >> 3;
    const size_t n = (size_t)B * 2 * h * 2 * w * C8;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int c8 = (int)(i % C8);
        size_t t = i / C8;
        const int x = (int)(t % (2 * w));
        t /= 2 * w;
        const int y = (int)(t % (2 * h)), b = (int)(t / (2 * h));
        *reinterpret_cast<uint4*>(out + i * 8) =
            *reinterpret_cast<const uint4*>(in + (((size_t)b * h + y / 2) * w + x / 2) * C + 8 * c8);
    }
}

// dz (h x w) = (sum over the 2x2 children of g (2h x 2w)) * gelu'(z)
__global__ void k_up2_bwd_gelu(const __nv_bfloat16* __restrict__ g, const __nv_bfloat16* __restrict__ z, int B, int h,
                               int w, int C, __nv_bfloat16* __restrict__ dz) {
    const size_t n = (size_t)B * h * w * C;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        size_t t = i / C;
        const int x = (int)(t % w);
        t /= w;
        const int y = (int)(t % h), b = (int)(t / h);
        const size_t W2 = 2 * (size_t)w, r0 = ((size_t)b * 2 * h + 2 * y) * W2 + 2 * x;
        const float s = bf(g[r0 * C + c]) + bf(g[(r0 + 1) * C + c]) + bf(g[(r0 + W2) * C + c]) + bf(g[(r0 + W2 + 1) * C + c]);
        dz[i] = __float2bfloat16(s * gelu_d(bf(z[i])));
    }
}

// dz (2h x 2w) = (g(parent) / 4 + skip) * gelu'(z)
__global__ void k_pool2_bwd_add_gelu(const __nv_bfloat16* __restrict__ g, const __nv_bfloat16* __restrict__ skip,
                                     const __nv_bfloat16* __restrict__ z, int B, int h, int w, int C,
                                     __nv_bfloat16* __restrict__ dz) {
    const size_t n = (size_t)B * 2 * h * 2 * w * C;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        size_t t = i / C;
        const int x = (int)(t % (2 * w));
        t /= 2 * w;
        const int y = (int)(t % (2 * h)), b = (int)(t / (2 * h));
        const float gp = bf(g[(((size_t)b * h + y / 2) * w + x / 2) * C + c]);
        dz[i] = __float2bfloat16((0.25f * gp + bf(skip[i])) * gelu_d(bf(z[i])));
    }
}

// gb[c] += sum over P pixels of dz[p][c].  Thread t of a block reads 8 channels (16 bytes) of
// one pixel: channel group t % (C / 8), pixel lane t / (C / 8); the block folds its partial
// sums per channel in shared memory and adds them with one atomic per channel.  C is a
// multiple of 8 and divides 8 * blockDim.x (blockDim.x = 256).
__global__ void __launch_bounds__(256) k_bias_grad(const __nv_bfloat16* __restrict__ dz, size_t P, int C,
                                                   float* __restrict__ gb) {
    __shared__ float part[256 * 8];
    const int C8 = C >> 3, lanes = blockDim.x / C8;
    const int cg = threadIdx.x % C8, pl = threadIdx.x / C8;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (pl < lanes)
        for (size_t p = blockIdx.x * (size_t)lanes + pl; p < P; p += (size_t)gridDim.x * lanes) {
            __align__(16) __nv_bfloat16 v[8];
            *reinterpret_cast<uint4*>(v) = *reinterpret_cast<const uint4*>(dz + p * C + 8 * cg);
#pragma unroll
            for (int k = 0; k < 8; ++k) acc[k] += bf(v[k]);
        }
#pragma unroll
    for (int k = 0; k < 8; ++k) part[threadIdx.x * 8 + k] = acc[k];
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
        float s = 0.0f;
        for (int l = 0; l < lanes; ++l) s += part[(l * C8 + (c >> 3)) * 8 + (c & 7)];
        atomicAdd(gb + c, s);
    }
}

// MSE on channel 0: loss += sum (o - t)^2 / P; dz channel 0 = 2 (o - t) / P, other channels 0.
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ t, size_t P, __nv_bfloat16* __restrict__ dz,
                      double* loss) {
    double acc = 0.0;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        const float e = out[p * NET_OUT] - t[p];
        acc += (double)e * e;
        dz[p * NET_OUT] = __float2bfloat16(2.0f * e / (float)P);
#pragma unroll
        for (int c = 1; c < NET_OUT; ++c) dz[p * NET_OUT + c] = __float2bfloat16(0.0f);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc / (double)P);
}

// AdamW (decoupled weight decay) on fp32 masters; refreshes the bf16 copy; clears the gradient.
__global__ void k_adamw(float* __restrict__ w, __nv_bfloat16* __restrict__ wb, float* __restrict__ g,
                        float* __restrict__ m, float* __restrict__ v, size_t n, float lr, float b1, float b2,
                        float eps, float wd, float bc1, float bc2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi, vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float upd = (mi / bc1) / (sqrtf(vi / bc2) + eps);
        const float wi = w[i] * (1.0f - lr * wd) - lr * upd;
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16(wi);
        g[i] = 0.0f;
    }
}

// Block sum of K values into out[0..K) with one atomic per block (blockDim.x = 256).
template <int K>
__device__ __forceinline__ void block_add(double (&v)[K], double* out) {
    __shared__ double sh[K][8];
#pragma unroll
    for (int j = 0; j < K; ++j)
        for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
    const int wid = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int j = 0; j < K; ++j) sh[j][wid] = v[j];
    __syncthreads();
    if (threadIdx.x < K) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[threadIdx.x][k];
        atomicAdd(out + threadIdx.x, t);
    }
}

// Raw features per coarse cell (f x f fine cells) into raw [h][w][5]; sums of the centred
// pressure's moments and of the residual's square into sums[0..3).
__global__ void __launch_bounds__(256) k_learn_pool(int n1, int n2, int f, const double* __restrict__ c,
                                                    const double* __restrict__ K, const double* __restrict__ q,
                                                    const double* __restrict__ x, const double* __restrict__ r,
                                                    double m14, double qnorm, float* __restrict__ raw,
                                                    double* sums) {
    const int h = n1 / f, w = n2 / f;
    const size_t m = (size_t)h * w;
    double acc[3] = {0.0, 0.0, 0.0};
    const double inv = 1.0 / ((double)f * f);
    const float m14f = (float)m14;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < m; k += (size_t)gridDim.x * blockDim.x) {
        const int I = (int)(k / w), J = (int)(k % w);
        // the logarithms in FP32 (the features are stored in bf16; FP64 transcendentals are slow)
        float lm = 0.0f, lk = 0.0f;
        double s[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < f; ++a)
            for (int b = 0; b < f; ++b) {
                const size_t g = (size_t)(I * f + a) * n2 + (size_t)J * f + b;
                const float cg = (float)c[g];
                lm += 4.0f * logf(1.0f - cg + m14f * cg);
                lk += K ? logf((float)K[g]) : 0.0f;
                s[0] += q[g];
                s[1] += x[g];
                s[2] += r[g];
            }
        const double xm = s[1] * inv, rm = s[2] * inv;
        raw[k * 5 + 0] = (float)(lm * inv);
        raw[k * 5 + 1] = (float)(lk * inv);
        raw[k * 5 + 2] = (float)(s[0] * qnorm);
        raw[k * 5 + 3] = (float)xm;
        raw[k * 5 + 4] = (float)rm;
        acc[0] += xm;
        acc[1] += xm * xm;
        acc[2] += rm * rm;
    }
    block_add<3>(acc, sums);
}

__global__ void k_learn_pack(size_t m, const float* __restrict__ raw, const double* __restrict__ sums,
                             __nv_bfloat16* __restrict__ X) {
    const double mean = sums[0] / (double)m;
    const double var = sums[1] / (double)m - mean * mean;
    const double sx = 1.0 / (sqrt(var > 0.0 ? var : 0.0) + 1e-300), sr = 1.0 / (sqrt(sums[2] / (double)m) + 1e-300);
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < m; k += (size_t)gridDim.x * blockDim.x) {
        const float v[NET_IN] = {raw[k * 5 + 0], raw[k * 5 + 1], raw[k * 5 + 2],
                                 (float)(((double)raw[k * 5 + 3] - mean) * sx), (float)((double)raw[k * 5 + 4] * sr),
                                 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int j = 0; j < NET_IN; ++j) X[k * NET_IN + j] = __float2bfloat16(v[j]);
    }
}

// Prediction (channel 0 of out [h][w][8]) to the fine grid, bilinear between coarse cell
// centres (constant beyond the outermost centres).
__global__ void k_learn_direction(int n1, int n2, int f, const float* __restrict__ out, double* __restrict__ d) {
    const int h = n1 / f, w = n2 / f;
    const size_t n = (size_t)n1 * n2;
    const float inv = 1.0f / (float)f;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(k / n2), j = (int)(k % n2);
        const float fi = ((float)i + 0.5f) * inv - 0.5f, fj = ((float)j + 0.5f) * inv - 0.5f;
        const int i0 = min(max((int)floorf(fi), 0), h - 1), j0 = min(max((int)floorf(fj), 0), w - 1);
        const int i1 = min(i0 + 1, h - 1), j1 = min(j0 + 1, w - 1);
        const float a = fminf(fmaxf(fi - (float)i0, 0.0f), 1.0f), b = fminf(fmaxf(fj - (float)j0, 0.0f), 1.0f);
        const float v00 = out[((size_t)i0 * w + j0) * NET_OUT], v01 = out[((size_t)i0 * w + j1) * NET_OUT];
        const float v10 = out[((size_t)i1 * w + j0) * NET_OUT], v11 = out[((size_t)i1 * w + j1) * NET_OUT];
        d[k] = (double)((1.0f - a) * ((1.0f - b) * v00 + b * v01) + a * ((1.0f - b) * v10 + b * v11));
    }
}

// Target of a recorded solve: mean over each coarse cell of (p - x0), then centred and scaled
// to unit RMS (second kernel).
__global__ void __launch_bounds__(256) k_learn_target(int n1, int n2, int f, const double* __restrict__ p,
                                                      const double* __restrict__ x0, float* __restrict__ T,
                                                      double* sums) {
    const int h = n1 / f, w = n2 / f;
    const size_t m = (size_t)h * w;
    double acc[2] = {0.0, 0.0};
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < m; k += (size_t)gridDim.x * blockDim.x) {
        const int I = (int)(k / w), J = (int)(k % w);
        double s = 0.0;
        for (int a = 0; a < f; ++a)
            for (int b = 0; b < f; ++b) {
                const size_t g = (size_t)(I * f + a) * n2 + (size_t)J * f + b;
                s += p[g] - x0[g];
            }
        s /= (double)f * f;
        T[k] = (float)s;
        acc[0] += s;
        acc[1] += s * s;
    }
    block_add<2>(acc, sums);
}

__global__ void k_learn_target_scale(size_t m, const double* __restrict__ sums, const float* __restrict__ T,
                                     float* __restrict__ out) {
    const double mean = sums[0] / (double)m, var = sums[1] / (double)m - mean * mean;
    const double sc = 1.0 / (sqrt(var > 0.0 ? var : 0.0) + 1e-300);
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < m; k += (size_t)gridDim.x * blockDim.x)
        out[k] = (float)(((double)T[k] - mean) * sc);
}

// ---------------------------------------------------------------- host side
static dim3 egrid(size_t n) {
    size_t b = (n + 255) / 256;
    return dim3((unsigned)(b < 8192 ? (b > 0 ? b : 1) : 8192));
}

static size_t level_pixels(const NetBuffers& nb, int level) {
    return (size_t)nb.B * (nb.H >> level) * (nb.W >> level);
}

static void free_buffers(NetBuffers& nb) {
    for (void* p : nb.all) cudaFree(p);
    nb = NetBuffers();
}

// Activation buffers for a batch shape; train adds the pre-activations and gradients.
static impec_status alloc_buffers(NetBuffers& nb, const impec_net* net, int B, int H, int W, bool train) {
    if (nb.B == B && nb.H == H && nb.W == W) return IMPEC_OK;
    free_buffers(nb);
    nb.B = B;
    nb.H = H;
    nb.W = W;
    auto alloc = [&](void** p, size_t bytes) -> impec_status {
        IMPEC_CUDA_TRY(cudaMalloc(p, bytes));
        nb.all.push_back(*p);
        return IMPEC_OK;
    };
    for (int l = 0; l < NET_LAYERS; ++l) {
        const size_t P = level_pixels(nb, net->L[l].level), e = P * net->L[l].cout * 2;
        IMPEC_TRY(alloc((void**)&nb.y[l], e));
        if (!train) continue;
        IMPEC_TRY(alloc((void**)&nb.z[l], e));
        IMPEC_TRY(alloc((void**)&nb.dz[l], e));
    }
    const size_t P0 = level_pixels(nb, 0), P1 = level_pixels(nb, 1), P2 = level_pixels(nb, 2), P3 = level_pixels(nb, 3);
    IMPEC_TRY(alloc((void**)&nb.d1, P1 * 32 * 2));
    IMPEC_TRY(alloc((void**)&nb.d2, P2 * 64 * 2));
    IMPEC_TRY(alloc((void**)&nb.d3, P3 * 128 * 2));
    IMPEC_TRY(alloc((void**)&nb.u2, P2 * 256 * 2));
    IMPEC_TRY(alloc((void**)&nb.u1, P1 * 128 * 2));
    IMPEC_TRY(alloc((void**)&nb.u0, P0 * 64 * 2));
    IMPEC_TRY(alloc((void**)&nb.out, P0 * NET_OUT * 4));
    if (!train) return IMPEC_OK;
    IMPEC_TRY(alloc((void**)&nb.graw, P0 * 64 * 2));
    IMPEC_TRY(alloc((void**)&nb.ds0, P0 * 32 * 2));
    IMPEC_TRY(alloc((void**)&nb.ds1, P1 * 64 * 2));
    IMPEC_TRY(alloc((void**)&nb.ds2, P2 * 128 * 2));
    IMPEC_TRY(alloc((void**)&nb.loss, sizeof(double)));
    return IMPEC_OK;
}

static impec_status ensure_buffers(impec_net* net, int B, int H, int W) {
    return alloc_buffers(net->buf, net, B, H, W, true);
}

static const __nv_bfloat16* layer_input(const NetBuffers& nb, const __nv_bfloat16* X, int l) {
    switch (l) {
        case 0: return X;
        case 2: return nb.d1;
        case 4: return nb.d2;
        case 6: return nb.d3;
        case 8: return nb.u2;
        case 10: return nb.u1;
        case 12: return nb.u0;
        default: return nb.y[l - 1];
    }
}

static impec_status conv_forward(impec_net* net, const NetBuffers& nb, const __nv_bfloat16* X, int l, bool train,
                                 cudaStream_t s) {
    const NetLayer& L = net->L[l];
    ConvArgs a = {};
    a.X = layer_input(nb, X, l);
    a.W = L.w;
    a.bias = L.b;
    a.Z = train ? nb.z[l] : nullptr;
    a.Y = l == NET_LAYERS - 1 ? nullptr : nb.y[l];
    a.Yf = l == NET_LAYERS - 1 ? nb.out : nullptr;
    a.skip = L.skip_from >= 0 ? nb.y[L.skip_from] : nullptr;
    a.B = nb.B;
    a.H = nb.H >> L.level;
    a.W_ = nb.W >> L.level;
    a.cin = L.cin;
    a.cout = L.cout;
    a.Kp = L.Kp;
    a.tapsign = 1;
    a.act = L.act;
    a.err = net->err;
    return launch_conv(a, s);
}

// Launch only (no host synchronisation): also used inside captured pressure solves.
static impec_status net_forward(impec_net* net, const NetBuffers& nb, const __nv_bfloat16* X, bool train,
                                cudaStream_t s) {
    const int B = nb.B, H = nb.H, W = nb.W;
    for (int l = 0; l < NET_LAYERS; ++l) {
        IMPEC_TRY(conv_forward(net, nb, X, l, train, s));
        switch (l) {
            case 1: k_pool2<<<egrid(level_pixels(nb, 1) * 4), 256, 0, s>>>(nb.y[1], B, H >> 1, W >> 1, 32, nb.d1); break;
            case 3: k_pool2<<<egrid(level_pixels(nb, 2) * 8), 256, 0, s>>>(nb.y[3], B, H >> 2, W >> 2, 64, nb.d2); break;
            case 5: k_pool2<<<egrid(level_pixels(nb, 3) * 16), 256, 0, s>>>(nb.y[5], B, H >> 3, W >> 3, 128, nb.d3); break;
            case 7: k_up2<<<egrid(level_pixels(nb, 2) * 32), 256, 0, s>>>(nb.y[7], B, H >> 3, W >> 3, 256, nb.u2); break;
            case 9: k_up2<<<egrid(level_pixels(nb, 1) * 16), 256, 0, s>>>(nb.y[9], B, H >> 2, W >> 2, 128, nb.u1); break;
            case 11: k_up2<<<egrid(level_pixels(nb, 0) * 8), 256, 0, s>>>(nb.y[11], B, H >> 1, W >> 1, 64, nb.u0); break;
            default: break;
        }
        IMPEC_CUDA_TRY(cudaGetLastError());
    }
    return IMPEC_OK;
}

// Input gradient of layer l: Y = gradient of the layer below's pre-activation (times gelu'),
// R = the raw gradient of the layer's input (for skips / pooling), either may be null.
static impec_status conv_input_grad(impec_net* net, int l, const __nv_bfloat16* gz, __nv_bfloat16* Y,
                                    __nv_bfloat16* R, cudaStream_t s) {
    const NetLayer& L = net->L[l];
    const NetBuffers& nb = net->buf;
    launch_wt_transpose(L.w, L.cin, L.cout, L.wd, s);
    ConvArgs a = {};
    a.X = nb.dz[l];
    a.W = L.wd;
    a.gz = gz;
    a.Y = gz ? Y : nullptr;
    a.R = gz ? R : nullptr;
    a.Yf = nullptr;
    a.B = nb.B;
    a.H = nb.H >> L.level;
    a.W_ = nb.W >> L.level;
    a.cin = L.cout;
    a.cout = L.cin;
    a.Kp = conv_kp(L.cout);
    a.tapsign = -1;
    a.err = net->err;
    if (!gz) a.Y = R;  // plain transposed convolution into R
    return launch_conv(a, s);
}

static impec_status net_backward(impec_net* net, const __nv_bfloat16* X, cudaStream_t s) {
    NetBuffers& nb = net->buf;
    const int B = nb.B, H = nb.H, W = nb.W;
    for (int l = NET_LAYERS - 1; l >= 0; --l) {
        const NetLayer& L = net->L[l];
        const int h = H >> L.level, w = W >> L.level;
        IMPEC_TRY(launch_wgrad(nb.dz[l], layer_input(nb, X, l), B, h, w, L.cin, L.cout, L.gw, net->err, net->num_sms, s));
        const size_t P = level_pixels(nb, L.level);
        {
            const size_t want = (P * (size_t)(L.cout / 8) + 255) / 256, cap = (size_t)net->num_sms * 8;
            k_bias_grad<<<(unsigned)(want < cap ? want : cap), 256, 0, s>>>(nb.dz[l], P, L.cout, L.gb);
        }
        switch (l) {
            case 0: break;
            case 14: case 7: case 5: case 3: case 1:  // input is a plain GELU output
                IMPEC_TRY(conv_input_grad(net, l, nb.z[l - 1], nb.dz[l - 1], nullptr, s));
                break;
            // input is a decoder output with a skip: its raw gradient is also the encoder's skip gradient
            case 13: IMPEC_TRY(conv_input_grad(net, l, nb.z[12], nb.dz[12], nb.ds0, s)); break;  // y12 = gelu(z12) + y1
            case 11: IMPEC_TRY(conv_input_grad(net, l, nb.z[10], nb.dz[10], nb.ds1, s)); break;  // y10 = gelu(z10) + y3
            case 9: IMPEC_TRY(conv_input_grad(net, l, nb.z[8], nb.dz[8], nb.ds2, s)); break;     // y8 = gelu(z8) + y5
            case 12: case 10: case 8: {  // input is an upsampled GELU output
                IMPEC_TRY(conv_input_grad(net, l, nullptr, nullptr, nb.graw, s));
                const int lo = l - 1, hl = h >> 1, wl = w >> 1;
                k_up2_bwd_gelu<<<egrid(level_pixels(nb, net->L[lo].level) * net->L[lo].cout), 256, 0, s>>>(
                    nb.graw, nb.z[lo], B, hl, wl, net->L[lo].cout, nb.dz[lo]);
                break;
            }
            case 6: case 4: case 2: {  // input is a pooled encoder output that also feeds a skip
                IMPEC_TRY(conv_input_grad(net, l, nullptr, nullptr, nb.graw, s));
                const int lo = l - 1;
                const __nv_bfloat16* skipg = l == 6 ? nb.ds2 : (l == 4 ? nb.ds1 : nb.ds0);
                k_pool2_bwd_add_gelu<<<egrid(level_pixels(nb, net->L[lo].level) * net->L[lo].cout), 256, 0, s>>>(
                    nb.graw, skipg, nb.z[lo], B, h, w, net->L[lo].cout, nb.dz[lo]);
                break;
            }
        }
        IMPEC_CUDA_TRY(cudaGetLastError());
    }
    return IMPEC_OK;
}

static impec_status net_init(impec_net* net, unsigned long long seed) {
    std::mt19937_64 rng(seed);
    for (int l = 0; l < NET_LAYERS; ++l) {
        NetLayer& L = net->L[l];
        L.cin = kLayerSpec[l][0];
        L.cout = kLayerSpec[l][1];
        L.level = kLayerSpec[l][2];
        L.act = kLayerSpec[l][3];
        L.skip_from = kLayerSpec[l][4];
        L.Kp = conv_kp(L.cin);
        const size_t nw = (size_t)L.cout * L.Kp;
        const double std = l == NET_LAYERS - 1 ? 0.1 * std::sqrt(1.0 / (9.0 * L.cin)) : std::sqrt(2.0 / (9.0 * L.cin));
        std::normal_distribution<double> nd(0.0, std);
        std::vector<float> wm(nw, 0.0f);
        for (int co = 0; co < L.cout; ++co)
            for (int k = 0; k < 9 * L.cin; ++k) wm[(size_t)co * L.Kp + k] = (float)nd(rng);
        std::vector<__nv_bfloat16> wb(nw);
        for (size_t i = 0; i < nw; ++i) wb[i] = __float2bfloat16(wm[i]);
        IMPEC_CUDA_TRY(cudaMalloc((void**)&L.w, nw * 2));
        IMPEC_CUDA_TRY(cudaMalloc((void**)&L.wd, (size_t)L.cin * conv_kp(L.cout) * 2));
        float** fbufs[] = {&L.wm, &L.gw, &L.mw, &L.vw};
        for (float** f : fbufs) {
            IMPEC_CUDA_TRY(cudaMalloc((void**)f, nw * 4));
            IMPEC_CUDA_TRY(cudaMemset(*f, 0, nw * 4));
        }
        float** bbufs[] = {&L.b, &L.gb, &L.mb, &L.vb};
        for (float** f : bbufs) {
            IMPEC_CUDA_TRY(cudaMalloc((void**)f, L.cout * 4));
            IMPEC_CUDA_TRY(cudaMemset(*f, 0, L.cout * 4));
        }
        IMPEC_CUDA_TRY(cudaMemcpy(L.wm, wm.data(), nw * 4, cudaMemcpyHostToDevice));
        IMPEC_CUDA_TRY(cudaMemcpy(L.w, wb.data(), nw * 2, cudaMemcpyHostToDevice));
    }
    return IMPEC_OK;
}

static void net_free(impec_net* net) {
    for (NetLayer& L : net->L) {
        void* ps[] = {L.w, L.wd, L.wm, L.b, L.gw, L.gb, L.mw, L.vw, L.mb, L.vb};
        for (void* p : ps)
            if (p) cudaFree(p);
    }
    free_buffers(net->buf);
}

static size_t net_param_count(const impec_net* net) {
    size_t n = 0;
    for (const NetLayer& L : net->L) n += (size_t)L.cout * L.Kp + L.cout;
    return n;
}

}  // namespace impec

using namespace impec;

extern "C" impec_status impec_net_create(unsigned long long seed, impec_net** out) {
    if (!out) return IMPEC_ERR_ARG;
    impec_net* net = new impec_net();
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&net->num_sms, cudaDevAttrMultiProcessorCount, dev);
    net->err = device_error_flag();
    impec_status s = net->err ? net_init(net, seed) : IMPEC_ERR_CUDA;
    if (s != IMPEC_OK) {
        net_free(net);
        delete net;
        return s;
    }
    *out = net;
    return IMPEC_OK;
}

extern "C" impec_status impec_net_destroy(impec_net* net) {
    if (!net) return IMPEC_OK;
    if (net->attached > 0) {
        set_error("impec_net_destroy: the network is still attached to a context (impec_learned_attach with NULL first)");
        return IMPEC_ERR_ARG;
    }
    cudaDeviceSynchronize();
    net_free(net);
    delete net;
    return IMPEC_OK;
}

static bool net_shape_ok(int B, int H, int W) { return B > 0 && H >= 8 && W >= 8 && H % 8 == 0 && W % 8 == 0; }

// One training step on a batch: X [B][H][W][8] bf16 features, T [B][H][W] fp32 targets.
extern "C" impec_status impec_net_train_batch(impec_net* net, const void* X, const float* T, int B, int H, int W,
                                              double lr, double weight_decay, double* loss, void* stream) {
    if (!net || !X || !T || !net_shape_ok(B, H, W)) {
        set_error("impec_net_train_batch: B >= 1 and H, W multiples of 8 required");
        return IMPEC_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    IMPEC_TRY(ensure_buffers(net, B, H, W));
    NetBuffers& nb = net->buf;
    const __nv_bfloat16* x = (const __nv_bfloat16*)X;
    IMPEC_TRY(net_forward(net, nb, x, true, s));
    const size_t P = level_pixels(nb, 0);
    IMPEC_CUDA_TRY(cudaMemsetAsync(nb.loss, 0, sizeof(double), s));
    k_mse<<<egrid(P), 256, 0, s>>>(nb.out, T, P, nb.dz[NET_LAYERS - 1], nb.loss);
    IMPEC_TRY(net_backward(net, x, s));
    net->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.0f - (float)std::pow(b1, (double)net->step), bc2 = 1.0f - (float)std::pow(b2, (double)net->step);
    for (NetLayer& L : net->L) {
        const size_t nw = (size_t)L.cout * L.Kp;
        k_adamw<<<egrid(nw), 256, 0, s>>>(L.wm, L.w, L.gw, L.mw, L.vw, nw, (float)lr, b1, b2, 1e-8f, (float)weight_decay,
                                          bc1, bc2);
        k_adamw<<<1, 256, 0, s>>>(L.b, nullptr, L.gb, L.mb, L.vb, L.cout, (float)lr, b1, b2, 1e-8f, 0.0f, bc1, bc2);
    }
    IMPEC_CUDA_TRY(cudaGetLastError());
    if (loss) IMPEC_CUDA_TRY(cudaMemcpyAsync(loss, nb.loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    return check_err(net->err, s, "impec_net_train_batch");
}

// Gradients of the last batch without updating (for checks): forward + backward only; the
// gradients are left in the parameter-gradient buffers, read by impec_net_gradients.
extern "C" impec_status impec_net_backprop(impec_net* net, const void* X, const float* T, int B, int H, int W,
                                           double* loss, void* stream) {
    if (!net || !X || !T || !net_shape_ok(B, H, W)) return IMPEC_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    IMPEC_TRY(ensure_buffers(net, B, H, W));
    NetBuffers& nb = net->buf;
    for (NetLayer& L : net->L) {
        IMPEC_CUDA_TRY(cudaMemsetAsync(L.gw, 0, (size_t)L.cout * L.Kp * 4, s));
        IMPEC_CUDA_TRY(cudaMemsetAsync(L.gb, 0, (size_t)L.cout * 4, s));
    }
    const __nv_bfloat16* x = (const __nv_bfloat16*)X;
    IMPEC_TRY(net_forward(net, nb, x, true, s));
    const size_t P = level_pixels(nb, 0);
    IMPEC_CUDA_TRY(cudaMemsetAsync(nb.loss, 0, sizeof(double), s));
    k_mse<<<egrid(P), 256, 0, s>>>(nb.out, T, P, nb.dz[NET_LAYERS - 1], nb.loss);
    IMPEC_TRY(net_backward(net, x, s));
    if (loss) IMPEC_CUDA_TRY(cudaMemcpyAsync(loss, nb.loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    return check_err(net->err, s, "impec_net_backprop");
}

// Prediction (channel 0) for X [B][H][W][8]: out [B][H][W] fp32.
extern "C" impec_status impec_net_forward(impec_net* net, const void* X, int B, int H, int W, float* out, void* stream) {
    if (!net || !X || !out || !net_shape_ok(B, H, W)) return IMPEC_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    IMPEC_TRY(ensure_buffers(net, B, H, W));
    IMPEC_TRY(net_forward(net, net->buf, (const __nv_bfloat16*)X, false, s));
    const size_t P = level_pixels(net->buf, 0);
    IMPEC_CUDA_TRY(cudaMemcpy2DAsync(out, sizeof(float), net->buf.out, NET_OUT * sizeof(float), sizeof(float), P,
                                     cudaMemcpyDeviceToDevice, s));
    return check_err(net->err, s, "impec_net_forward");
}

// Parameter count; copies to/from a host buffer in layer order (weights [cout][Kp] then bias).
extern "C" impec_status impec_net_parameters(impec_net* net, float* host_out, const float* host_in, size_t* count,
                                             int which) {
    if (!net || !count) return IMPEC_ERR_ARG;
    *count = net_param_count(net);
    size_t off = 0;
    for (NetLayer& L : net->L) {
        const size_t nw = (size_t)L.cout * L.Kp;
        float* w = which == 1 ? L.gw : L.wm;
        float* b = which == 1 ? L.gb : L.b;
        if (host_out) {
            IMPEC_CUDA_TRY(cudaMemcpy(host_out + off, w, nw * 4, cudaMemcpyDeviceToHost));
            IMPEC_CUDA_TRY(cudaMemcpy(host_out + off + nw, b, L.cout * 4, cudaMemcpyDeviceToHost));
        }
        if (host_in && which == 0) {
            IMPEC_CUDA_TRY(cudaMemcpy(L.wm, host_in + off, nw * 4, cudaMemcpyHostToDevice));
            IMPEC_CUDA_TRY(cudaMemcpy(L.b, host_in + off + nw, L.cout * 4, cudaMemcpyHostToDevice));
            std::vector<__nv_bfloat16> wb(nw);
            for (size_t i = 0; i < nw; ++i) wb[i] = __float2bfloat16(host_in[off + i]);
            IMPEC_CUDA_TRY(cudaMemcpy(L.w, wb.data(), nw * 2, cudaMemcpyHostToDevice));
        }
        off += nw + L.cout;
    }
    return IMPEC_OK;
}

// ---------------------------------------------------------------- pressure-solve hook
namespace impec {

bool learned_predicts(const impec_ctx* ctx) { return ctx->learned && ctx->learned->mode == 1; }

// Inside pressure_prepare, after x = the previous pressure and r0 = f - A x (launch only):
// features of this solve, a copy of x, and (predicting) the direction d on the fine grid.
impec_status learned_predict(impec_ctx* ctx, const double* x, const double* r0, double* d) {
    LearnedHook* H = ctx->learned;
    const int N1 = ctx->P.N1, N2 = ctx->P.N2;
    const size_t n = (size_t)N1 * N2, m = (size_t)H->h * H->w;
    cudaStream_t s = ctx->stream;
    IMPEC_CUDA_TRY(cudaMemsetAsync(H->sums, 0, 3 * sizeof(double), s));
    const double qnorm = ctx->G.dA / (ctx->P.I != 0.0 ? ctx->P.I : 1.0);
    ++ctx->nlaunch;
    k_learn_pool<<<egrid(m), 256, 0, s>>>(N1, N2, H->factor, ctx->c, ctx->K11, ctx->q, x, r0, ctx->G.mob1over4, qnorm,
                                          H->raw, H->sums);
    ++ctx->nlaunch;
    k_learn_pack<<<egrid(m), 256, 0, s>>>(m, H->raw, H->sums, H->X);
    IMPEC_CUDA_TRY(cudaGetLastError());
    IMPEC_CUDA_TRY(cudaMemcpyAsync(H->x0, x, n * 8, cudaMemcpyDeviceToDevice, s));
    if (H->mode != 1) return IMPEC_OK;
    IMPEC_TRY(net_forward(H->net, H->nb, H->X, false, s));
    ctx->nlaunch += NET_LAYERS + 6;
    ++ctx->nlaunch;
    k_learn_direction<<<egrid(n), 256, 0, s>>>(N1, N2, H->factor, H->nb.out, d);
    IMPEC_CUDA_TRY(cudaGetLastError());
    return IMPEC_OK;
}

void learned_release(impec_ctx* ctx) {
    LearnedHook* H = ctx->learned;
    if (!H) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream); else cudaDeviceSynchronize();
    free_buffers(H->nb);
    void* ps[] = {H->X, H->raw, H->T, H->x0, H->sums, ctx->lrn_r0, ctx->lrn_d, ctx->lrn_Ad, ctx->lrn_alpha};
    for (void* p : ps)
        if (p) cudaFree(p);
    ctx->lrn_r0 = ctx->lrn_d = ctx->lrn_Ad = ctx->lrn_alpha = nullptr;
    if (H->net) H->net->attached--;
    delete H;
    ctx->learned = nullptr;
}

}  // namespace impec

extern "C" impec_status impec_learned_attach(impec_ctx* ctx, impec_net* net, int factor, int mode) {
    if (!ctx) return IMPEC_ERR_ARG;
    if (!buffers_movable(ctx, "impec_learned_attach")) return IMPEC_ERR_ARG;
    if (ctx->stream) IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream)); else IMPEC_CUDA_TRY(cudaDeviceSynchronize());
    invalidate_step_graph(ctx);
    learned_release(ctx);
    if (!net || mode == 0) return IMPEC_OK;
    const int N1 = ctx->P.N1, N2 = ctx->P.N2;
    if ((mode != 1 && mode != 2) || (factor != 1 && factor != 2 && factor != 4 && factor != 8 && factor != 16) ||
        N1 % (8 * factor) != 0 || N2 % (8 * factor) != 0) {
        set_error("impec_learned_attach: mode 1 or 2, factor 1, 2, 4, 8 or 16 with N1 and N2 multiples of 8 * factor");
        return IMPEC_ERR_ARG;
    }
    if (!ctx->singular || !ctx->P.warm_start) {
        set_error("impec_learned_attach: needs warm_start and a pure-Neumann (well-driven) pressure system");
        return IMPEC_ERR_ARG;
    }
    LearnedHook* H = new LearnedHook();
    ctx->learned = H;
    H->net = net;
    net->attached++;
    H->factor = factor;
    H->mode = mode;
    H->h = N1 / factor;
    H->w = N2 / factor;
    const size_t n = (size_t)N1 * N2, m = (size_t)H->h * H->w;
    auto fail = [&](impec_status st) { learned_release(ctx); return st; };
    if (alloc_buffers(H->nb, net, 1, H->h, H->w, false) != IMPEC_OK) return fail(IMPEC_ERR_CUDA);
    if (cudaMalloc((void**)&H->X, m * NET_IN * 2) != cudaSuccess || cudaMalloc((void**)&H->raw, m * 5 * 4) != cudaSuccess ||
        cudaMalloc((void**)&H->T, m * 4) != cudaSuccess || cudaMalloc((void**)&H->x0, n * 8) != cudaSuccess ||
        cudaMalloc((void**)&H->sums, 8 * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void**)&ctx->lrn_r0, n * 8) != cudaSuccess || cudaMalloc((void**)&ctx->lrn_d, n * 8) != cudaSuccess ||
        cudaMalloc((void**)&ctx->lrn_Ad, n * 8) != cudaSuccess || cudaMalloc((void**)&ctx->lrn_alpha, sizeof(double)) != cudaSuccess)
        return fail(IMPEC_ERR_CUDA);
    cudaStream_t s = ctx->stream;
    IMPEC_CUDA_TRY(cudaMemsetAsync(H->X, 0, m * NET_IN * 2, s));
    IMPEC_CUDA_TRY(cudaMemsetAsync(H->x0, 0, n * 8, s));
    IMPEC_CUDA_TRY(cudaMemsetAsync(ctx->lrn_alpha, 0, sizeof(double), s));
    // one forward outside any capture: kernel attributes are set before the solve graph records it
    impec_status st = net_forward(net, H->nb, H->X, false, s);
    if (st != IMPEC_OK) return fail(st);
    st = check_err(net->err, s, "impec_learned_attach");
    if (st != IMPEC_OK) return fail(st);
    return IMPEC_OK;
}

// Features of the last solve (bf16 [N1/f][N2/f][8], device).
extern "C" impec_status impec_learned_features(impec_ctx* ctx, void* X) {
    if (!ctx || !ctx->learned || !X) return IMPEC_ERR_ARG;
    LearnedHook* H = ctx->learned;
    IMPEC_CUDA_TRY(cudaMemcpyAsync(X, H->X, (size_t)H->h * H->w * NET_IN * 2, cudaMemcpyDeviceToDevice, ctx->stream));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IMPEC_OK;
}

// Training target of the last solve from the resident (converged) pressure: fp32 [N1/f][N2/f], device.
extern "C" impec_status impec_learned_target(impec_ctx* ctx, float* T) {
    if (!ctx || !ctx->learned || !T) return IMPEC_ERR_ARG;
    LearnedHook* H = ctx->learned;
    const size_t m = (size_t)H->h * H->w;
    cudaStream_t s = ctx->stream;
    IMPEC_CUDA_TRY(cudaMemsetAsync(H->sums + 3, 0, 2 * sizeof(double), s));
    k_learn_target<<<egrid(m), 256, 0, s>>>(ctx->P.N1, ctx->P.N2, H->factor, ctx->p, H->x0, H->T, H->sums + 3);
    k_learn_target_scale<<<egrid(m), 256, 0, s>>>(m, H->sums + 3, H->T, T);
    IMPEC_CUDA_TRY(cudaGetLastError());
    IMPEC_CUDA_TRY(cudaStreamSynchronize(s));
    return IMPEC_OK;
}

// Step length alpha of the last solve's learned correction (0 when the prediction was
// rejected); IMPEC_ERR_CUDA if a tensor-core wait of the network gave up (the solve itself
// is unaffected: its alpha is then whatever the partial prediction gave, or 0).
extern "C" impec_status impec_learned_alpha(impec_ctx* ctx, double* alpha) {
    if (!ctx || !ctx->learned || !alpha) return IMPEC_ERR_ARG;
    IMPEC_CUDA_TRY(cudaMemcpyAsync(alpha, ctx->lrn_alpha, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    return check_err(ctx->learned->net->err, ctx->stream, "impec_learned_alpha");
}
