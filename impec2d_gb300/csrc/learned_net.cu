// Learned pressure warm start: a 4-level convolutional encoder-decoder that predicts the
// pressure of an IMPES step from [log mobility ratio, log permeability, well rate, previous
// pressure], used only as the initial guess of the pressure solve (which still converges to
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

}  // namespace impec

struct impec_net {
    impec::NetLayer L[impec::NET_LAYERS];
    impec::NetBuffers buf;
    long long step = 0;
    int num_sms = 148;
    int* err = nullptr;
    double* dscal = nullptr;  // [0] sum of squares, [1] RMS scale of the previous pressure
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

__global__ void k_pool2(const __nv_bfloat16* __restrict__ in, int B, int h, int w, int C, __nv_bfloat16* __restrict__ out) {
    const size_t n = (size_t)B * h * w * C;  // output elements, h x w = the pooled size
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        size_t t = i / C;
        const int x = (int)(t % w);
        t /= w;
        const int y = (int)(t % h), b = (int)(t / h);
        const size_t W2 = 2 * (size_t)w, r0 = ((size_t)b * 2 * h + 2 * y) * W2 + 2 * x;
        const float s = bf(in[r0 * C + c]) + bf(in[(r0 + 1) * C + c]) + bf(in[(r0 + W2) * C + c]) +
                        bf(in[(r0 + W2 + 1) * C + c]);
        out[i] = __float2bfloat16(0.25f * s);
    }
}

__global__ void k_up2(const __nv_bfloat16* __restrict__ in, int B, int h, int w, int C, __nv_bfloat16* __restrict__ out) {
    const size_t n = (size_t)B * 2 * h * 2 * w * C;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        size_t t = i / C;
        const int x = (int)(t % (2 * w));
        t /= 2 * w;
        const int y = (int)(t % (2 * h)), b = (int)(t / (2 * h));
        out[i] = in[(((size_t)b * h + y / 2) * w + x / 2) * C + c];
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

// gb[c] += sum over P pixels of dz[p][c]; each block folds a slab of pixels per channel.
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ dz, size_t P, int C, float* __restrict__ gb) {
    const int c = threadIdx.x % C, lanes = blockDim.x / C;
    if ((int)threadIdx.x >= lanes * C) return;
    const int l = threadIdx.x / C;
    float s = 0.0f;
    for (size_t p = blockIdx.x * (size_t)lanes + l; p < P; p += (size_t)gridDim.x * lanes) s += bf(dz[p * C + c]);
    atomicAdd(gb + c, s);
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

// Features of a resident IMPES state: [4 log(1 - c + M^(1/4) c) (= log of the mobility
// ratio to the resident fluid), log K, q dA / I, p / s, 0, 0, 0, 0], s = RMS of p.
__global__ void k_rms(const double* __restrict__ p, size_t n, double* out) {
    __shared__ double sh[32];
    double s = 0.0;
    for (size_t k = threadIdx.x; k < n; k += blockDim.x) s += p[k] * p[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
        out[0] = t;
        out[1] = sqrt(t / (double)n) + 1e-300;
    }
}

__global__ void k_features(size_t n, const double* __restrict__ c, const double* __restrict__ K,
                           const double* __restrict__ q, const double* __restrict__ p, double m14, double qnorm,
                           const double* __restrict__ scal, __nv_bfloat16* __restrict__ X) {
    const double inv_s = 1.0 / scal[1];
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const double ck = c[k];
        float f[NET_IN] = {(float)(4.0 * log(1.0 - ck + m14 * ck)), K ? (float)log(K[k]) : 0.0f, (float)(q[k] * qnorm),
                           (float)(p[k] * inv_s), 0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int j = 0; j < NET_IN; ++j) X[k * NET_IN + j] = __float2bfloat16(f[j]);
    }
}

__global__ void k_prediction_to_pressure(size_t n, const float* __restrict__ out, const double* __restrict__ scal,
                                         double* __restrict__ p) {
    const double s = scal[1];
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        p[k] = s * (double)out[k * NET_OUT];
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

static impec_status ensure_buffers(impec_net* net, int B, int H, int W) {
    NetBuffers& nb = net->buf;
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
        IMPEC_TRY(alloc((void**)&nb.z[l], e));
        IMPEC_TRY(alloc((void**)&nb.y[l], e));
        IMPEC_TRY(alloc((void**)&nb.dz[l], e));
    }
    const size_t P0 = level_pixels(nb, 0), P1 = level_pixels(nb, 1), P2 = level_pixels(nb, 2), P3 = level_pixels(nb, 3);
    IMPEC_TRY(alloc((void**)&nb.d1, P1 * 32 * 2));
    IMPEC_TRY(alloc((void**)&nb.d2, P2 * 64 * 2));
    IMPEC_TRY(alloc((void**)&nb.d3, P3 * 128 * 2));
    IMPEC_TRY(alloc((void**)&nb.u2, P2 * 256 * 2));
    IMPEC_TRY(alloc((void**)&nb.u1, P1 * 128 * 2));
    IMPEC_TRY(alloc((void**)&nb.u0, P0 * 64 * 2));
    IMPEC_TRY(alloc((void**)&nb.graw, P0 * 64 * 2));
    IMPEC_TRY(alloc((void**)&nb.ds0, P0 * 32 * 2));
    IMPEC_TRY(alloc((void**)&nb.ds1, P1 * 64 * 2));
    IMPEC_TRY(alloc((void**)&nb.ds2, P2 * 128 * 2));
    IMPEC_TRY(alloc((void**)&nb.out, P0 * NET_OUT * 4));
    IMPEC_TRY(alloc((void**)&nb.loss, sizeof(double)));
    return IMPEC_OK;
}

static const __nv_bfloat16* layer_input(const impec_net* net, const __nv_bfloat16* X, int l) {
    const NetBuffers& nb = net->buf;
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

static impec_status conv_forward(impec_net* net, const __nv_bfloat16* X, int l, bool train, cudaStream_t s) {
    const NetLayer& L = net->L[l];
    const NetBuffers& nb = net->buf;
    ConvArgs a = {};
    a.X = layer_input(net, X, l);
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

static impec_status net_forward(impec_net* net, const __nv_bfloat16* X, bool train, cudaStream_t s) {
    NetBuffers& nb = net->buf;
    const int B = nb.B, H = nb.H, W = nb.W;
    for (int l = 0; l < NET_LAYERS; ++l) {
        IMPEC_TRY(conv_forward(net, X, l, train, s));
        switch (l) {
            case 1: k_pool2<<<egrid(level_pixels(nb, 1) * 32), 256, 0, s>>>(nb.y[1], B, H >> 1, W >> 1, 32, nb.d1); break;
            case 3: k_pool2<<<egrid(level_pixels(nb, 2) * 64), 256, 0, s>>>(nb.y[3], B, H >> 2, W >> 2, 64, nb.d2); break;
            case 5: k_pool2<<<egrid(level_pixels(nb, 3) * 128), 256, 0, s>>>(nb.y[5], B, H >> 3, W >> 3, 128, nb.d3); break;
            case 7: k_up2<<<egrid(level_pixels(nb, 2) * 256), 256, 0, s>>>(nb.y[7], B, H >> 3, W >> 3, 256, nb.u2); break;
            case 9: k_up2<<<egrid(level_pixels(nb, 1) * 128), 256, 0, s>>>(nb.y[9], B, H >> 2, W >> 2, 128, nb.u1); break;
            case 11: k_up2<<<egrid(level_pixels(nb, 0) * 64), 256, 0, s>>>(nb.y[11], B, H >> 1, W >> 1, 64, nb.u0); break;
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
        IMPEC_TRY(launch_wgrad(nb.dz[l], layer_input(net, X, l), B, h, w, L.cin, L.cout, L.gw, net->err, net->num_sms, s));
        const size_t P = level_pixels(nb, L.level);
        k_bias_grad<<<256, 256, 0, s>>>(nb.dz[l], P, L.cout, L.gb);
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
    if (net->dscal) cudaFree(net->dscal);
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
    if (s == IMPEC_OK && cudaMalloc((void**)&net->dscal, 4 * sizeof(double)) != cudaSuccess) s = IMPEC_ERR_CUDA;
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
    IMPEC_TRY(net_forward(net, x, true, s));
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
    IMPEC_TRY(net_forward(net, x, true, s));
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
    IMPEC_TRY(net_forward(net, (const __nv_bfloat16*)X, false, s));
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

// Features of the context's resident state (c, K, q and the current p as the previous
// pressure) into X [N1][N2][8] bf16; *scale = RMS of p (the unit of the pressure channel and of
// the prediction).
extern "C" impec_status impec_net_features(impec_ctx* ctx, impec_net* net, void* X, double* scale) {
    if (!ctx || !net || !X) return IMPEC_ERR_ARG;
    const size_t n = (size_t)ctx->P.N1 * ctx->P.N2;
    cudaStream_t s = ctx->stream;
    k_rms<<<1, 1024, 0, s>>>(ctx->p, n, net->dscal);
    const double qnorm = ctx->G.dA / (ctx->P.I != 0.0 ? ctx->P.I : 1.0);
    k_features<<<egrid(n), 256, 0, s>>>(n, ctx->c, ctx->K11, ctx->q, ctx->p, ctx->G.mob1over4, qnorm, net->dscal,
                                         (__nv_bfloat16*)X);
    IMPEC_CUDA_TRY(cudaGetLastError());
    if (scale) {
        double h[2];
        IMPEC_CUDA_TRY(cudaMemcpyAsync(h, net->dscal, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        IMPEC_CUDA_TRY(cudaStreamSynchronize(s));
        *scale = h[1];
    }
    return IMPEC_OK;
}

// Learned initial guess for the next pressure solve: features of the resident state, one
// forward pass, p := RMS(p) * prediction.  The context's solve must use warm_start for the guess
// to matter; it still converges to its tolerance.
extern "C" impec_status impec_net_warm_start(impec_ctx* ctx, impec_net* net, void* workspace) {
    if (!ctx || !net || !workspace || !net_shape_ok(1, ctx->P.N1, ctx->P.N2)) {
        set_error("impec_net_warm_start: N1 and N2 must be multiples of 8");
        return IMPEC_ERR_ARG;
    }
    const int N1 = ctx->P.N1, N2 = ctx->P.N2;
    const size_t n = (size_t)N1 * N2;
    IMPEC_TRY(impec_net_features(ctx, net, workspace, nullptr));
    cudaStream_t s = ctx->stream;
    IMPEC_TRY(ensure_buffers(net, 1, N1, N2));
    IMPEC_TRY(net_forward(net, (const __nv_bfloat16*)workspace, false, s));
    k_prediction_to_pressure<<<egrid(n), 256, 0, s>>>(n, net->buf.out, net->dscal, ctx->p);
    IMPEC_CUDA_TRY(cudaGetLastError());
    return check_err(net->err, s, "impec_net_warm_start");
}
