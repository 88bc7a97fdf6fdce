// Tensor-core (tcgen05) kernels of the learned pressure warm start.
//
// GEMM core: C[M x N] (fp32) = A[M x K] (bf16, rows K-contiguous) * B[N x K]^T (bf16, rows
// K-contiguous).  One CTA of 128 threads owns a 128 x 128 output tile.  Per 64-wide K stage
// the threads copy both operand tiles into shared memory (cp.async, canonical K-major
// core-matrix layout), one thread issues four 128x128x16 tcgen05.mma into the TMEM
// accumulator and commits them to an mbarrier, and everybody waits for that mbarrier before
// the next stage overwrites the tiles.  The epilogue reads the accumulator with tcgen05.ld
// (warp w owns accumulator rows 32w .. 32w+31).  Every mbarrier wait is bounded: on timeout
// the CTA records an error, waits once more (bounded) for its own MMAs and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <cstdlib>
#include <string>

#include "learned.cuh"
#include "umma.cuh"

namespace impec {

constexpr int GB_M = 128, GB_N = 128, GB_K = 64, GB_THREADS = 128;
constexpr int GB_TILE_BYTES = GB_M * GB_K * 2;  // 16 KB per operand tile
constexpr uint32_t GB_TMEM_COLS = 128;
constexpr uint32_t GB_WAIT_TRIES = 1u << 24;

// Byte offset of element (row r, k) of a 128 x 64 bf16 tile in the K-major core-matrix layout.
__device__ __forceinline__ uint32_t tile_off(int r, int kg) { return (r >> 3) * 1024 + kg * 128 + (r & 7) * 16; }

__global__ void __launch_bounds__(GB_THREADS) k_gemm_bf16_tn(int M, int N, int K, const __nv_bfloat16* __restrict__ A,
                                                             int lda, const __nv_bfloat16* __restrict__ B, int ldb,
                                                             float* __restrict__ C, int ldc, int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char gb_smem[];
    unsigned char* sA = gb_smem;
    unsigned char* sB = gb_smem + GB_TILE_BYTES;
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * GB_M, n0 = blockIdx.x * GB_N;
    if (warp == 0) umma::tmem_alloc(&tslot, GB_TMEM_COLS);
    if (tid == 0) umma::mbar_init(&mbar, 1);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;
    const uint32_t idesc = umma::idesc_bf16_f32(GB_M, GB_N);
    const int nk = K / GB_K;
    bool ok = true;
    int issued = 0;  // stages whose MMAs were committed
    for (int kt = 0; kt < nk; ++kt) {
        for (int c = tid; c < GB_M * (GB_K / 8); c += GB_THREADS) {
            const int r = c >> 3, kg = c & 7;
            const uint32_t off = tile_off(r, kg);
            const int gm = m0 + r, gn = n0 + r;
            const __nv_bfloat16* sa = gm < M ? A + (size_t)gm * lda + (size_t)kt * GB_K + kg * 8 : A;
            const __nv_bfloat16* sb = gn < N ? B + (size_t)gn * ldb + (size_t)kt * GB_K + kg * 8 : B;
            umma::cp_async16(sA + off, sa, gm < M ? 16u : 0u);
            umma::cp_async16(sB + off, sb, gn < N ? 16u : 0u);
        }
        umma::cp_async_wait_all();
        umma::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after();
#pragma unroll
            for (int ks = 0; ks < GB_K / 16; ++ks) {  // 16 K-elements = two core matrices = 256 B
                const uint64_t ad = umma::smem_desc(umma::smem_u32(sA) + ks * 256, 128, 1024);
                const uint64_t bd = umma::smem_desc(umma::smem_u32(sB) + ks * 256, 128, 1024);
                umma::mma_bf16(tmem, ad, bd, idesc, (kt > 0 || ks > 0) ? 1u : 0u);
            }
            umma::commit(&mbar);
        }
        issued = kt + 1;
        const bool done = umma::mbar_wait(&mbar, (uint32_t)(kt & 1), GB_WAIT_TRIES);
        ok = __syncthreads_and(done) != 0;
        if (!ok) break;
        umma::fence_after();
    }
    if (ok && nk > 0) {
#pragma unroll 1
        for (int cb = 0; cb < GB_N / 32; ++cb) {
            float v[32];
            umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cb * 32), v);
            const int gm = m0 + warp * 32 + lane;
            if (gm < M) {
#pragma unroll
                for (int k = 0; k < 32; ++k) {
                    const int gn = n0 + cb * 32 + k;
                    if (gn < N) C[(size_t)gm * ldc + gn] = v[k];
                }
            }
        }
    } else if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        // the last committed stage may still be running: wait for it once more before freeing TMEM
        umma::mbar_wait(&mbar, (uint32_t)((issued - 1) & 1), GB_WAIT_TRIES);
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    if (warp == 0) umma::tmem_free(tmem, GB_TMEM_COLS);
}

// ---------------------------------------------------------------- 3x3 convolution (implicit GEMM)
// Activations are NHWC bf16 with C a multiple of 8.  Weights are [cout rows][Kp] bf16 with
// k = tap * cin + c (tap = 3 * (dy + 1) + (dx + 1)), Kp = 9 cin rounded up to 64, zero beyond.
// GEMM rows are the B*H*W output pixels (128 per CTA), columns the output channels (BN per
// CTA), K the taps x input channels: each 16-byte chunk of the A tile is one tap's 8 channels
// of one pixel, copied from the neighbour (y + s dy, x + s dx) or zero-filled outside the image
// (s = +1 forward; s = -1 gives the transposed convolution of the input gradient, with the
// weights rearranged by k_conv_wt_transpose).  Epilogue per (pixel, channel):
//   v = acc + bias;  then either  Z = v, Y = act(v) (+ skip)          (forward)
//                    or           Y = (v + add) * gelu'(gz)            (input gradient)

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// Epilogue of the convolution kernels, on NW (4 or 8) warps: warp w reads TMEM lanes
// 32 (w % 4) .. + 31 (one output pixel per thread) and the 16-column groups w / 4,
// w / 4 + NW / 4, ... of the accumulator.
template <int BN, int NW>
__device__ __forceinline__ void conv_epilogue(const ConvArgs& a, uint32_t tmem, int m0, int n0, int warp, int lane,
                                              int M) {
    const int quarter = warp & 3, part = warp >> 2;
    const int m = m0 + quarter * 32 + lane;
#pragma unroll 1
    for (int g = part; g < (BN + 15) / 16; g += NW / 4) {
        float v[16];
        umma::tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(g * 16), v);
        if (m >= M) continue;
        const size_t row = (size_t)m * a.cout;
        const int nb = n0 + g * 16;
        if (nb + 16 <= a.cout && (a.cout & 7) == 0) {  // 16 whole channels: 16-byte accesses
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                float z[8], y[8];
                const size_t o = row + nb + 8 * q;
#pragma unroll
                for (int k = 0; k < 8; ++k) z[k] = v[8 * q + k] + (a.bias ? a.bias[nb + 8 * q + k] : 0.0f);
                if (a.gz) {
                    __align__(16) __nv_bfloat16 g8[8], ad8[8], o8[8];
                    *reinterpret_cast<uint4*>(g8) = *reinterpret_cast<const uint4*>(a.gz + o);
                    if (a.add) *reinterpret_cast<uint4*>(ad8) = *reinterpret_cast<const uint4*>(a.add + o);
                    if (a.R) {
#pragma unroll
                        for (int k = 0; k < 8; ++k) o8[k] = __float2bfloat16(z[k]);
                        *reinterpret_cast<uint4*>(a.R + o) = *reinterpret_cast<const uint4*>(o8);
                    }
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        float t = z[k];
                        if (a.add) t += __bfloat162float(ad8[k]);
                        y[k] = t * gelu_grad(__bfloat162float(g8[k]));
                    }
                } else {
                    if (a.Z) {
                        __align__(16) __nv_bfloat16 o8[8];
#pragma unroll
                        for (int k = 0; k < 8; ++k) o8[k] = __float2bfloat16(z[k]);
                        *reinterpret_cast<uint4*>(a.Z + o) = *reinterpret_cast<const uint4*>(o8);
                    }
                    __align__(16) __nv_bfloat16 s8[8];
                    if (a.skip) *reinterpret_cast<uint4*>(s8) = *reinterpret_cast<const uint4*>(a.skip + o);
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        y[k] = a.act ? gelu_f(z[k]) : z[k];
                        if (a.skip) y[k] += __bfloat162float(s8[k]);
                    }
                }
                if (a.Y) {
                    __align__(16) __nv_bfloat16 o8[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) o8[k] = __float2bfloat16(y[k]);
                    *reinterpret_cast<uint4*>(a.Y + o) = *reinterpret_cast<const uint4*>(o8);
                }
                if (a.Yf) {
#pragma unroll
                    for (int k = 0; k < 8; ++k) a.Yf[o + k] = y[k];
                }
            }
            continue;
        }
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const int n = nb + k;
            if (n >= a.cout || g * 16 + k >= BN) continue;
            float z = v[k] + (a.bias ? a.bias[n] : 0.0f);
            if (a.gz) {  // input gradient: (acc + add) * gelu'(gz)
                if (a.R) a.R[row + n] = __float2bfloat16(z);
                if (a.add) z += __bfloat162float(a.add[row + n]);
                z *= gelu_grad(__bfloat162float(a.gz[row + n]));
                if (a.Y) a.Y[row + n] = __float2bfloat16(z);
                if (a.Yf) a.Yf[row + n] = z;
                continue;
            }
            if (a.Z) a.Z[row + n] = __float2bfloat16(z);
            float y = a.act ? gelu_f(z) : z;
            if (a.skip) y += __bfloat162float(a.skip[row + n]);
            if (a.Y) a.Y[row + n] = __float2bfloat16(y);
            if (a.Yf) a.Yf[row + n] = y;
        }
    }
}

// Warp-specialised pipeline over CV_STAGES shared-memory stages.  Warps 0-3 copy the operand
// tiles with cp.async; each copy arrives on the stage's "full" mbarrier when it lands
// (cp.async.mbarrier.arrive.noinc, 128 arrivals per phase).  One thread of warp 4 waits for a
// full stage, issues its four MMAs and commits them to the stage's "empty" mbarrier, which the
// copiers wait for before refilling the slot; after the last stage it commits to "done".  Warps
// 0-3 then read the accumulator (warp w owns TMEM lanes 32w .. 32w + 31).  Thread t of the
// copiers always copies chunk t % 8 of rows t / 8 + 16 i, so it resolves its pixels once.
constexpr int CV_STAGES = 4, CV_COPIERS = 128, CV_THREADS = 160;

template <int BN>
constexpr int conv_smem_bytes() { return CV_STAGES * (GB_TILE_BYTES + BN * GB_K * 2) + 1024; }

template <int BN>
__global__ void __launch_bounds__(CV_THREADS) k_conv3x3(ConvArgs a) {
    extern __shared__ __align__(1024) unsigned char cv_smem[];
    constexpr int B_BYTES = BN * GB_K * 2, STAGE = GB_TILE_BYTES + B_BYTES;
    constexpr int AR = GB_M * 8 / CV_COPIERS, BR = BN * 8 / CV_COPIERS;  // rows per copier (A: 8, B: BN / 16)
    __shared__ uint64_t full[CV_STAGES], empty[CV_STAGES], done;
    __shared__ uint32_t tslot;
    __shared__ volatile int fail;
    constexpr uint32_t TCOLS = BN < 32 ? 32 : BN;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int M = a.B * a.H * a.W_;
    const int m0 = blockIdx.y * GB_M, n0 = blockIdx.x * BN;
    if (warp == 0) umma::tmem_alloc(&tslot, TCOLS);
    if (tid == 0) {
        for (int st = 0; st < CV_STAGES; ++st) {
            umma::mbar_init(&full[st], CV_COPIERS);
            umma::mbar_init(&empty[st], 1);
        }
        umma::mbar_init(&done, 1);
        fail = 0;
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;
    const int nk = a.Kp / GB_K, K9 = 9 * a.cin;
    if (warp < 4) {  // copiers
        const int kg = tid & 7, r0 = tid >> 3;
        int pix[AR], py[AR], px[AR];
#pragma unroll
        for (int i = 0; i < AR; ++i) {
            const int m = m0 + r0 + 16 * i;
            pix[i] = m < M ? m : -1;
            const int mm = m < M ? m : 0;
            px[i] = mm % a.W_;
            py[i] = (mm / a.W_) % a.H;
        }
        for (int kt = 0; kt < nk; ++kt) {
            const int slot = kt % CV_STAGES, use = kt / CV_STAGES;
            if (use > 0 && !umma::mbar_wait(&empty[slot], (uint32_t)((use - 1) & 1), GB_WAIT_TRIES)) {
                fail = 1;
                break;
            }
            unsigned char* sA = cv_smem + slot * STAGE;
            unsigned char* sB = sA + GB_TILE_BYTES;
            const int k0 = kt * GB_K + kg * 8;
            const bool kin = k0 < K9;
            const int tap = kin ? k0 / a.cin : 0, ch = k0 - tap * a.cin;
            const int dy = a.tapsign * (tap / 3 - 1), dx = a.tapsign * (tap % 3 - 1);
            const long long shift = ((long long)dy * a.W_ + dx) * a.cin + ch;
#pragma unroll
            for (int i = 0; i < AR; ++i) {
                const int yy = py[i] + dy, xx = px[i] + dx;
                const bool in = kin && pix[i] >= 0 && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W_;
                const __nv_bfloat16* src = in ? a.X + (long long)pix[i] * a.cin + shift : a.X;
                umma::cp_async16(sA + tile_off(r0 + 16 * i, kg), src, in ? 16u : 0u);
            }
#pragma unroll
            for (int i = 0; i < BR; ++i) {
                const int n = n0 + r0 + 16 * i;
                const bool in = n < a.cout;
                umma::cp_async16(sB + tile_off(r0 + 16 * i, kg),
                                 in ? a.W + (size_t)n * a.Kp + (size_t)kt * GB_K + kg * 8 : a.W, in ? 16u : 0u);
            }
            umma::cp_async_mbar_arrive(&full[slot]);
        }
        umma::cp_async_wait_all();
    } else {  // warp 4: one thread issues the MMAs
        if (lane == 0) {
            const uint32_t idesc = umma::idesc_bf16_f32(GB_M, BN);
            for (int kt = 0; kt < nk; ++kt) {
                const int slot = kt % CV_STAGES, use = kt / CV_STAGES;
                if (!umma::mbar_wait(&full[slot], (uint32_t)(use & 1), GB_WAIT_TRIES)) {
                    fail = 1;
                    break;
                }
                umma::fence_proxy_async();  // the copies, acquired through the mbarrier, to the tensor core
                umma::fence_after();
                const uint32_t base = umma::smem_u32(cv_smem + slot * STAGE);
#pragma unroll
                for (int ks = 0; ks < GB_K / 16; ++ks) {
                    const uint64_t ad = umma::smem_desc(base + ks * 256, 128, 1024);
                    const uint64_t bd = umma::smem_desc(base + GB_TILE_BYTES + ks * 256, 128, 1024);
                    umma::mma_bf16(tmem, ad, bd, idesc, (kt > 0 || ks > 0) ? 1u : 0u);
                }
                umma::commit(&empty[slot]);
            }
            umma::commit(&done);  // every MMA issued above has completed
        }
        __syncwarp();
    }
    // all MMAs issued (or given up); the accumulator is final once "done" completes
    const bool fin = warp < 4 ? umma::mbar_wait(&done, 0u, GB_WAIT_TRIES) : true;
    const bool ok = __syncthreads_and(fin) != 0 && fail == 0;
    if (ok && warp < 4) {
        umma::fence_after();
        conv_epilogue<BN, 4>(a, tmem, m0, n0, warp, lane, M);
    }
    if (!ok && tid == 0) atomicExch(a.err, 1);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    if (warp == 0) umma::tmem_free(tmem, TCOLS);
}

// TMA variant for cin a multiple of 32 and tiles of whole image rows (see conv_tma_plan): one
// K stage is one tap's KS-channel slice (KS = 64: 128-byte swizzle; KS = 32: 64-byte swizzle).
// The activation tile of a stage is one 4D box (KS channels x wbox x hbox x bbox pixels = the
// 128 output pixels of the tile) at the tap's offset, zero-filled outside the image by the
// TMA; the weight tile is one 2D box.
//
// Persistent: each CTA walks the tiles blockIdx.x, blockIdx.x + gridDim.x, ... with the
// accumulator double-buffered in TMEM, so that the loads and MMAs of tile i+1 overlap the
// epilogue of tile i.  Roles: lane 0 of the producer warp issues both loads of every stage on
// the stage's "full" mbarrier (expected bytes); lane 0 of the MMA warp waits for the accumulator buffer
// to be free ("tmem_empty", one arrival per epilogue warp), issues the MMAs of each stage,
// commits them to the stage's "empty" mbarrier and, after a tile's last stage, to the
// buffer's "tmem_full"; the epilogue warps wait for "tmem_full", run the epilogue and release the
// buffer.  Stages: as many as fit in 200 KB (at most 8).  Stage and buffer uses are counted
// across tiles, which gives every wait its phase parity.  (Warp numbers: the epilogue runs on
// warps 0 .. EPI_WARPS - 1, two per TMEM lane quarter; the producer is warp EPI_WARPS and the
// MMA issuer warp EPI_WARPS + 1.)
constexpr int CT_THREADS = 320, CT_MAX_STAGES = 8, EPI_WARPS = 8;

struct ConvTmaPlan {
    int ks, stages, wbox, hbox, bbox;
};

template <int BN, int KS>
__global__ void __launch_bounds__(CT_THREADS) k_conv3x3_tma(const __grid_constant__ CUtensorMap tx,
                                                            const __grid_constant__ CUtensorMap tw, ConvArgs a,
                                                            int stages) {
    extern __shared__ __align__(1024) unsigned char ct_smem[];
    constexpr int A_BYTES = GB_M * KS * 2, B_BYTES = BN * KS * 2, STAGE = A_BYTES + B_BYTES;
    constexpr uint32_t TC = BN < 32 ? 32 : BN;  // TMEM columns of one accumulator buffer
    __shared__ uint64_t full[CT_MAX_STAGES], empty[CT_MAX_STAGES], tfull[2], tempty[2], done;
    __shared__ uint32_t tslot;
    __shared__ volatile int fail, tma_issued;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int M = a.B * a.H * a.W_;
    const int mt = (M + GB_M - 1) / GB_M, nt = (a.cout + BN - 1) / BN, tiles = mt * nt;
    unsigned char* base = ct_smem + ((1024 - (umma::smem_u32(ct_smem) & 1023)) & 1023);  // 1024-byte aligned
    if (warp == 0) umma::tmem_alloc(&tslot, 2 * TC);
    if (tid == 0) {
        for (int st = 0; st < stages; ++st) {
            umma::mbar_init(&full[st], 1);
            umma::mbar_init(&empty[st], 1);
        }
        for (int b = 0; b < 2; ++b) {
            umma::mbar_init(&tfull[b], 1);
            umma::mbar_init(&tempty[b], EPI_WARPS);
        }
        umma::mbar_init(&done, 1);
        fail = 0;
        tma_issued = 0;
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;
    const int cs = a.cin / KS, nk = 9 * cs, hw = a.H * a.W_;
    if (warp == EPI_WARPS) {
        if (lane == 0) {  // TMA producer
            int g = 0;
            for (int t = blockIdx.x; t < tiles && !fail; t += gridDim.x) {
                const int m0 = (t / nt) * GB_M, n0 = (t % nt) * BN;
                const int b0 = m0 / hw, rem = m0 - b0 * hw, y0 = rem / a.W_, x0 = rem - y0 * a.W_;
                for (int kt = 0; kt < nk; ++kt, ++g) {
                    const int slot = g % stages, use = g / stages;
                    if (use > 0 && !umma::mbar_wait(&empty[slot], (uint32_t)((use - 1) & 1), GB_WAIT_TRIES)) {
                        fail = 1;
                        break;
                    }
                    const int tap = kt / cs, c0 = (kt - tap * cs) * KS;
                    const int dy = a.tapsign * (tap / 3 - 1), dx = a.tapsign * (tap % 3 - 1);
                    unsigned char* sA = base + slot * STAGE;
                    umma::mbar_expect_tx(&full[slot], (uint32_t)STAGE);
                    umma::tma_load_4d(sA, &tx, c0, x0 + dx, y0 + dy, b0, &full[slot]);
                    umma::tma_load_2d(sA + A_BYTES, &tw, tap * a.cin + c0, n0, &full[slot]);
                    tma_issued = g + 1;
                }
            }
        }
        __syncwarp();
    } else if (warp == EPI_WARPS + 1) {
        if (lane == 0) {  // MMA issuer
            const uint32_t idesc = umma::idesc_bf16_f32(GB_M, BN);
            int g = 0, i = 0;
            for (int t = blockIdx.x; t < tiles && !fail; t += gridDim.x, ++i) {
                const int buf = i & 1, buse = i >> 1;
                if (buse > 0 && !umma::mbar_wait(&tempty[buf], (uint32_t)((buse - 1) & 1), GB_WAIT_TRIES)) {
                    fail = 1;
                    break;
                }
                umma::fence_after();
                const uint32_t acc = tmem + (uint32_t)buf * TC;
                for (int kt = 0; kt < nk; ++kt, ++g) {
                    const int slot = g % stages, use = g / stages;
                    if (!umma::mbar_wait(&full[slot], (uint32_t)(use & 1), GB_WAIT_TRIES)) {
                        fail = 1;
                        break;
                    }
                    umma::fence_after();
                    const uint32_t sa = umma::smem_u32(base + slot * STAGE);
#pragma unroll
                    for (int ks = 0; ks < KS / 16; ++ks) {
                        const uint64_t ad = umma::smem_desc_sw(sa + ks * 32, KS * 2);
                        const uint64_t bd = umma::smem_desc_sw(sa + A_BYTES + ks * 32, KS * 2);
                        umma::mma_bf16(acc, ad, bd, idesc, (kt > 0 || ks > 0) ? 1u : 0u);
                    }
                    umma::commit(&empty[slot]);
                }
                if (fail) break;
                umma::commit(&tfull[buf]);
            }
            if (fail)  // let the loads already issued land before the CTA ends (bounded)
                for (int j = g; j < tma_issued; ++j)
                    umma::mbar_wait(&full[j % stages], (uint32_t)((j / stages) & 1), GB_WAIT_TRIES >> 4);
            umma::commit(&done);  // completes once every MMA issued above has
            umma::mbar_wait(&done, 0u, GB_WAIT_TRIES);
        }
        __syncwarp();
    } else {  // warps 0 .. EPI_WARPS - 1: epilogue
        int i = 0;
        for (int t = blockIdx.x; t < tiles && !fail; t += gridDim.x, ++i) {
            const int buf = i & 1, buse = i >> 1;
            if (!umma::mbar_wait(&tfull[buf], (uint32_t)(buse & 1), GB_WAIT_TRIES)) {
                fail = 1;
                break;
            }
            umma::fence_after();
            conv_epilogue<BN, EPI_WARPS>(a, tmem + (uint32_t)buf * TC, (t / nt) * GB_M, (t % nt) * BN, warp, lane, M);
            umma::fence_before();
            __syncwarp();
            if (lane == 0) umma::mbar_arrive(&tempty[buf]);
        }
    }
    __syncthreads();
    if (fail && tid == 0) atomicExch(a.err, 1);
    umma::fence_after();
    if (warp == 0) umma::tmem_free(tmem, 2 * TC);
}

// Halo variant for cin = 8, 32 or 64 and W a multiple of 128 (a tile is 128 pixels of one image
// row).  CIN is the channel width of the boxes: 64, 32, or 16 for 8-channel inputs, whose box
// channels 8..15 lie outside the tensor and load as zeros (they meet the next tap's weights in
// the MMA, which therefore add nothing).  Per tile, one 4D TMA box brings the halo: CIN channels x 130 pixels (x0 - 1 .. x0 + 128)
// x 3 rows (y0 - 1 .. y0 + 1), zero-filled outside the image, as 390 swizzled rows of CIN * 2
// bytes.  The A operand of tap (dy, dx) is the 128 rows starting at row (1 + dy) * 130 + 1 + dx
// of that box: the descriptor's start moves there, and since the hardware applies the swizzle
// on absolute shared-memory addresses (base offset 0), no copy or realignment is needed.  One
// load serves all 9 taps: 390 instead of 9 x 128 TMA rows per tile.  Each CTA keeps the weights
// of its BN output channels for all 9 taps resident (loaded once) and walks the tiles
// blockIdx.x / nt, + gridDim.x / nt, ...; the halo and the TMEM accumulator are
// double-buffered so that the next tile's load and MMAs overlap the epilogue.  Roles as in
// k_conv3x3_tma (producer, MMA issuer and EPI_WARPS epilogue warps).
constexpr int CH_THREADS = 320, CH_PIX = 130, CH_ROWS = 3 * CH_PIX;

template <int CIN>
__host__ __device__ constexpr int halo_bytes() { return (CH_ROWS * CIN * 2 + 1023) / 1024 * 1024; }
template <int BN, int CIN>
__host__ __device__ constexpr int halo_smem() { return 9 * BN * CIN * 2 + 2 * halo_bytes<CIN>() + 1024; }

template <int BN, int CIN>
__global__ void __launch_bounds__(CH_THREADS) k_conv3x3_halo(const __grid_constant__ CUtensorMap tx,
                                                             const __grid_constant__ CUtensorMap tw, ConvArgs a) {
    extern __shared__ __align__(1024) unsigned char ch_smem[];
    constexpr int ROWB = CIN * 2, W_TAP = BN * ROWB, HALO = halo_bytes<CIN>();
    constexpr uint32_t TC = BN < 32 ? 32 : BN;
    __shared__ uint64_t wfull, hfull[2], hempty[2], tfull[2], tempty[2], done;
    __shared__ uint32_t tslot;
    __shared__ volatile int fail, halo_issued;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int M = a.B * a.H * a.W_, mt = M / GB_M, nt = (a.cout + BN - 1) / BN;
    const int n_tile = blockIdx.x % nt, g0 = blockIdx.x / nt, G = gridDim.x / nt, n0 = n_tile * BN;
    unsigned char* base = ch_smem + ((1024 - (umma::smem_u32(ch_smem) & 1023)) & 1023);
    unsigned char* sW = base;                       // 9 taps x BN rows x ROWB
    unsigned char* sH = base + 9 * W_TAP;           // 2 halo buffers (9 * W_TAP is a multiple of 1024)
    if (warp == 0) umma::tmem_alloc(&tslot, 2 * TC);
    if (tid == 0) {
        umma::mbar_init(&wfull, 1);
        for (int b = 0; b < 2; ++b) {
            umma::mbar_init(&hfull[b], 1);
            umma::mbar_init(&hempty[b], 1);
            umma::mbar_init(&tfull[b], 1);
            umma::mbar_init(&tempty[b], EPI_WARPS);
        }
        umma::mbar_init(&done, 1);
        fail = 0;
        halo_issued = 0;
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;
    const int hw = a.H * a.W_;
    if (warp == EPI_WARPS) {
        if (lane == 0) {  // TMA producer: weights once, then one halo box per tile
            umma::mbar_expect_tx(&wfull, (uint32_t)(9 * W_TAP));
            for (int tap = 0; tap < 9; ++tap)
                umma::tma_load_2d(sW + tap * W_TAP, &tw, tap * a.cin, n0, &wfull);
            int i = 0;
            for (int t = g0; t < mt && !fail; t += G, ++i) {
                const int buf = i & 1, use = i >> 1;
                if (use > 0 && !umma::mbar_wait(&hempty[buf], (uint32_t)((use - 1) & 1), GB_WAIT_TRIES)) {
                    fail = 1;
                    break;
                }
                const int m0 = t * GB_M, b0 = m0 / hw, rem = m0 - b0 * hw, y0 = rem / a.W_, x0 = rem - y0 * a.W_;
                umma::mbar_expect_tx(&hfull[buf], (uint32_t)(CH_ROWS * ROWB));
                umma::tma_load_4d(sH + buf * HALO, &tx, 0, x0 - 1, y0 - 1, b0, &hfull[buf]);
                halo_issued = i + 1;
            }
        }
        __syncwarp();
    } else if (warp == EPI_WARPS + 1) {
        if (lane == 0) {  // MMA issuer
            const uint32_t idesc = umma::idesc_bf16_f32(GB_M, BN);
            bool wok = umma::mbar_wait(&wfull, 0u, GB_WAIT_TRIES);
            if (!wok) fail = 1;
            int i = 0;
            for (int t = g0; t < mt && !fail; t += G, ++i) {
                const int buf = i & 1, use = i >> 1;
                if (!umma::mbar_wait(&hfull[buf], (uint32_t)(use & 1), GB_WAIT_TRIES) ||
                    (use > 0 && !umma::mbar_wait(&tempty[buf], (uint32_t)((use - 1) & 1), GB_WAIT_TRIES))) {
                    fail = 1;
                    break;
                }
                umma::fence_after();
                const uint32_t acc = tmem + (uint32_t)buf * TC;
                const uint32_t h0 = umma::smem_u32(sH + buf * HALO), w0 = umma::smem_u32(sW);
#pragma unroll 1
                for (int tap = 0; tap < 9; ++tap) {
                    const int dy = a.tapsign * (tap / 3 - 1), dx = a.tapsign * (tap % 3 - 1);
                    const uint32_t row0 = (uint32_t)((1 + dy) * CH_PIX + 1 + dx);
#pragma unroll
                    for (int ks = 0; ks < CIN / 16; ++ks) {
                        const uint64_t ad = umma::smem_desc_sw(h0 + row0 * ROWB + ks * 32, ROWB);
                        const uint64_t bd = umma::smem_desc_sw(w0 + tap * W_TAP + ks * 32, ROWB);
                        umma::mma_bf16(acc, ad, bd, idesc, (tap > 0 || ks > 0) ? 1u : 0u);
                    }
                }
                umma::commit(&hempty[buf]);
                umma::commit(&tfull[buf]);
            }
            if (fail) {  // let the halo loads already issued land (bounded)
                for (int j = i; j < halo_issued; ++j)
                    umma::mbar_wait(&hfull[j & 1], (uint32_t)((j >> 1) & 1), GB_WAIT_TRIES >> 4);
                if (!wok) umma::mbar_wait(&wfull, 0u, GB_WAIT_TRIES >> 4);
            }
            umma::commit(&done);
            umma::mbar_wait(&done, 0u, GB_WAIT_TRIES);
        }
        __syncwarp();
    } else {  // warps 0 .. EPI_WARPS - 1: epilogue
        int i = 0;
        for (int t = g0; t < mt && !fail; t += G, ++i) {
            const int buf = i & 1, use = i >> 1;
            if (!umma::mbar_wait(&tfull[buf], (uint32_t)(use & 1), GB_WAIT_TRIES)) {
                fail = 1;
                break;
            }
            umma::fence_after();
            conv_epilogue<BN, EPI_WARPS>(a, tmem + (uint32_t)buf * TC, t * GB_M, n0, warp, lane, M);
            umma::fence_before();
            __syncwarp();
            if (lane == 0) umma::mbar_arrive(&tempty[buf]);
        }
    }
    __syncthreads();
    if (fail && tid == 0) atomicExch(a.err, 1);
    umma::fence_after();
    if (warp == 0) umma::tmem_free(tmem, 2 * TC);
}

// Weights of the input-gradient convolution: Wd[ci][tap * cout + co] = W[co][tap * cin + ci],
// Kd = 9 cout rounded up to 64.  The taps keep their index: k_conv3x3 with tapsign = -1 reads
// the neighbour at -d, which is the transposed convolution.
__global__ void k_conv_wt_transpose(const __nv_bfloat16* __restrict__ W, int cin, int cout, int Kp,
                                    __nv_bfloat16* __restrict__ Wd, int Kd) {
    const size_t n = (size_t)cin * Kd;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int ci = (int)(idx / Kd), k = (int)(idx % Kd);
        __nv_bfloat16 v = __float2bfloat16(0.0f);
        if (k < 9 * cout) {
            const int tap = k / cout, co = k % cout;
            v = W[(size_t)co * Kp + (size_t)tap * cin + ci];
        }
        Wd[idx] = v;
    }
}

// Weight gradient: dW[co][tap * cin + ci] += sum over pixels p of dZ[p][co] * X[p + d(tap)][ci].
// GEMM rows: output channels (128 per CTA), columns: (tap, ci) pairs (128 per CTA), K: pixels,
// split over blockIdx.z (each CTA adds its partial sums with fp32 atomics).  Both operands are
// channel-contiguous in memory, so the staging transposes them: every 16-byte load (8 channels
// of one pixel) is scattered into 8 rows of the K-major tile.
__global__ void __launch_bounds__(GB_THREADS) k_conv_wgrad(const __nv_bfloat16* __restrict__ dZ,
                                                           const __nv_bfloat16* __restrict__ X, int B, int H, int W_,
                                                           int cin, int cout, int Kp, int pix_per_split,
                                                           float* __restrict__ dW, int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char wg_smem[];
    unsigned char* sA = wg_smem;
    unsigned char* sB = wg_smem + GB_TILE_BYTES;
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int P = B * H * W_, K9 = 9 * cin;
    const int co0 = blockIdx.y * GB_M, k0 = blockIdx.x * GB_N;
    const int p_begin = blockIdx.z * pix_per_split;
    const int p_end = p_begin + pix_per_split < P ? p_begin + pix_per_split : P;
    if (warp == 0) umma::tmem_alloc(&tslot, GB_TMEM_COLS);
    if (tid == 0) umma::mbar_init(&mbar, 1);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;
    const uint32_t idesc = umma::idesc_bf16_f32(GB_M, GB_N);
    const int nk = p_end > p_begin ? (p_end - p_begin + GB_K - 1) / GB_K : 0;
    bool ok = true;
    int issued = 0;
    __nv_bfloat16* a16 = reinterpret_cast<__nv_bfloat16*>(sA);
    __nv_bfloat16* b16 = reinterpret_cast<__nv_bfloat16*>(sB);
    for (int kt = 0; kt < nk; ++kt) {
        const int pb = p_begin + kt * GB_K;
        // A: rows co (128), K = 64 pixels.  One task = 8 channels of one pixel (16 bytes).
        for (int c = tid; c < (GB_M / 8) * GB_K; c += GB_THREADS) {
            const int cg = c / GB_K, kk = c % GB_K, p = pb + kk, co = co0 + cg * 8;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (p < p_end && co < cout) v = *reinterpret_cast<const uint4*>(dZ + (size_t)p * cout + co);
            const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&v);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int r = cg * 8 + q;  // tile row
                a16[(tile_off(r, kk >> 3) >> 1) + (kk & 7)] = e[q];
            }
        }
        // B: rows n = (tap, ci) (128), K = 64 pixels.  One task = 8 input channels of one tap.
        for (int c = tid; c < (GB_N / 8) * GB_K; c += GB_THREADS) {
            const int ng = c / GB_K, kk = c % GB_K, p = pb + kk, n = k0 + ng * 8;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (p < p_end && n < K9) {
                const int tap = n / cin, ci = n - tap * cin;
                const int x = p % W_, t = p / W_, y = t % H, b = t / H;
                const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
                if (yy >= 0 && yy < H && xx >= 0 && xx < W_)
                    v = *reinterpret_cast<const uint4*>(X + (((size_t)b * H + yy) * W_ + xx) * cin + ci);
            }
            const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&v);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int r = ng * 8 + q;
                b16[(tile_off(r, kk >> 3) >> 1) + (kk & 7)] = e[q];
            }
        }
        umma::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after();
#pragma unroll
            for (int ks = 0; ks < GB_K / 16; ++ks) {
                const uint64_t ad = umma::smem_desc(umma::smem_u32(sA) + ks * 256, 128, 1024);
                const uint64_t bd = umma::smem_desc(umma::smem_u32(sB) + ks * 256, 128, 1024);
                umma::mma_bf16(tmem, ad, bd, idesc, (kt > 0 || ks > 0) ? 1u : 0u);
            }
            umma::commit(&mbar);
        }
        issued = kt + 1;
        const bool done = umma::mbar_wait(&mbar, (uint32_t)(kt & 1), GB_WAIT_TRIES);
        ok = __syncthreads_and(done) != 0;
        if (!ok) break;
        umma::fence_after();
    }
    if (ok && nk > 0) {
        const int co = co0 + warp * 32 + lane;
#pragma unroll 1
        for (int cb = 0; cb < GB_N / 32; ++cb) {
            float v[32];
            umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cb * 32), v);
            if (co >= cout) continue;
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                const int k = k0 + cb * 32 + q;
                if (k < K9) atomicAdd(dW + (size_t)co * Kp + k, v[q]);
            }
        }
    } else if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        umma::mbar_wait(&mbar, (uint32_t)((issued - 1) & 1), GB_WAIT_TRIES);
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    if (warp == 0) umma::tmem_free(tmem, GB_TMEM_COLS);
}

// Weight gradient on TMA boxes, both operands MN-major (no transposing stores).  GEMM rows:
// output channels (128 per CTA), columns: (tap, ci) pairs (128 per CTA), K: 64 pixels per
// stage over the CTA's slice of the pixels (blockIdx.z), partial sums added to dW with fp32
// atomics.  Per stage: A = 128 / CA boxes of dZ [pixels][cout] (CA channels x 64 pixels, rows =
// pixels, CA-element MN blocks), B = 128 / CB boxes of the layer input at one tap's offset (CB
// channels x the stage's 64 pixels as a 4D box, zero-filled outside the image; column blocks
// beyond 9 cin point past the channels and load zeros).  CA, CB = 64 (128-byte swizzle) or 32
// (64-byte).  8-channel operands use 32-channel boxes, whose channels 8..31 lie outside the
// tensor and load as zeros: for cout = 8 these are rows of zeros, for cin = 8 each column block
// holds one tap (columns c >= cin of a block are discarded).  Roles as in k_conv3x3_tma, one
// tile per CTA.
constexpr int WG_THREADS = 192, WG_STAGES = 6, WG_PIX = 64;

template <int CA, int CB>
__global__ void __launch_bounds__(WG_THREADS) k_conv_wgrad_tma(const __grid_constant__ CUtensorMap tz,
                                                               const __grid_constant__ CUtensorMap tx, int H, int W_,
                                                               int cin, int cout, int Kp, int P, int pix_per_split,
                                                               float* __restrict__ dW, int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char wt_smem[];
    constexpr int A_BLK = WG_PIX * CA * 2, B_BLK = WG_PIX * CB * 2;  // bytes of one MN block
    constexpr int A_BYTES = 128 / CA * A_BLK, STAGE = A_BYTES + 128 / CB * B_BLK;
    __shared__ uint64_t full[WG_STAGES], empty[WG_STAGES], done;
    __shared__ uint32_t tslot;
    __shared__ volatile int fail, tma_issued;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int co0 = blockIdx.y * 128, k0 = blockIdx.x * 128;
    const int p_begin = blockIdx.z * pix_per_split;
    const int p_end = p_begin + pix_per_split < P ? p_begin + pix_per_split : P;
    const int nk = p_end > p_begin ? (p_end - p_begin + WG_PIX - 1) / WG_PIX : 0;
    unsigned char* base = wt_smem + ((1024 - (umma::smem_u32(wt_smem) & 1023)) & 1023);
    if (warp == 0) umma::tmem_alloc(&tslot, 128);
    if (tid == 0) {
        for (int st = 0; st < WG_STAGES; ++st) {
            umma::mbar_init(&full[st], 1);
            umma::mbar_init(&empty[st], 1);
        }
        umma::mbar_init(&done, 1);
        fail = 0;
        tma_issued = 0;
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;
    if (warp == 4) {
        if (lane == 0) {  // TMA producer
            const int hw = H * W_;
            for (int kt = 0; kt < nk; ++kt) {
                const int slot = kt % WG_STAGES, use = kt / WG_STAGES;
                if (use > 0 && !umma::mbar_wait(&empty[slot], (uint32_t)((use - 1) & 1), GB_WAIT_TRIES)) {
                    fail = 1;
                    break;
                }
                const int p0 = p_begin + kt * WG_PIX, b0 = p0 / hw, rem = p0 - b0 * hw, y0 = rem / W_,
                          x0 = rem - y0 * W_;
                unsigned char* sA = base + slot * STAGE;
                umma::mbar_expect_tx(&full[slot], (uint32_t)STAGE);
#pragma unroll
                for (int i = 0; i < 128 / CA; ++i) umma::tma_load_2d(sA + i * A_BLK, &tz, co0 + i * CA, p0, &full[slot]);
#pragma unroll
                for (int j = 0; j < 128 / CB; ++j) {
                    int tap, c0;
                    if (cin >= CB) {
                        const int k = k0 + j * CB;
                        tap = k / cin;
                        c0 = k - tap * cin;
                    } else {  // one tap per block
                        tap = blockIdx.x * (128 / CB) + j;
                        c0 = 0;
                    }
                    if (tap >= 9) c0 = cin;  // past the taps: a box of zeros
                    const int t = tap < 9 ? tap : 4;
                    umma::tma_load_4d(sA + A_BYTES + j * B_BLK, &tx, c0, x0 + t % 3 - 1, y0 + t / 3 - 1, b0,
                                      &full[slot]);
                }
                tma_issued = kt + 1;
            }
        }
        __syncwarp();
    } else if (warp == 5) {
        if (lane == 0) {  // MMA issuer
            const uint32_t idesc = umma::idesc_bf16_f32_mn(128, 128);
            int kt = 0;
            for (; kt < nk; ++kt) {
                const int slot = kt % WG_STAGES, use = kt / WG_STAGES;
                if (!umma::mbar_wait(&full[slot], (uint32_t)(use & 1), GB_WAIT_TRIES)) {
                    fail = 1;
                    for (int j = kt + 1; j < tma_issued; ++j)
                        umma::mbar_wait(&full[j % WG_STAGES], (uint32_t)((j / WG_STAGES) & 1), GB_WAIT_TRIES >> 4);
                    break;
                }
                umma::fence_after();
                const uint32_t sa = umma::smem_u32(base + slot * STAGE), sb = sa + A_BYTES;
#pragma unroll
                for (int ks = 0; ks < WG_PIX / 16; ++ks) {  // 16 pixels = two 8-row K groups
                    const uint64_t ad = umma::smem_desc_mn(sa + ks * 2 * 8 * CA * 2, A_BLK, 8 * CA * 2, CA * 2);
                    const uint64_t bd = umma::smem_desc_mn(sb + ks * 2 * 8 * CB * 2, B_BLK, 8 * CB * 2, CB * 2);
                    umma::mma_bf16(tmem, ad, bd, idesc, (kt > 0 || ks > 0) ? 1u : 0u);
                }
                umma::commit(&empty[slot]);
            }
            umma::commit(&done);
        }
        __syncwarp();
    }
    const bool fin = warp < 4 && nk > 0 ? umma::mbar_wait(&done, 0u, GB_WAIT_TRIES) : true;
    const bool ok = __syncthreads_and(fin) != 0 && fail == 0;
    if (ok && nk > 0 && warp < 4) {
        umma::fence_after();
        const int co = co0 + warp * 32 + lane;
#pragma unroll 1
        for (int cb = 0; cb < 4; ++cb) {
            float v[32];
            umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cb * 32), v);
            if (co >= cout) continue;
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                const int col = cb * 32 + q;
                int k;
                if (cin >= CB) {
                    k = k0 + col;
                } else {  // column block col / CB is tap blockIdx.x * (128 / CB) + col / CB
                    const int tap = blockIdx.x * (128 / CB) + col / CB, c = col % CB;
                    k = tap < 9 && c < cin ? tap * cin + c : 9 * cin;
                }
                if (k < 9 * cin) atomicAdd(dW + (size_t)co * Kp + k, v[q]);
            }
        }
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    if (warp == 0) umma::tmem_free(tmem, 128);
}

void launch_wt_transpose(const __nv_bfloat16* W, int cin, int cout, __nv_bfloat16* Wd, cudaStream_t s) {
    k_conv_wt_transpose<<<128, 256, 0, s>>>(W, cin, cout, conv_kp(cin), Wd, conv_kp(cout));
}

int* device_error_flag() {
    static int* flag = nullptr;
    if (!flag) {
        if (cudaMalloc((void**)&flag, sizeof(int)) != cudaSuccess) return nullptr;
        cudaMemset(flag, 0, sizeof(int));
    }
    return flag;
}

impec_status gemm_bf16_tn(int M, int N, int K, const void* A, int lda, const void* B, int ldb, float* C, int ldc,
                          cudaStream_t s, int* err) {
    static bool attr = false;
    const int smem = 2 * GB_TILE_BYTES + 1024;
    if (!attr) {
        IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_gemm_bf16_tn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    dim3 g((N + GB_N - 1) / GB_N, (M + GB_M - 1) / GB_M);
    k_gemm_bf16_tn<<<g, GB_THREADS, smem, s>>>(M, N, K, (const __nv_bfloat16*)A, lda, (const __nv_bfloat16*)B, ldb,
                                                 C, ldc, err);
    IMPEC_CUDA_TRY(cudaGetLastError());
    return IMPEC_OK;
}

int conv_kp(int cin) { return (9 * cin + GB_K - 1) / GB_K * GB_K; }

template <int BN>
static impec_status launch_conv_bn(const ConvArgs& a, cudaStream_t s) {
    static bool attr = false;
    const int smem = conv_smem_bytes<BN>();
    if (!attr) {
        IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_conv3x3<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    const int M = a.B * a.H * a.W_;
    dim3 g((a.cout + BN - 1) / BN, (M + GB_M - 1) / GB_M);
    k_conv3x3<BN><<<g, CV_THREADS, smem, s>>>(a);
    IMPEC_CUDA_TRY(cudaGetLastError());
    return IMPEC_OK;
}

// ---- TMA path: tensor maps through the CUDA driver API's cuTensorMapEncodeTiled (runtime entry point).
typedef CUresult (*TmapEncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static TmapEncodeFn tmap_encoder() {
    static TmapEncodeFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (TmapEncodeFn)p;
    }
    return fn;
}

// Whether the TMA kernel applies: cin a multiple of 32, and the 128 pixels of a tile form one
// box of whole rows (W a multiple of 128, or W dividing 128 with H a power-of-two multiple or
// divisor of 128 / W, so that a box never straddles two images).
static bool conv_tma_plan(const ConvArgs& a, int BN, ConvTmaPlan& p) {
    static const bool off = [] {
        const char* e = getenv("IMPEC_CONV_TMA");
        return e && e[0] == '0';
    }();
    if (off || a.cin % 32 != 0 || !tmap_encoder()) return false;
    const int W = a.W_, H = a.H;
    if (W >= GB_M) {
        if (W % GB_M) return false;
        p.wbox = GB_M, p.hbox = 1, p.bbox = 1;
    } else {
        if (GB_M % W) return false;
        const int hb = GB_M / W;
        p.wbox = W;
        if (hb >= H) {
            if (hb % H) return false;
            p.hbox = H, p.bbox = hb / H;
        } else {
            if (H % hb) return false;
            p.hbox = hb, p.bbox = 1;
        }
    }
    p.ks = a.cin % 64 == 0 ? 64 : 32;
    const int stage = (GB_M + BN) * p.ks * 2;
    p.stages = 200 * 1024 / stage;
    if (p.stages > CT_MAX_STAGES) p.stages = CT_MAX_STAGES;
    if (p.stages < 2) p.stages = 2;
    return true;
}

template <int BN, int KS>
static impec_status launch_conv_tma(const ConvArgs& a, const ConvTmaPlan& p, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_conv3x3_tma<BN, KS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            200 * 1024 + 1024));
        attr = true;
    }
    TmapEncodeFn enc = tmap_encoder();
    const CUtensorMapSwizzle sw = KS == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
    CUtensorMap tx, tw;
    const cuuint64_t xd[4] = {(cuuint64_t)a.cin, (cuuint64_t)a.W_, (cuuint64_t)a.H, (cuuint64_t)a.B};
    const cuuint64_t xs[3] = {(cuuint64_t)a.cin * 2, (cuuint64_t)a.W_ * a.cin * 2, (cuuint64_t)a.H * a.W_ * a.cin * 2};
    const cuuint32_t xb[4] = {(cuuint32_t)KS, (cuuint32_t)p.wbox, (cuuint32_t)p.hbox, (cuuint32_t)p.bbox};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    if (enc(&tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)a.X, xd, xs, xb, es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
        set_error("conv: cuTensorMapEncodeTiled (activations) failed");
        return IMPEC_ERR_CUDA;
    }
    const cuuint64_t wd[2] = {(cuuint64_t)a.Kp, (cuuint64_t)a.cout};
    const cuuint64_t ws[1] = {(cuuint64_t)a.Kp * 2};
    const cuuint32_t wb[2] = {(cuuint32_t)KS, (cuuint32_t)BN};
    if (enc(&tw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)a.W, wd, ws, wb, es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
        set_error("conv: cuTensorMapEncodeTiled (weights) failed");
        return IMPEC_ERR_CUDA;
    }
    const int M = a.B * a.H * a.W_;
    const int smem = p.stages * (GB_M + BN) * KS * 2 + 1024;
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    const long long tiles = (long long)((M + GB_M - 1) / GB_M) * ((a.cout + BN - 1) / BN);
    const int per_sm = smem <= 110 * 1024 ? 2 : 1;  // resident CTAs per SM (shared memory)
    const int grid = (int)(tiles < (long long)sms * per_sm ? tiles : (long long)sms * per_sm);
    k_conv3x3_tma<BN, KS><<<grid, CT_THREADS, smem, s>>>(tx, tw, a, p.stages);
    IMPEC_CUDA_TRY(cudaGetLastError());
    return IMPEC_OK;
}

template <int BN, int CIN>
static impec_status launch_conv_halo(const ConvArgs& a, cudaStream_t s) {
    constexpr int smem = halo_smem<BN, CIN>();
    static bool attr = false;
    if (!attr) {
        IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_conv3x3_halo<BN, CIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    TmapEncodeFn enc = tmap_encoder();
    const CUtensorMapSwizzle sw = CIN == 64 ? CU_TENSOR_MAP_SWIZZLE_128B
                                            : (CIN == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
    CUtensorMap tx, tw;
    const cuuint64_t xd[4] = {(cuuint64_t)a.cin, (cuuint64_t)a.W_, (cuuint64_t)a.H, (cuuint64_t)a.B};
    const cuuint64_t xs[3] = {(cuuint64_t)a.cin * 2, (cuuint64_t)a.W_ * a.cin * 2, (cuuint64_t)a.H * a.W_ * a.cin * 2};
    const cuuint32_t xb[4] = {(cuuint32_t)CIN, (cuuint32_t)CH_PIX, 3, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    if (enc(&tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)a.X, xd, xs, xb, es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
        set_error("conv: cuTensorMapEncodeTiled (halo) failed");
        return IMPEC_ERR_CUDA;
    }
    const cuuint64_t wd[2] = {(cuuint64_t)a.Kp, (cuuint64_t)a.cout};
    const cuuint64_t ws[1] = {(cuuint64_t)a.Kp * 2};
    const cuuint32_t wb[2] = {(cuuint32_t)CIN, (cuuint32_t)BN};
    if (enc(&tw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)a.W, wd, ws, wb, es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
        set_error("conv: cuTensorMapEncodeTiled (halo weights) failed");
        return IMPEC_ERR_CUDA;
    }
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    const int M = a.B * a.H * a.W_, mt = M / GB_M, nt = (a.cout + BN - 1) / BN;
    const int per_sm = smem <= 110 * 1024 ? 2 : 1;
    int G = (sms * per_sm) / nt;
    if (G < 1) G = 1;
    if (G > mt) G = mt;
    k_conv3x3_halo<BN, CIN><<<nt * G, CH_THREADS, smem, s>>>(tx, tw, a);
    IMPEC_CUDA_TRY(cudaGetLastError());
    return IMPEC_OK;
}

// The halo kernel: cin 8, 32 or 64, tiles of 128 pixels of one image row, output-channel tiles
// of at most 64 (the weights of all taps stay in shared memory).
static bool conv_halo_ok(const ConvArgs& a) {
    static const bool off = [] {
        const char* e = getenv("IMPEC_CONV_HALO");
        return e && e[0] == '0';
    }();
    return !off && (a.cin == 8 || a.cin == 32 || a.cin == 64) && a.W_ % GB_M == 0 && tmap_encoder();
}

template <int BN>
static impec_status launch_conv_any(const ConvArgs& a, cudaStream_t s) {
    constexpr int HB = BN <= 64 ? BN : 64;
    if (BN <= 64 && conv_halo_ok(a))
        return a.cin == 64 ? launch_conv_halo<HB, 64>(a, s)
                           : (a.cin == 32 ? launch_conv_halo<HB, 32>(a, s) : launch_conv_halo<HB, 16>(a, s));
    ConvTmaPlan p;
    if (conv_tma_plan(a, BN, p)) return p.ks == 64 ? launch_conv_tma<BN, 64>(a, p, s) : launch_conv_tma<BN, 32>(a, p, s);
    return launch_conv_bn<BN>(a, s);
}

// The output-channel tile: the widest of 128, 64, 32 (not beyond cout) that still gives one
// CTA per SM; small layers take 32 for more CTAs.
impec_status launch_conv(const ConvArgs& a, cudaStream_t s) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    const long long mt = ((long long)a.B * a.H * a.W_ + GB_M - 1) / GB_M;
    auto ctas = [&](int bn) { return mt * ((a.cout + bn - 1) / bn); };
    if (conv_halo_ok(a)) return a.cout >= 64 ? launch_conv_any<64>(a, s) : launch_conv_any<32>(a, s);
    if (a.cout >= 128 && ctas(128) >= sms) return launch_conv_any<128>(a, s);
    if (a.cout >= 64 && ctas(64) >= sms) return launch_conv_any<64>(a, s);
    return launch_conv_any<32>(a, s);
}

// Boxes of 64 pixels: whole rows (W a multiple of 64) or whole-row groups of one image, as in
// conv_tma_plan; cin and cout multiples of 32; P a multiple of 64.
static bool wgrad_tma_plan(int B, int H, int W, int cin, int cout, int* wb, int* hb, int* bb) {
    static const bool off = [] {
        const char* e = getenv("IMPEC_CONV_TMA");
        return e && e[0] == '0';
    }();
    if (off || (cin % 32 && cin != 8) || (cout % 32 && cout != 8) || ((long long)B * H * W) % WG_PIX ||
        !tmap_encoder())
        return false;
    if (W >= WG_PIX) {
        if (W % WG_PIX) return false;
        *wb = WG_PIX, *hb = 1, *bb = 1;
        return true;
    }
    if (WG_PIX % W) return false;
    const int r = WG_PIX / W;
    *wb = W;
    if (r >= H) {
        if (r % H) return false;
        *hb = H, *bb = r / H;
    } else {
        if (H % r) return false;
        *hb = r, *bb = 1;
    }
    return true;
}

template <int CA, int CB>
static impec_status launch_wgrad_tma(const __nv_bfloat16* dZ, const __nv_bfloat16* X, int B, int H, int W_, int cin,
                                     int cout, float* dW, int* err, int num_sms, int wb, int hb, int bb,
                                     cudaStream_t s) {
    constexpr int STAGE = 128 * WG_PIX * 2 * 2;
    const int smem = WG_STAGES * STAGE + 1024;
    static bool attr = false;
    if (!attr) {
        IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_conv_wgrad_tma<CA, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    TmapEncodeFn enc = tmap_encoder();
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const int P = B * H * W_, Kp = conv_kp(cin);
    CUtensorMap tz, tx;
    const cuuint64_t zd[2] = {(cuuint64_t)cout, (cuuint64_t)P};
    const cuuint64_t zs[1] = {(cuuint64_t)cout * 2};
    const cuuint32_t zb[2] = {(cuuint32_t)CA, (cuuint32_t)WG_PIX};
    if (enc(&tz, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)dZ, zd, zs, zb, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CA == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
        set_error("wgrad: cuTensorMapEncodeTiled (gradients) failed");
        return IMPEC_ERR_CUDA;
    }
    const cuuint64_t xd[4] = {(cuuint64_t)cin, (cuuint64_t)W_, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t xs[3] = {(cuuint64_t)cin * 2, (cuuint64_t)W_ * cin * 2, (cuuint64_t)H * W_ * cin * 2};
    const cuuint32_t xb[4] = {(cuuint32_t)CB, (cuuint32_t)wb, (cuuint32_t)hb, (cuuint32_t)bb};
    if (enc(&tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)X, xd, xs, xb, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CB == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
        set_error("wgrad: cuTensorMapEncodeTiled (activations) failed");
        return IMPEC_ERR_CUDA;
    }
    const int nt = cin >= CB ? (9 * cin + 127) / 128 : (9 + 128 / CB - 1) / (128 / CB), mt = (cout + 127) / 128;
    int splits = (2 * num_sms + nt * mt - 1) / (nt * mt);
    int per = (P + splits - 1) / splits;
    per = (per + WG_PIX - 1) / WG_PIX * WG_PIX;
    splits = (P + per - 1) / per;
    dim3 g(nt, mt, splits);
    k_conv_wgrad_tma<CA, CB><<<g, WG_THREADS, smem, s>>>(tz, tx, H, W_, cin, cout, Kp, P, per, dW, err);
    IMPEC_CUDA_TRY(cudaGetLastError());
    return IMPEC_OK;
}

impec_status launch_wgrad(const __nv_bfloat16* dZ, const __nv_bfloat16* X, int B, int H, int W_, int cin, int cout,
                          float* dW, int* err, int num_sms, cudaStream_t s) {
    int wb, hb, bb;
    if (wgrad_tma_plan(B, H, W_, cin, cout, &wb, &hb, &bb)) {
        const bool a64 = cout % 64 == 0, b64 = cin % 64 == 0;  // 8-channel operands take 32-channel boxes
        if (a64 && b64) return launch_wgrad_tma<64, 64>(dZ, X, B, H, W_, cin, cout, dW, err, num_sms, wb, hb, bb, s);
        if (a64) return launch_wgrad_tma<64, 32>(dZ, X, B, H, W_, cin, cout, dW, err, num_sms, wb, hb, bb, s);
        if (b64) return launch_wgrad_tma<32, 64>(dZ, X, B, H, W_, cin, cout, dW, err, num_sms, wb, hb, bb, s);
        return launch_wgrad_tma<32, 32>(dZ, X, B, H, W_, cin, cout, dW, err, num_sms, wb, hb, bb, s);
    }
    static bool attr = false;
    const int smem = 2 * GB_TILE_BYTES + 1024;
    if (!attr) {
        IMPEC_CUDA_TRY(cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    const int P = B * H * W_, Kp = conv_kp(cin);
    const int nt = (9 * cin + GB_N - 1) / GB_N, mt = (cout + GB_M - 1) / GB_M;
    int splits = (2 * num_sms + nt * mt - 1) / (nt * mt);  // about two waves of CTAs
    int per = (P + splits - 1) / splits;
    per = (per + GB_K - 1) / GB_K * GB_K;
    splits = (P + per - 1) / per;
    dim3 g(nt, mt, splits);
    k_conv_wgrad<<<g, GB_THREADS, smem, s>>>(dZ, X, B, H, W_, cin, cout, Kp, per, dW, err);
    IMPEC_CUDA_TRY(cudaGetLastError());
    return IMPEC_OK;
}

impec_status check_err(int* err, cudaStream_t s, const char* what) {
    int h = 0;
    IMPEC_CUDA_TRY(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(s));
    if (h) {
        cudaMemsetAsync(err, 0, sizeof(int), s);
        set_error(std::string(what) + ": a tensor-core wait timed out");
        return IMPEC_ERR_CUDA;
    }
    return IMPEC_OK;
}

}  // namespace impec

using namespace impec;

static bool conv_shape_ok(int B, int H, int W, int cin, int cout) {
    return B > 0 && H > 0 && W > 0 && cin > 0 && cout > 0 && cin % 8 == 0 && cout % 8 == 0 &&
           (long long)B * H * W < (1LL << 31) / 256;
}

extern "C" impec_status impec_conv3x3_forward(const void* X, int B, int H, int W, int cin, const void* Wt,
                                              const float* bias, int cout, int act, void* Z, void* Y, float* Yf,
                                              const void* skip, void* stream) {
    if (!X || !Wt || !conv_shape_ok(B, H, W, cin, cout) || (!Z && !Y && !Yf)) {
        set_error("impec_conv3x3_forward: bad arguments (channels must be multiples of 8)");
        return IMPEC_ERR_ARG;
    }
    int* err = device_error_flag();
    if (!err) return IMPEC_ERR_CUDA;
    ConvArgs a = {};
    a.X = (const __nv_bfloat16*)X; a.W = (const __nv_bfloat16*)Wt; a.bias = bias;
    a.Z = (__nv_bfloat16*)Z; a.Y = (__nv_bfloat16*)Y; a.Yf = Yf; a.skip = (const __nv_bfloat16*)skip;
    a.B = B; a.H = H; a.W_ = W; a.cin = cin; a.cout = cout; a.Kp = conv_kp(cin); a.tapsign = 1; a.act = act; a.err = err;
    cudaStream_t s = (cudaStream_t)stream;
    IMPEC_TRY(launch_conv(a, s));
    return check_err(err, s, "impec_conv3x3_forward");
}

// dX (or the gradient of the pre-activation below, when gz is given) from dZ: the transposed
// convolution with weights rearranged from W.
extern "C" impec_status impec_conv3x3_input_grad(const void* dZ, int B, int H, int W, int cout, const void* Wt,
                                                 int cin, const void* gz, const void* add, void* Y, float* Yf,
                                                 void* stream) {
    if (!dZ || !Wt || !conv_shape_ok(B, H, W, cin, cout) || (!Y && !Yf)) {
        set_error("impec_conv3x3_input_grad: bad arguments");
        return IMPEC_ERR_ARG;
    }
    int* err = device_error_flag();
    if (!err) return IMPEC_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    const int Kp = conv_kp(cin), Kd = conv_kp(cout);
    __nv_bfloat16* Wd = nullptr;
    IMPEC_CUDA_TRY(cudaMallocAsync((void**)&Wd, (size_t)cin * Kd * 2, s));
    k_conv_wt_transpose<<<64, 256, 0, s>>>((const __nv_bfloat16*)Wt, cin, cout, Kp, Wd, Kd);
    ConvArgs a = {};
    a.X = (const __nv_bfloat16*)dZ; a.W = Wd; a.gz = (const __nv_bfloat16*)gz; a.add = (const __nv_bfloat16*)add;
    a.Y = (__nv_bfloat16*)Y; a.Yf = Yf;
    a.B = B; a.H = H; a.W_ = W; a.cin = cout; a.cout = cin; a.Kp = Kd; a.tapsign = -1; a.err = err;
    impec_status st = launch_conv(a, s);
    cudaFreeAsync(Wd, s);
    IMPEC_TRY(st);
    return check_err(err, s, "impec_conv3x3_input_grad");
}

// dW (fp32 [cout][Kp], accumulated into) from dZ and the layer input X.
extern "C" impec_status impec_conv3x3_weight_grad(const void* dZ, const void* X, int B, int H, int W, int cin,
                                                  int cout, float* dW, void* stream) {
    if (!dZ || !X || !dW || !conv_shape_ok(B, H, W, cin, cout)) {
        set_error("impec_conv3x3_weight_grad: bad arguments");
        return IMPEC_ERR_ARG;
    }
    int* err = device_error_flag();
    if (!err) return IMPEC_ERR_CUDA;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t s = (cudaStream_t)stream;
    IMPEC_TRY(launch_wgrad((const __nv_bfloat16*)dZ, (const __nv_bfloat16*)X, B, H, W, cin, cout, dW, err, sms, s));
    return check_err(err, s, "impec_conv3x3_weight_grad");
}

extern "C" impec_status impec_gemm_bf16(const void* A, int lda, const void* B, int ldb, float* C, int ldc, int M,
                                        int N, int K, void* stream) {
    if (!A || !B || !C || M < 1 || N < 1 || K < GB_K || K % GB_K || lda % 8 || ldb % 8 || lda < K || ldb < K ||
        ldc < N || ((uintptr_t)A & 15) || ((uintptr_t)B & 15)) {
        set_error("impec_gemm_bf16: need K a multiple of 64, lda/ldb multiples of 8 and >= K, 16-byte aligned operands");
        return IMPEC_ERR_ARG;
    }
    int* err = device_error_flag();
    if (!err) return IMPEC_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    IMPEC_TRY(gemm_bf16_tn(M, N, K, A, lda, B, ldb, C, ldc, s, err));
    int h = 0;
    IMPEC_CUDA_TRY(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    IMPEC_CUDA_TRY(cudaStreamSynchronize(s));
    if (h) {
        cudaMemsetAsync(err, 0, sizeof(int), s);
        set_error("impec_gemm_bf16: a tensor-core wait timed out");
        return IMPEC_ERR_CUDA;
    }
    return IMPEC_OK;
}

// ---------------------------------------------------------------- bounded-wait self-test
// One thread initialises an mbarrier that expects one arrival.  With arrive != 0 it arrives
// first, so the wait completes; otherwise nothing ever arrives and the wait gives up after
// max_tries polls, exactly as the tensor-core kernels' waits do when a copy never lands.  The
// outcome goes to *timed_out (1: gave up, 0: completed); the kernel always returns.
__global__ void k_selftest_bounded_wait(uint32_t max_tries, int arrive, int* __restrict__ timed_out) {
    __shared__ __align__(8) uint64_t mbar;
    if (threadIdx.x != 0) return;
    umma::mbar_init(&mbar, 1);
    if (arrive) umma::mbar_arrive(&mbar);
    *timed_out = umma::mbar_wait(&mbar, 0u, max_tries) ? 0 : 1;
}

extern "C" impec_status impec_selftest_bounded_wait(unsigned max_tries, int arrive, int* timed_out) {
    if (!timed_out || max_tries == 0 || max_tries > (1u << 20)) {
        set_error("impec_selftest_bounded_wait: max_tries must be in [1, 1048576]");
        return IMPEC_ERR_ARG;
    }
    int* flag = device_error_flag();
    if (!flag) return IMPEC_ERR_CUDA;
    IMPEC_CUDA_TRY(cudaMemset(flag, 0xff, sizeof(int)));
    k_selftest_bounded_wait<<<1, 32>>>((uint32_t)max_tries, arrive, flag);
    IMPEC_LAUNCH_CHECK();
    int h = -1;
    IMPEC_CUDA_TRY(cudaMemcpy(&h, flag, sizeof(int), cudaMemcpyDeviceToHost));
    IMPEC_CUDA_TRY(cudaMemset(flag, 0, sizeof(int)));
    if (h != 0 && h != 1) {
        set_error("impec_selftest_bounded_wait: the kernel did not report");
        return IMPEC_ERR_CUDA;
    }
    *timed_out = h;
    return IMPEC_OK;
}
