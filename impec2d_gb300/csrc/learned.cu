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
#include <cuda_bf16.h>

#include <cstdint>

#include "internal.cuh"
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

static int* device_error_flag() {
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

}  // namespace impec

using namespace impec;

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
