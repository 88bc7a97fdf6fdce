// Deterministic block reductions: every block writes its partial, the last block to
// finish (ticket counter) folds the partials in a fixed order.  Reruns are bit-identical
// because the grid size and the per-thread assignment are fixed.
#pragma once
#include <cuda_runtime.h>

namespace impec {

constexpr int RED_THREADS = 256;

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Reduce K values across the block; result valid in thread 0.  maxmask bit k selects max.
// A shared-memory tree (128, 64, 32 pairs) and then one warp's shuffle tree: 12 FP64 warp
// instructions per value instead of 45 for a shuffle tree in every warp.  An FP64 instruction
// costs the same whether all lanes or some take part, so the pairing count is what matters.
// Requires blockDim.x == RED_THREADS.
template <int K>
__device__ __forceinline__ void block_reduce(double (&v)[K], unsigned maxmask) {
    __shared__ double sh[K][RED_THREADS];
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < K; ++k) sh[k][t] = v[k];
    __syncthreads();
#pragma unroll
    for (int s = RED_THREADS / 2; s >= 32; s >>= 1) {
        if (t < s)
#pragma unroll
            for (int k = 0; k < K; ++k)
                sh[k][t] = ((maxmask >> k) & 1) ? fmax(sh[k][t], sh[k][t + s]) : sh[k][t] + sh[k][t + s];
        __syncthreads();
    }
    if (t < 32) {
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = ((maxmask >> k) & 1) ? warp_max(sh[k][t]) : warp_sum(sh[k][t]);
    }
}

// Blocks for a row-segment walk over an n1 x n2 grid: one block per segment of RED_THREADS
// cells of a row, at most max_blocks (larger grids loop).
static inline int seg_blocks(int n1, int n2, int max_blocks) {
    const long units = (long)n1 * ((n2 + RED_THREADS - 1) / RED_THREADS);
    return (int)(units < max_blocks ? units : max_blocks);
}

// Block limit for the reductions: four blocks per SM, so that each thread folds several cells
// before the FP64 warp sums (five additions per reduced value and thread) are paid.
static inline int red_cap(int num_sms, int max_blocks) { return num_sms * 4 < max_blocks ? num_sms * 4 : max_blocks; }

// Blocks for a flat walk over n values: one value per thread, at most max_blocks.
static inline int flat_blocks(size_t n, int max_blocks) {
    const size_t b = (n + RED_THREADS - 1) / RED_THREADS;
    return (int)(b < (size_t)max_blocks ? (b > 0 ? b : 1) : (size_t)max_blocks);
}

// Row-segment walk (grid of seg_blocks blocks of RED_THREADS): f(i, j, k) for every cell,
// k = i*n2 + j.  A block issues the loads of a whole segment at once and no thread divides
// per cell, which keeps the walk bandwidth- rather than latency-bound.
template <class F>
__device__ __forceinline__ void for_cells(int n1, int n2, F&& f) {
    const int segs = (n2 + RED_THREADS - 1) / RED_THREADS, units = n1 * segs;
    for (int u = blockIdx.x; u < units; u += gridDim.x) {
        const int i = u / segs, j = (u - i * segs) * RED_THREADS + (int)threadIdx.x;
        if (j < n2) f(i, j, (size_t)i * n2 + j);
    }
}

// Grid-level reduction with last-block finalisation.  Requires blockDim.x == RED_THREADS,
// 1-D grid with gridDim.x <= max_blocks.  out[k] receives the reduced values.  Returns true in
// every thread of the last block (thread 0 of which wrote out[]).
template <int K>
__device__ bool grid_reduce(double (&v)[K], unsigned maxmask, double* partials, int max_blocks,
                            unsigned* counter, double* out) {
    __shared__ bool last;
    block_reduce<K>(v, maxmask);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) partials[k * max_blocks + blockIdx.x] = v[k];
        __threadfence();
        unsigned ticket = atomicAdd(counter, 1u);
        last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double w[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const bool mx = (maxmask >> k) & 1;
        double a = mx ? -INFINITY : 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
            double p = ((volatile double*)partials)[k * max_blocks + b];
            a = mx ? fmax(a, p) : a + p;
        }
        w[k] = a;
    }
    block_reduce<K>(w, maxmask);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) out[k] = w[k];
        *counter = 0u;
    }
    return true;
}

}  // namespace impec
