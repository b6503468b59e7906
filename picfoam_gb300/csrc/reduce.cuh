// reduce.cuh -- fixed-order block and grid reductions of the FP64 solvers.
//
// Every sum runs in one tree order independent of timing: a block of 256
// threads stores its values, lane l of warp 0 adds threads l, l+32, ...,
// l+224 in turn, then the 32 lanes meet in an xor-tree; the block that
// arrives last at a grid-wide ticket combines the block partials in the same
// order.  The result is therefore bit-reproducible run to run.
#pragma once

#include <cuda_runtime.h>

namespace pgd {

// Blocks have 256 threads (1-D, or a 2-D tile); the flat thread index orders
// every sum.
__device__ __forceinline__ int flat_tid() { return threadIdx.x + blockDim.x * threadIdx.y; }
__device__ __forceinline__ unsigned int grid_blocks() { return gridDim.x * gridDim.y * gridDim.z; }
__device__ __forceinline__ int flat_bid() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }

// Sum over the block in the fixed tree order: lane l of warp 0 adds the
// values of threads l, l+32, ..., l+224 in turn, then the 32 lanes meet in an
// xor-tree.  One warp does the FP64 adds (the FP64 pipe is the scarce unit on
// this part).  ws holds 256 doubles; the result is valid in every lane of
// warp 0.
__device__ __forceinline__ double block_tree(double v, double* ws) {
    const int t = flat_tid();
    ws[t] = v;
    __syncthreads();
    double r = 0.0;
    if (t < 32) {
        r = ws[t];
#pragma unroll
        for (int j = 1; j < 8; ++j) r = r + ws[t + 32 * j];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) r = r + __shfl_xor_sync(0xffffffffu, r, off);
    }
    __syncthreads();
    return r;
}

// Last-block finalisation: returns true in the block that arrives last; the
// block partials are then visible to it.
__device__ __forceinline__ bool arrive_last(unsigned int* ticket) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (flat_tid() == 0) {
        const unsigned int t = atomicAdd(ticket, 1u);
        last = (t == grid_blocks() - 1);
        if (last) *ticket = 0u;
    }
    __syncthreads();
    return last;
}

// Thread t adds part[t], part[t + 256], ... in that order; the loads are
// issued eight at a time so that they overlap.
__device__ __forceinline__ double final_sum(const double* part, int nb, double* ws) {
    double s = 0.0;
    int i = flat_tid();
    for (; i + 7 * 256 < nb; i += 8 * 256) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = __ldcg(part + i + u * 256);
#pragma unroll
        for (int u = 0; u < 8; ++u) s = s + v[u];
    }
    for (; i < nb; i += 256) s = s + __ldcg(part + i);
    return block_tree(s, ws);
}

// FP32 variant of block_tree (same order); ws holds 256 floats.
__device__ __forceinline__ float block_tree_f(float v, float* ws) {
    const int t = flat_tid();
    ws[t] = v;
    __syncthreads();
    float r = 0.f;
    if (t < 32) {
        r = ws[t];
#pragma unroll
        for (int j = 1; j < 8; ++j) r += ws[t + 32 * j];
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;
}

}  // namespace pgd
