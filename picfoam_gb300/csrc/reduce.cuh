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

// Sum over the block in the fixed tree order: lane l of warp 0 adds the
// values of threads l, l+32, ..., l+224 in turn, then the 32 lanes meet in an
// xor-tree.  One warp does the FP64 adds (the FP64 pipe is the scarce unit on
// this part).  ws holds 256 doubles; the result is valid in every lane of
// warp 0.
__device__ __forceinline__ double block_tree(double v, double* ws) {
    ws[threadIdx.x] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = ws[threadIdx.x];
#pragma unroll
        for (int j = 1; j < 8; ++j) r = r + ws[threadIdx.x + 32 * j];
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
    if (threadIdx.x == 0) {
        const unsigned int t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1);
        if (last) *ticket = 0u;
    }
    __syncthreads();
    return last;
}

__device__ __forceinline__ double final_sum(const double* part, int nb, double* ws) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += 256) s = s + __ldcg(part + i);
    return block_tree(s, ws);
}

}  // namespace pgd
