// unet.h -- the learned Poisson warm start: a 3-level 3D U-Net on the cell
// grid with BF16 tensor-core convolutions (FP32 accumulation), trained on
// the GPU by its own forward and backward kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

namespace pgd {

// ------------------------------------------------ tensor-core convolution --
struct ConvGrid {
    int X, Y, Z;  // the output (and full-resolution input) grid, x fastest
};

// One channels-last BF16 input of a convolution: C channels (a multiple of
// 8) at full resolution, or (up = 1) at half resolution and read by nearest
// upsampling.  C = 0 marks an absent second source.
struct ConvSrc {
    const __nv_bfloat16* p;
    int C;
    int up;
};

enum { kEpiReluBf16 = 0, kEpiF32 = 1 };

// out[v][co] = epi( sum_{tap, ci} in[v + tap][ci] * w[tap][co][ci] ), zero
// padding; w is BF16 [27][cout][cin] with taps ordered (dz, dy, dx) from -1.
// X*Y*Z must be a multiple of 128.  *err is raised if a bounded wait timed out.
bool conv_tc_supported(int cin, int cout);
cudaError_t launch_conv_tc(int cin, int cout, int epi, const ConvGrid& g, const ConvSrc& s1, const ConvSrc& s2,
                           const __nv_bfloat16* w, void* out, int* err, cudaStream_t st);

}  // namespace pgd
