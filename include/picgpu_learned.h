/*
 * picgpu_learned.h -- the learned Poisson warm start of the GB300 library
 * (a 3-level 3D U-Net on the cell grid, BF16 tensor-core convolutions with
 * FP32 accumulation, trained on the GPU by its own forward and backward
 * kernels).  picFoam has no counterpart: its ElectroStaticSolver starts the
 * PCG from the previous potential (ElectroStaticSolver.C:61-64).  These entry
 * points expose the network for testing and for hosts that train or inspect
 * it directly; picgpu_config.learned switches it on inside picgpu_step.
 */
#ifndef PICGPU_LEARNED_H
#define PICGPU_LEARNED_H

#include "picgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One 3x3x3 "same" convolution (zero padding) on the tensor cores, on host
 * buffers.  Grid X x Y x Z (x fastest, X*Y*Z a multiple of 128); the input is
 * the channel concatenation of in1 (cin1 channels, at half resolution and
 * read by nearest upsampling when up1 = 1) and in2 (cin2 channels, may be
 * 0), BF16 bit patterns, channels last; w is BF16 [27][cout][cin1+cin2] with
 * taps ordered (dz, dy, dx) from -1; out is FP32 [X*Y*Z][cout], after ReLU
 * when relu = 1 (the ReLU form stores BF16 on the device; out then holds
 * those values).  Returns PICGPU_NOT_SUPPORTED for channel pairs the kernel
 * is not instantiated for. */
picgpu_status picgpu_test_conv3d(int X, int Y, int Z, int cin1, int cin2, int up1, int cout, int relu,
                                 const uint16_t* in1, const uint16_t* in2, const uint16_t* w, float* out);

#ifdef __cplusplus
}
#endif
#endif
