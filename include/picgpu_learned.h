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

/* The warm-start network on its own (host buffers).  Grid X x Y x Z (x
 * fastest) must be a multiple of 4 per direction with X*Y*Z/64 a multiple of
 * 128.  Weights are FP32, all layers back to back in the order c1a c1b c2a
 * c2b c3a c3b d2a d2b d1a d1b co, each [27][cout][cin] with the (cin, cout)
 * pairs (2,16) (16,16) (16,32) (32,32) (32,64) (64,64) (96,32) (32,32)
 * (48,16) (16,16) (16,1); picgpu_unet_param_count() floats in all.  The input
 * is FP32 [X*Y*Z][2] (scaled residual, domain mask), the output FP32
 * [X*Y*Z].  The loss of a sample is sum m (out - t)^2 / sum m t^2 with mask m. */
typedef struct picgpu_unet picgpu_unet;

size_t picgpu_unet_param_count(void);
picgpu_status picgpu_unet_create(int X, int Y, int Z, uint64_t seed, picgpu_unet** out);
void picgpu_unet_destroy(picgpu_unet* net);
picgpu_status picgpu_unet_set_weights(picgpu_unet* net, const float* w);
picgpu_status picgpu_unet_get_weights(picgpu_unet* net, float* w);
picgpu_status picgpu_unet_forward(picgpu_unet* net, const float* in, float* out);
/* Loss and its gradient with respect to every weight (same layout as w). */
picgpu_status picgpu_unet_gradients(picgpu_unet* net, const float* in, const float* target, const float* mask,
                                    float* grad, double* loss);
/* iters Adam steps (learning rate lr) on one sample; loss of the last step. */
picgpu_status picgpu_unet_train(picgpu_unet* net, const float* in, const float* target, const float* mask,
                                int iters, double lr, double* loss);

#ifdef __cplusplus
}
#endif
#endif
