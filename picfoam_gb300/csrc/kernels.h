// kernels.h -- host-side declarations of the kernel launchers.
#pragma once

#include "common.cuh"

namespace pgd {

cudaError_t move_fp64_set_tables(const TetConst& t, const PatchConst& p);
void launch_move_fp64(const MoveParams& P, int grid, cudaStream_t s);
// Returns the number of kernels launched (in-cell mover + crossing tracker, or
// the general kernel).
int launch_move_fp32(const MoveParams& P, int grid, cudaStream_t s);
// Velocity push of every live particle by tt without tracking (FP64 or FP32 store).
void launch_push_only(const MoveParams& P, bool fp32, double tt, int grid, cudaStream_t s);

}  // namespace pgd
