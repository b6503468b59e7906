// move_fp32.cu -- FP32 mixed form of the fused push + track + deposit.
// Barycentric coordinates, velocity and fields in FP32 (FMA contraction on);
// the charge is accumulated in FP64 or 64-bit fixed point.
#include "kernels.h"
#include "move_impl.cuh"

namespace pgd {

__constant__ TetConst c_tet32;
__constant__ PatchConst c_patch32;

__global__ void __launch_bounds__(256) move_kernel_fp32(MoveParams P) {
    unsigned ts = 0, fc = 0, wl = 0, ab = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x) {
        TrackTally td{0u, 0u, 0u, true, false, false};
        const bool alive = P.p.tet[i] >= 0;
        move_one<float>(P, c_tet32, c_patch32, i, td);
        ts += td.tet_steps;
        fc += td.faces;
        wl += td.walls;
        ab += (alive && !td.keep) ? 1u : 0u;
    }
    warp_add_counter<double>(&P.counters->tet_steps, ts);
    warp_add_counter<double>(&P.counters->faces, fc);
    warp_add_counter<double>(&P.counters->walls, wl);
    warp_add_counter<double>(&P.counters->absorbed, ab);
}

cudaError_t move_fp32_set_tables(const TetConst& t, const PatchConst& p) {
    cudaError_t e = cudaMemcpyToSymbol(c_tet32, &t, sizeof t);
    if (e != cudaSuccess) return e;
    return cudaMemcpyToSymbol(c_patch32, &p, sizeof p);
}

void launch_move_fp32(const MoveParams& P, int grid, cudaStream_t s) {
    move_kernel_fp32<<<grid, 256, 0, s>>>(P);
}

}  // namespace pgd
