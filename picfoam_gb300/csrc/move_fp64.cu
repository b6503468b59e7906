// move_fp64.cu -- FP64 (exact) form of the fused push + track + deposit.
// Built with --fmad=false: every product and sum rounds on its own, in the
// evaluation order of the CPU oracle, so the two agree bit for bit.
#include "kernels.h"
#include "move_impl.cuh"

namespace pgd {

__constant__ TetConst c_tet64;
__constant__ PatchConst c_patch64;

__global__ void __launch_bounds__(256) move_kernel_fp64(MoveParams P) {
    unsigned ts = 0, fc = 0, wl = 0, ab = 0;
    for (int i = P.first + blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x) {
        TrackTally td{0u, 0u, 0u, true, false, false};
        const bool alive = P.p.tet[i] >= 0;
        move_one<double>(P, c_tet64, c_patch64, i, td);
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

cudaError_t move_fp64_set_tables(const TetConst& t, const PatchConst& p) {
    cudaError_t e = cudaMemcpyToSymbol(c_tet64, &t, sizeof t);
    if (e != cudaSuccess) return e;
    return cudaMemcpyToSymbol(c_patch64, &p, sizeof p);
}

void launch_move_fp64(const MoveParams& P, int grid, cudaStream_t s) {
    move_kernel_fp64<<<grid, 256, 0, s>>>(P);
}

}  // namespace pgd
