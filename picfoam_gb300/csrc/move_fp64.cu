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

// Push only, no tracking, of slots [first, n): initalizeLeapFrog
// (picInitialise.C:219-227) calls the pusher's updateVelocity(p, -dt/2) on
// every parcel, moving or not; an emitted parcel is synchronised the same way
// (ParticleEmitter.C:401, PICParcel.C:220-227).
template <class Real>
__global__ void __launch_bounds__(256) push_only_kernel(MoveParams P, Real tt) {
    for (int i = P.first + blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x) {
        const int tetg = P.p.tet[i];
        if (tetg < 0) continue;
        PState<Real> s;
        s.cell = tetg / 12;
        s.tet = tetg - 12 * s.cell;
        s.y[1] = ybuf<Real>(P.p, 0)[i];
        s.y[2] = ybuf<Real>(P.p, 1)[i];
        s.y[3] = ybuf<Real>(P.p, 2)[i];
        s.y[0] = Real(1) - s.y[1] - s.y[2] - s.y[3];
        s.U[0] = ubuf<Real>(P.p, 0)[i];
        s.U[1] = ubuf<Real>(P.p, 1)[i];
        s.U[2] = ubuf<Real>(P.p, 2)[i];
        load_attributes(P, i, s);
        push<Real>(P, c_tet64, s, tt);
        ubuf<Real>(P.p, 0)[i] = s.U[0];
        ubuf<Real>(P.p, 1)[i] = s.U[1];
        ubuf<Real>(P.p, 2)[i] = s.U[2];
    }
}

void launch_push_only(const MoveParams& P, bool fp32, double tt, int grid, cudaStream_t s) {
    if (fp32) push_only_kernel<float><<<grid, 256, 0, s>>>(P, float(tt));
    else push_only_kernel<double><<<grid, 256, 0, s>>>(P, tt);
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
