// move_fp32.cu -- FP32 form of the fused push + track + deposit.
//
// The per-particle algorithm of move_impl.cuh (PICParcel::move / moveForward,
// PICMCCFVM/parcels/Templates/PICParcel/PICParcel.C:38-144), laid out for
// throughput rather than for bit-exact agreement with the oracle:
//   * barycentric coordinates and velocity in FP32, fast-math intrinsics;
//   * one flat loop of tet steps: after an internal or cyclic cell-face
//     crossing the particle continues with the unused fraction of the same
//     displacement (the FP64 form recomputes f dt U - d, which is the same
//     vector); the displacement is recomputed only after a wall reflection;
//   * a tet step first tries the common case "no coordinate reaches zero"
//     (no division); the hit search runs only when one does;
//   * E at the particle from a per-cell block of 9 float4 (centre + 8
//     corners), so the gather needs no cell -> point indirection;
//   * tet geometry and the tet-crossing tables of the canonical hex in shared
//     memory (lanes index them by different tets; constant memory would
//     serialise that);
//   * charge deposited as 2^-25 fixed-point weights into per-cell corner slots
//     (order-independent integer sums), reduced to points by the charge update.
#include "kernels.h"
#include "move_impl.cuh"

namespace pgd {

__constant__ Tables32 c_t32;

namespace {

__device__ __forceinline__ float pick(unsigned s, float y0, float y1, float y2, float y3) {
    return s == 0u ? y0 : s == 1u ? y1 : s == 2u ? y2 : s == 3u ? y3 : 0.f;
}

struct S32 {
    int cell, tet;
    float y[4];
    float U[3];
};

__device__ __forceinline__ void field32(const MoveParams& P, const Tables32& T, const S32& s, float* E) {
    const float4* e = P.Ec4 + 9 * s.cell;
    const float4 a = __ldg(e);
    if (P.field_weighting == PICGPU_WEIGHTING_CELL_AVERAGE) {
        E[0] = a.x; E[1] = a.y; E[2] = a.z;
        return;
    }
    const unsigned tri = T.tri[s.tet];
    const float4 b = __ldg(e + 1 + (tri & 15u));
    const float4 c = __ldg(e + 1 + ((tri >> 4) & 15u));
    const float4 d = __ldg(e + 1 + ((tri >> 8) & 15u));
    E[0] = a.x * s.y[0] + b.x * s.y[1] + c.x * s.y[2] + d.x * s.y[3];
    E[1] = a.y * s.y[0] + b.y * s.y[1] + c.y * s.y[2] + d.y * s.y[3];
    E[2] = a.z * s.y[0] + b.z * s.y[1] + c.z * s.y[2] + d.z * s.y[3];
}

// Relativistic Boris (BorisPusher.C:69-112) in FP32: the Lorentz factor of
// the incoming velocity is reused for the averaged factor of the rotation.
__device__ __forceinline__ void boris32(const MoveParams& P, const float* E, float* U, float tt) {
    constexpr float ic2 = float(1.0 / (kC * kC));
    const float u2 = U[0] * U[0] + U[1] * U[1] + U[2] * U[2];
    const float g_in = rsqrtf(1.f - u2 * ic2);  // gamma of the incoming velocity
    float r0 = U[0] * g_in, r1 = U[1] * g_in, r2 = U[2] * g_in;
    const float qdm = P.qm_f * (0.5f * tt);
    const float e0 = qdm * E[0], e1 = qdm * E[1], e2 = qdm * E[2];
    r0 += e0; r1 += e1; r2 += e2;
    if (P.rotation) {
        const float g_mid = sqrtf(1.f + (r0 * r0 + r1 * r1 + r2 * r2) * ic2);
        const float k = qdm * __fdividef(2.f, g_in + g_mid);
        const float t0 = k * P.B_f[0], t1 = k * P.B_f[1], t2 = k * P.B_f[2];
        const float d0 = r0 + (r1 * t2 - r2 * t1);
        const float d1 = r1 + (r2 * t0 - r0 * t2);
        const float d2 = r2 + (r0 * t1 - r1 * t0);
        const float h = __fdividef(2.f, 1.f + t0 * t0 + t1 * t1 + t2 * t2);
        const float s0 = h * t0, s1 = h * t1, s2 = h * t2;
        r0 += d1 * s2 - d2 * s1;
        r1 += d2 * s0 - d0 * s2;
        r2 += d0 * s1 - d1 * s0;
    }
    r0 += e0; r1 += e1; r2 += e2;
    const float g_out = rsqrtf(1.f + (r0 * r0 + r1 * r1 + r2 * r2) * ic2);
    U[0] = r0 * g_out; U[1] = r1 * g_out; U[2] = r2 * g_out;
}

template <int PUSHER>
__device__ __forceinline__ void push32(const MoveParams& P, const Tables32& T, S32& s, float tt) {
    float E[3];
    field32(P, T, s, E);
    if (PUSHER == PICGPU_PUSHER_BORIS) boris32(P, E, s.U, tt);
    else if (PUSHER == PICGPU_PUSHER_BORIS_NR) push_boris_nr<float>(P, E, s.U, tt);
    else if (PUSHER == PICGPU_PUSHER_VAY) push_vay<float>(P, E, s.U, tt);
    else if (PUSHER == PICGPU_PUSHER_HIGUERA_CARY) push_hc<float>(P, E, s.U, tt);
}

__device__ __forceinline__ void remap(unsigned code, S32& s) {
    const float y0 = s.y[0], y1 = s.y[1], y2 = s.y[2], y3 = s.y[3];
#pragma unroll
    for (int j = 0; j < 4; ++j) s.y[j] = pick((code >> (4 + 3 * j)) & 7u, y0, y1, y2, y3);
    s.tet = int(code & 15u);
}

// Tracking displacement dt_frac U - d, U constrained to the solution
// directions, d the deviation from the mesh centre in the empty ones
// (PICParcel.C:119-126).
__device__ __forceinline__ void displacement(const MoveParams& P, const Tables32& T, const S32& s, float fdt,
                                             float* disp) {
    disp[0] = fdt * s.U[0];
    disp[1] = fdt * s.U[1];
    disp[2] = fdt * s.U[2];
    if (!P.m.any_empty) return;
    const float* off = P.m.uniform ? T.off : P.m.offset32 + size_t(P.m.cell_class[s.cell]) * 24;
    const unsigned tri = T.tri[s.tet];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!P.m.empty[a]) continue;
        const float x = P.m.cc32[3 * s.cell + a] + s.y[1] * off[3 * (tri & 15u) + a] +
                        s.y[2] * off[3 * ((tri >> 4) & 15u) + a] + s.y[3] * off[3 * ((tri >> 8) & 15u) + a];
        disp[a] = -(x - P.centre_f[a]);
    }
}

struct Tally {
    unsigned tet_steps, faces, walls;
    bool keep;
};

// The push of PICParcel::move (once per step, before tracking); false when
// the particle reached the speed of light (it is then removed).
template <int PUSHER>
__device__ __forceinline__ bool push_phase(const MoveParams& P, const Tables32& T, S32& s, Tally& td) {
    if (P.charged) push32<PUSHER>(P, T, s, P.dt_f);
    if (!(s.U[0] * s.U[0] + s.U[1] * s.U[1] + s.U[2] * s.U[2] < float(kC) * float(kC))) {
        td.keep = false;
        atomicMax(&P.counters->error, int(PICGPU_SPEED_OF_LIGHT));
        return false;
    }
    return true;
}

template <int PUSHER>
__device__ __forceinline__ void track32(const MoveParams& P, const Tables32& T, S32& s, Tally& td);

template <int PUSHER>
__device__ __forceinline__ void move32(const MoveParams& P, const Tables32& T, S32& s, Tally& td) {
    if (!push_phase<PUSHER>(P, T, s, td)) return;
    track32<PUSHER>(P, T, s, td);
}

// Tracking of one time step after the push (PICParcel::moveForward).
template <int PUSHER>
__device__ __forceinline__ void track32(const MoveParams& P, const Tables32& T, S32& s, Tally& td) {
    const float dt = P.dt_f;
    float disp[3];
    displacement(P, T, s, dt, disp);
    float rem = 1.f;     // unused fraction of disp
    float base = 0.f;    // step fraction at which disp was formed
    int resync = 0;
    for (int budget = P.max_steps; budget > 0; --budget) {
        td.tet_steps++;
        const float* inv = P.m.uniform ? T.inv + 9 * s.tet
                                       : P.m.tetinv32 + (size_t(P.m.cell_class[s.cell]) * 12 + s.tet) * 9;
        const float dx0 = rem * disp[0], dx1 = rem * disp[1], dx2 = rem * disp[2];
        float dy[4];
        dy[1] = inv[0] * dx0 + inv[1] * dx1 + inv[2] * dx2;
        dy[2] = inv[3] * dx0 + inv[4] * dx1 + inv[5] * dx2;
        dy[3] = inv[6] * dx0 + inv[7] * dx1 + inv[8] * dx2;
        dy[0] = -(dy[1] + dy[2] + dy[3]);
        float yn[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) yn[i] = s.y[i] + dy[i];
        if (fminf(fminf(yn[0], yn[1]), fminf(yn[2], yn[3])) >= 0.f) {
            // the displacement ends inside this tet
#pragma unroll
            for (int i = 0; i < 4; ++i) s.y[i] = yn[i];
            return;
        }
        const float S = fabsf(dy[0]) + fabsf(dy[1]) + fabsf(dy[2]) + fabsf(dy[3]);
        const float thr = -1e-6f * S;
        float lam = 1.f;
        int hit = -1;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (dy[i] < thr) {
                const float l = __fdividef(-s.y[i], dy[i]);
                if (l < lam) { lam = l; hit = i; }
            }
        }
        float y[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) y[i] = (i == hit) ? 0.f : fmaxf(s.y[i] + lam * dy[i], 0.f);
        const float r = __fdividef(1.f, y[0] + y[1] + y[2] + y[3]);
#pragma unroll
        for (int i = 0; i < 4; ++i) s.y[i] = y[i] * r;
        if (hit < 0) return;
        rem *= (1.f - lam);
        if (hit > 0) {
            remap(T.inner[4 * s.tet + hit], s);
            continue;
        }
        const int nb = __ldg(P.m.nbr + 6 * s.cell + (s.tet >> 1));
        td.faces++;
        if (nb >= 0) {
            remap(T.cross[s.tet], s);
            s.cell = nb;
            continue;
        }
        // patch hit (PICParcel::hitPatch, PICParcel.C:153-184)
        const int patch = -nb - 1;
        const int kind = T.kind[patch];
        if (kind == PICGPU_PATCH_ABSORB) { td.keep = false; return; }
        if (kind == PICGPU_PATCH_FLOATING || (kind == PICGPU_PATCH_CIRCUIT && P.q != 0.0)) {
            td.keep = false;
            atomicAdd(P.qconv + patch, P.weight * P.q);
            return;
        }
        const float sf = base + (1.f - base) * (1.f - rem);
        const int f = s.tet >> 1;
        const float* n =
            P.m.uniform ? T.normal + 3 * f : P.m.fnormal32 + size_t(P.m.cell_class[s.cell]) * 18 + 3 * f;
        const bool wall = kind == PICGPU_PATCH_WALL || kind == PICGPU_PATCH_CIRCUIT;
        if (wall) {
            if (P.sync && P.charged) push32<PUSHER>(P, T, s, (sf - 0.5f) * dt);
            td.walls++;
        }
        const float Un = s.U[0] * n[0] + s.U[1] * n[1] + s.U[2] * n[2];
        if (Un > 0.f) {
            const float t = 2.f * Un;
            s.U[0] -= t * n[0];
            s.U[1] -= t * n[1];
            s.U[2] -= t * n[2];
        }
        if (wall && ++resync <= 1 && P.sync && P.charged) push32<PUSHER>(P, T, s, (0.5f - sf) * dt);
        base = sf;
        rem = 1.f;
        displacement(P, T, s, (1.f - sf) * dt, disp);
    }
    td.keep = false;
    atomicMax(&P.counters->error, int(PICGPU_TRACK_LOOP_CAP));
}

// Deposit into the block's shared-memory window of cells [w0, w0 + kWindow)
// (the store is kept in cell order, so a block's contiguous chunk of
// particles covers a short cell range); particles outside the window go
// straight to the global accumulators.  Window slots are 32-bit: an add that
// wraps carries 2^32 into the cell's 64-bit global slot, so the integer sums
// stay exact.
constexpr int kWindow = 1024;

__device__ __forceinline__ void win_add(unsigned* slot, unsigned long long* gslot, unsigned v) {
    const unsigned old = atomicAdd(slot, v);
    if (old + v < old) atomicAdd(gslot, 1ull << 32);
}

__device__ __forceinline__ void deposit32(const MoveParams& P, const Tables32& T, const S32& s, int w0,
                                          unsigned* win) {
    if (!P.has_value) return;
    constexpr float kScale = float(1u << kDepositBits);
    const int rel = s.cell - w0;
    unsigned long long* g = P.acc9 + 9 * size_t(s.cell);
    const bool average = P.charge_distribution == PICGPU_WEIGHTING_CELL_AVERAGE;
    const unsigned tri = T.tri[s.tet];
    const unsigned w0v = average ? (1u << kDepositBits) : __float2uint_rn(s.y[0] * kScale);
    if (unsigned(rel) < unsigned(kWindow)) {
        unsigned* a = win + 9 * rel;
        win_add(a, g, w0v);
        if (average) return;
        const unsigned k1 = 1 + (tri & 15u), k2 = 1 + ((tri >> 4) & 15u), k3 = 1 + ((tri >> 8) & 15u);
        win_add(a + k1, g + k1, __float2uint_rn(s.y[1] * kScale));
        win_add(a + k2, g + k2, __float2uint_rn(s.y[2] * kScale));
        win_add(a + k3, g + k3, __float2uint_rn(s.y[3] * kScale));
        return;
    }
    atomicAdd(g, (unsigned long long)w0v);
    if (average) return;
    atomicAdd(g + 1 + (tri & 15u), (unsigned long long)__float2uint_rn(s.y[1] * kScale));
    atomicAdd(g + 1 + ((tri >> 4) & 15u), (unsigned long long)__float2uint_rn(s.y[2] * kScale));
    atomicAdd(g + 1 + ((tri >> 8) & 15u), (unsigned long long)__float2uint_rn(s.y[3] * kScale));
}

struct Rec {
    int tet;
    float y1, y2, y3, u0, u1, u2;
};

__device__ __forceinline__ Rec load_rec(const DSpecies& p, int i) {
    Rec r;
    r.tet = __ldcs(p.tet + i);
    r.y1 = __ldcs(p.y32[0] + i);
    r.y2 = __ldcs(p.y32[1] + i);
    r.y3 = __ldcs(p.y32[2] + i);
    r.u0 = __ldcs(p.u32[0] + i);
    r.u1 = __ldcs(p.u32[1] + i);
    r.u2 = __ldcs(p.u32[2] + i);
    return r;
}

// Each block moves one contiguous chunk of the store, 256 particles per
// tile; the next tile's records are loaded before the current tile is
// processed, so their DRAM latency overlaps the push and the tracking.
template <int PUSHER>
__global__ void __launch_bounds__(256, 5) move_kernel_fp32(MoveParams P, int chunk) {
    __shared__ Tables32 T;
    extern __shared__ unsigned win[];  // kWindow * 9 slots (32-bit, carry to global)
    int n_end = P.n, first = P.first, ch = chunk;
    if (P.n_dev) {
        // counts live on the device: split [first, n) over the grid here
        n_end = *P.n_dev;
        first = P.first_dev ? *P.first_dev : 0;
        const long tiles = (long(n_end) - first + 255) / 256;
        ch = int(((tiles + gridDim.x - 1) / gridDim.x) * 256);
        if (ch <= 0) ch = 256;
    }
    const int start = first + blockIdx.x * ch;
    const int end = min(n_end, start + ch);
    if (start >= end) return;  // block-uniform: nothing to move (e.g. no secondaries this step)
    {
        const unsigned* src = reinterpret_cast<const unsigned*>(&c_t32);
        unsigned* dst = reinterpret_cast<unsigned*>(&T);
        for (int k = threadIdx.x; k < int(sizeof(Tables32) / 4); k += blockDim.x) dst[k] = src[k];
        for (int k = threadIdx.x; k < kWindow * 9; k += blockDim.x) win[k] = 0u;
    }
    __shared__ int w0s;
    if (threadIdx.x == 0) {
        int c0 = 0;
        for (int k = start; k < end && k < start + 64; ++k) {
            const int t = P.p.tet[k];
            if (t >= 0) { c0 = t / 12; break; }
        }
        w0s = max(0, c0 - kWindow / 16);
    }
    __syncthreads();
    const int w0 = w0s;
    unsigned ts = 0, fc = 0, wl = 0, ab = 0;
    int i = start + threadIdx.x;
    Rec next{-1, 0, 0, 0, 0, 0, 0};
    if (i < end) next = load_rec(P.p, i);
    for (int base = start; base < end; base += 256) {
        const Rec r = next;
        const int ci = i;
        i += 256;
        if (i < end) next = load_rec(P.p, i);
        if (ci >= end || r.tet < 0) continue;
        S32 s;
        s.cell = r.tet / 12;
        s.tet = r.tet - 12 * s.cell;
        s.y[1] = r.y1;
        s.y[2] = r.y2;
        s.y[3] = r.y3;
        s.y[0] = 1.f - s.y[1] - s.y[2] - s.y[3];
        s.U[0] = r.u0;
        s.U[1] = r.u1;
        s.U[2] = r.u2;
        Tally td{0u, 0u, 0u, true};
        if (P.solve_movement) move32<PUSHER>(P, T, s, td);
        ts += td.tet_steps;
        fc += td.faces;
        wl += td.walls;
        if (!td.keep) {
            P.p.tet[ci] = -1;
            ++ab;
            continue;
        }
        if (P.solve_movement) {
            __stcs(P.p.tet + ci, 12 * s.cell + s.tet);
            __stcs(P.p.y32[0] + ci, s.y[1]);
            __stcs(P.p.y32[1] + ci, s.y[2]);
            __stcs(P.p.y32[2] + ci, s.y[3]);
            __stcs(P.p.u32[0] + ci, s.U[0]);
            __stcs(P.p.u32[1] + ci, s.U[1]);
            __stcs(P.p.u32[2] + ci, s.U[2]);
        }
        deposit32(P, T, s, w0, win);
    }
    __syncthreads();
    // flush the window
    if (P.has_value) {
        const int nslot = min(kWindow, P.m.n_cells - w0) * 9;
        unsigned long long* g = P.acc9 + 9 * size_t(w0);
        for (int k = threadIdx.x; k < nslot; k += blockDim.x) {
            const unsigned v = win[k];
            if (v) atomicAdd(g + k, (unsigned long long)v);
        }
    }
    warp_add_counter<float>(&P.counters->tet_steps, ts);
    warp_add_counter<float>(&P.counters->faces, fc);
    warp_add_counter<float>(&P.counters->walls, wl);
    warp_add_counter<float>(&P.counters->absorbed, ab);
}



}  // namespace

cudaError_t move_fp32_set_tables(const Tables32& t) { return cudaMemcpyToSymbol(c_t32, &t, sizeof t); }

// grid: the number of resident blocks to use (5 per SM); each block takes one
// contiguous chunk (a multiple of 256 particles) of [P.first, P.n).  With
// P.n_dev set the counts are read on the device and all grid blocks launch.
void launch_move_fp32(const MoveParams& P, int grid, cudaStream_t s) {
    int blocks, chunk;
    if (P.n_dev) {
        // device-resident counts: the kernel sizes its chunks; grid fixed
        blocks = grid;
        chunk = 0;
    } else {
        const long work = long(P.n) - P.first;
        if (work <= 0) return;
        const long tiles = (work + 255) / 256;
        const long per = (tiles + grid - 1) / grid;
        chunk = int(per * 256);
        blocks = int((work + chunk - 1) / chunk);
    }
    const size_t smem = size_t(kWindow) * 9 * sizeof(unsigned);
    switch (P.pusher) {
        case PICGPU_PUSHER_BORIS:
            move_kernel_fp32<PICGPU_PUSHER_BORIS><<<blocks, 256, smem, s>>>(P, chunk);
            break;
        case PICGPU_PUSHER_BORIS_NR:
            move_kernel_fp32<PICGPU_PUSHER_BORIS_NR><<<blocks, 256, smem, s>>>(P, chunk);
            break;
        case PICGPU_PUSHER_VAY: move_kernel_fp32<PICGPU_PUSHER_VAY><<<blocks, 256, smem, s>>>(P, chunk); break;
        case PICGPU_PUSHER_HIGUERA_CARY:
            move_kernel_fp32<PICGPU_PUSHER_HIGUERA_CARY><<<blocks, 256, smem, s>>>(P, chunk);
            break;
        default: move_kernel_fp32<PICGPU_PUSHER_NONE><<<blocks, 256, smem, s>>>(P, chunk); break;
    }
}

}  // namespace pgd
