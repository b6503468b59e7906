// move_fp32.cu -- FP32 form of the fused push + track + deposit.
//
// The per-particle algorithm of move_impl.cuh (PICParcel::move / moveForward,
// PICMCCFVM/parcels/Templates/PICParcel/PICParcel.C:38-144), laid out for
// throughput rather than for bit-exact agreement with the oracle:
//   * barycentric coordinates and velocity in FP32, fast-math intrinsics;
//   * on a uniform block mesh, the in-cell mover (move_cell_kernel_fp32)
//     pushes every particle, moves it in cell coordinates normalised by the
//     cell size and, when the end point lies in the same cell, finds its tet
//     directly: the face pyramid from the dominant coordinate, the side of the
//     face diagonal from one dot product.  Crossings of the tet faces inside a
//     cell are no events of the physics (no patch, no field change), so this
//     is the barycentric tracker's end state without its per-face loop, and
//     every lane of a warp runs the same instructions.  A particle whose end
//     point lies outside its cell is queued with its pushed velocity, and the
//     crossing tracker (track_queue_kernel_fp32) follows it face by face with
//     the barycentric tracker below, patches included, on full warps;
//   * the general kernel (move_kernel_fp32) serves meshes of several cell
//     shapes: one flat loop of tet steps; after an internal or cyclic
//     cell-face crossing the particle continues with the unused fraction of
//     the same displacement (the FP64 form recomputes f dt U - d, which is the
//     same vector); a tet step first tries the common case "no coordinate
//     reaches zero" (no division); the hit search runs only when one does;
//   * E at the particle from a per-cell block of 9 float4 (centre + 8
//     corners), so the gather needs no cell -> point indirection;
//   * tet geometry and the tet-crossing tables of the canonical hex in shared
//     memory (lanes index them by different tets; constant memory would
//     serialise that), copied from the context's own device tables;
//   * charge deposited as 2^-25 fixed-point weights into per-cell corner slots
//     (order-independent integer sums), reduced to points by the charge update.
#include "kernels.h"
#include "move_impl.cuh"

namespace pgd {

namespace {

__device__ __forceinline__ float pick(unsigned s, float y0, float y1, float y2, float y3) {
    return s == 0u ? y0 : s == 1u ? y1 : s == 2u ? y2 : s == 3u ? y3 : 0.f;
}

struct S32 {
    int cell, tet;
    float y[4];
    float U[3];
    float zf;   // charge modifier (1 without per-parcel attributes)
    float dm;   // deposit multiple: chargeModifier x nParticle / species weight (1 without)
};

// The parcel's charge modifier and deposit multiple: from the store's
// per-parcel attributes in the kernels built for them (ATTRS), else the
// constants 1 and 1, which the compiler folds away.
template <bool ATTRS>
__device__ __forceinline__ void load_attributes32(const MoveParams& P, int i, S32& s) {
    if (ATTRS) {
        const int z = P.p.zq[i];
        s.zf = float(z);
        s.dm = float(double(z) * P.p.nw[i] / P.weight);
    } else {
        s.zf = 1.f;
        s.dm = 1.f;
    }
}

// Charge a parcel leaves on a floating or circuit patch: nParticle x charge.
__device__ __forceinline__ double parcel_charge(const MoveParams& P, const S32& s) {
    return double(s.dm) * P.weight * P.q;
}

__device__ __forceinline__ void field32(const MoveParams& P, const unsigned* tri_of, const S32& s, float* E) {
    const float4* e = P.Ec4 + 9 * s.cell;
    const float4 a = __ldg(e);
    if (P.field_weighting == PICGPU_WEIGHTING_CELL_AVERAGE) {
        E[0] = a.x; E[1] = a.y; E[2] = a.z;
        return;
    }
    const unsigned tri = tri_of[s.tet];
    const float4 b = __ldg(e + 1 + (tri & 15u));
    const float4 c = __ldg(e + 1 + ((tri >> 4) & 15u));
    const float4 d = __ldg(e + 1 + ((tri >> 8) & 15u));
    E[0] = a.x * s.y[0] + b.x * s.y[1] + c.x * s.y[2] + d.x * s.y[3];
    E[1] = a.y * s.y[0] + b.y * s.y[1] + c.y * s.y[2] + d.y * s.y[3];
    E[2] = a.z * s.y[0] + b.z * s.y[1] + c.z * s.y[2] + d.z * s.y[3];
}

// Lorentz factors in FP32 through their distance from 1.  At plasma
// energies gamma = 1 + 5e-6 rounds to 1 + k 2^-23 in FP32, and the rounding
// of gamma on the way in (u = gamma v) and on the way out (v = u / gamma)
// does not cancel: the kinetic energy then drifts by ~1e-7 per push (3e-4
// over the 2000 steps of the plasma oscillation).  With a = v^2/c^2,
// b = u^2/c^2 the pushers use
//   gamma - 1     = a / (s (1 + s)),  s = sqrt(1 - a)   (v -> u: u = v + v (gamma - 1))
//   1 - 1 / gamma = b / (q (1 + q)),  q = sqrt(1 + b)   (u -> v: v = u - u (1 - 1/gamma))
// whose rounding scales with gamma - 1, not with gamma.
__device__ __forceinline__ float gamma_less_one(float a) {
    const float s = sqrtf(1.f - a);
    return __fdividef(a, s * (1.f + s));
}
__device__ __forceinline__ float one_less_inv_gamma(float b) {
    const float q = sqrtf(1.f + b);
    return __fdividef(b, q * (1.f + q));
}

// Relativistic Boris (BorisPusher.C:69-112) in FP32: the Lorentz factor of
// the incoming velocity is reused for the averaged factor of the rotation.
__device__ __forceinline__ void boris32(const MoveParams& P, const float* E, const float* Bv, float* U, float tt,
                                        float zf) {
    constexpr float ic2 = float(1.0 / (kC * kC));
    const float dg_in = gamma_less_one((U[0] * U[0] + U[1] * U[1] + U[2] * U[2]) * ic2);
    float r0 = U[0] + U[0] * dg_in, r1 = U[1] + U[1] * dg_in, r2 = U[2] + U[2] * dg_in;
    const float qdm = P.qm_f * zf * (0.5f * tt);
    const float e0 = qdm * E[0], e1 = qdm * E[1], e2 = qdm * E[2];
    r0 += e0; r1 += e1; r2 += e2;
    if (P.rotation) {
        const float g_mid = sqrtf(1.f + (r0 * r0 + r1 * r1 + r2 * r2) * ic2);
        const float k = qdm * __fdividef(2.f, 1.f + dg_in + g_mid);
        const float t0 = k * Bv[0], t1 = k * Bv[1], t2 = k * Bv[2];
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
    const float dg_out = one_less_inv_gamma((r0 * r0 + r1 * r1 + r2 * r2) * ic2);
    U[0] = r0 - r0 * dg_out; U[1] = r1 - r1 * dg_out; U[2] = r2 - r2 * dg_out;
}

// VayPusher::updateVelocity (VayPusher.C:54-100) in FP32, U x T with v
// (VayPusher.C:81), the Lorentz factors of the conversions as above.
__device__ __forceinline__ void vay32(const MoveParams& P, const float* E, const float* Bv, float* U, float tt,
                                      float zf) {
    constexpr float ic = float(1.0 / kC), ic2 = float(1.0 / (kC * kC));
    const float dg = gamma_less_one((U[0] * U[0] + U[1] * U[1] + U[2] * U[2]) * ic2);
    const float qe = P.qm_f * zf * tt, qb = P.qm_f * zf * (0.5f * tt);
    float u0 = U[0] + U[0] * dg + qe * E[0], u1 = U[1] + U[1] * dg + qe * E[1], u2 = U[2] + U[2] * dg + qe * E[2];
    float T0 = qb * Bv[0], T1 = qb * Bv[1], T2 = qb * Bv[2];
    u0 += U[1] * T2 - U[2] * T1;
    u1 += U[2] * T0 - U[0] * T2;
    u2 += U[0] * T1 - U[1] * T0;
    const float alpha0 = 1.f + (u0 * u0 + u1 * u1 + u2 * u2) * ic2;
    const float TT = T0 * T0 + T1 * T1 + T2 * T2;
    const float sg = alpha0 - TT;
    const float udt = (u0 * T0 + u1 * T1 + u2 * T2) * ic;
    const float inv_g = rsqrtf(0.5f * (sg + sqrtf(sg * sg + 4.f * (TT + udt * udt))));
    T0 *= inv_g; T1 *= inv_g; T2 *= inv_g;
    const float sc = __fdividef(1.f, 1.f + T0 * T0 + T1 * T1 + T2 * T2);
    const float ut = u0 * T0 + u1 * T1 + u2 * T2;
    const float r0 = sc * ((u0 + ut * T0) + (u1 * T2 - u2 * T1));
    const float r1 = sc * ((u1 + ut * T1) + (u2 * T0 - u0 * T2));
    const float r2 = sc * ((u2 + ut * T2) + (u0 * T1 - u1 * T0));
    const float dg_out = one_less_inv_gamma((r0 * r0 + r1 * r1 + r2 * r2) * ic2);
    U[0] = r0 - r0 * dg_out; U[1] = r1 - r1 * dg_out; U[2] = r2 - r2 * dg_out;
}

// HigueraCaryPusher::updateVelocity (HigueraCary.C:69-115) in FP32, the
// Lorentz factors of the conversions as above.
__device__ __forceinline__ void hc32(const MoveParams& P, const float* E, const float* Bv, float* U, float tt,
                                     float zf) {
    constexpr float ic2 = float(1.0 / (kC * kC));
    const float dg = gamma_less_one((U[0] * U[0] + U[1] * U[1] + U[2] * U[2]) * ic2);
    float r0 = U[0] + U[0] * dg, r1 = U[1] + U[1] * dg, r2 = U[2] + U[2] * dg;
    const float qdm = P.qm_f * zf * (0.5f * tt);
    const float e0 = qdm * E[0], e1 = qdm * E[1], e2 = qdm * E[2];
    r0 += e0; r1 += e1; r2 += e2;
    if (P.rotation) {
        const float gfm2 = 1.f + (r0 * r0 + r1 * r1 + r2 * r2) * ic2;
        float t0 = qdm * Bv[0], t1 = qdm * Bv[1], t2 = qdm * Bv[2];
        const float beta2 = t0 * t0 + t1 * t1 + t2 * t2;
        const float gb = gfm2 - beta2;
        const float tr = t0 * r0 + t1 * r1 + t2 * r2;
        // (t . u)^2 without the 1/c^2 of the textbook form, as HigueraCary.C:103 has it
        const float iG = rsqrtf(0.5f * (gb + sqrtf(gb * gb + 4.f * (beta2 + tr * tr))));
        t0 *= iG; t1 *= iG; t2 *= iG;
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
    const float dg_out = one_less_inv_gamma((r0 * r0 + r1 * r1 + r2 * r2) * ic2);
    U[0] = r0 - r0 * dg_out; U[1] = r1 - r1 * dg_out; U[2] = r2 - r2 * dg_out;
}

template <int PUSHER>
__device__ __forceinline__ void push32(const MoveParams& P, const unsigned* tri_of, S32& s, float tt) {
    float E[3], Bv[3];
    field32(P, tri_of, s, E);
    if (P.Bc4) {
        // per-cell magnetic field (B[celli])
        const float4 b = __ldg(P.Bc4 + s.cell);
        Bv[0] = b.x;
        Bv[1] = b.y;
        Bv[2] = b.z;
    } else {
        Bv[0] = P.B_f[0];
        Bv[1] = P.B_f[1];
        Bv[2] = P.B_f[2];
    }
    if (PUSHER == PICGPU_PUSHER_BORIS) boris32(P, E, Bv, s.U, tt, s.zf);
    else if (PUSHER == PICGPU_PUSHER_BORIS_NR) push_boris_nr<float>(P, E, Bv, s.U, tt, s.zf);
    else if (PUSHER == PICGPU_PUSHER_VAY) vay32(P, E, Bv, s.U, tt, s.zf);
    else if (PUSHER == PICGPU_PUSHER_HIGUERA_CARY) hc32(P, E, Bv, s.U, tt, s.zf);
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
    if (P.charged && s.zf != 0.f) push32<PUSHER>(P, T.tri, s, P.dt_f);
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
            atomicAdd(P.qconv + patch, parcel_charge(P, s));
            return;
        }
        const float sf = base + (1.f - base) * (1.f - rem);
        const int f = s.tet >> 1;
        const float* n =
            P.m.uniform ? T.normal + 3 * f : P.m.fnormal32 + size_t(P.m.cell_class[s.cell]) * 18 + 3 * f;
        const bool wall = kind == PICGPU_PATCH_WALL || kind == PICGPU_PATCH_CIRCUIT;
        if (wall) {
            if (P.sync && P.charged && s.zf != 0.f) push32<PUSHER>(P, T.tri, s, (sf - 0.5f) * dt);
            td.walls++;
        }
        const float Un = s.U[0] * n[0] + s.U[1] * n[1] + s.U[2] * n[2];
        if (Un > 0.f) {
            const float t = 2.f * Un;
            s.U[0] -= t * n[0];
            s.U[1] -= t * n[1];
            s.U[2] -= t * n[2];
        }
        if (wall && ++resync <= 1 && P.sync && P.charged && s.zf != 0.f) push32<PUSHER>(P, T.tri, s, (0.5f - sf) * dt);
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

// A parcel whose deposit multiple exceeds 64 (merged or multiply charged
// parcels with per-parcel attributes): its fixed-point weights may pass
// 2^31, so they go straight to the 64-bit cell slots.
__device__ __noinline__ void deposit_heavy32(const MoveParams& P, const unsigned* tri_of, const S32& s) {
    const float sc = float(1u << kDepositBits) * s.dm;
    unsigned long long* g = P.acc9 + 9 * size_t(s.cell);
    if (P.charge_distribution == PICGPU_WEIGHTING_CELL_AVERAGE) {
        atomicAdd(g, __float2ull_rn(sc));
        return;
    }
    const unsigned tri = tri_of[s.tet];
    atomicAdd(g, __float2ull_rn(s.y[0] * sc));
    atomicAdd(g + 1 + (tri & 15u), __float2ull_rn(s.y[1] * sc));
    atomicAdd(g + 1 + ((tri >> 4) & 15u), __float2ull_rn(s.y[2] * sc));
    atomicAdd(g + 1 + ((tri >> 8) & 15u), __float2ull_rn(s.y[3] * sc));
}

__device__ __forceinline__ void deposit32(const MoveParams& P, const unsigned* tri_of, const S32& s, int w0,
                                          unsigned* win) {
    if (!P.has_value) return;
    if (s.dm > 64.f) {
        deposit_heavy32(P, tri_of, s);
        return;
    }
    const float kScale = float(1u << kDepositBits) * s.dm;
    const int rel = s.cell - w0;
    unsigned long long* g = P.acc9 + 9 * size_t(s.cell);
    const bool average = P.charge_distribution == PICGPU_WEIGHTING_CELL_AVERAGE;
    const unsigned tri = tri_of[s.tet];
    const unsigned w0v = average ? __float2uint_rn(kScale) : __float2uint_rn(s.y[0] * kScale);
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

// The in-cell mover's window: per cell kCellSub copies of the centre slot,
// lane l adding to copy l % kCellSub (the store is cell-sorted, so most
// lanes of a warp share a cell and would otherwise serialise on one
// address), then the 8 corner slots; the flush adds the copies.
constexpr int kCellSub = 4;
constexpr int kCellSlots = kCellSub + 8;
constexpr int kCellWindow = 768;

__device__ __forceinline__ void deposit_cell32(const MoveParams& P, const unsigned* tri_of, const S32& s, int w0,
                                               unsigned* win) {
    if (!P.has_value) return;
    if (s.dm > 64.f) {
        deposit_heavy32(P, tri_of, s);
        return;
    }
    const float kScale = float(1u << kDepositBits) * s.dm;
    const int rel = s.cell - w0;
    unsigned long long* g = P.acc9 + 9 * size_t(s.cell);
    const bool average = P.charge_distribution == PICGPU_WEIGHTING_CELL_AVERAGE;
    const unsigned tri = tri_of[s.tet];
    const unsigned w0v = average ? __float2uint_rn(kScale) : __float2uint_rn(s.y[0] * kScale);
    if (unsigned(rel) < unsigned(kCellWindow)) {
        unsigned* a = win + kCellSlots * rel;
        win_add(a + (threadIdx.x & (kCellSub - 1)), g, w0v);
        if (average) return;
        const unsigned k1 = tri & 15u, k2 = (tri >> 4) & 15u, k3 = (tri >> 8) & 15u;
        win_add(a + kCellSub + k1, g + 1 + k1, __float2uint_rn(s.y[1] * kScale));
        win_add(a + kCellSub + k2, g + 1 + k2, __float2uint_rn(s.y[2] * kScale));
        win_add(a + kCellSub + k3, g + 1 + k3, __float2uint_rn(s.y[3] * kScale));
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
template <int PUSHER, bool ATTRS>
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
        const unsigned* src = reinterpret_cast<const unsigned*>(P.t32);
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
        load_attributes32<ATTRS>(P, ci, s);
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
        deposit32(P, T.tri, s, w0, win);
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

// ------------------------------------------------------ in-cell mover ---

// The canonical hex in the normalised cell frame (centre 0, corners at
// +-1/2).  Tet t = 2 f + k lies on local face f (normal axis a = f / 2,
// outward side + for odd f); its corners are the face's base point p0 and
// p1, p2 (k = 0) or p2, p3 (k = 1).  In the face's own axes -- the normal n
// and the in-plane axes u, v with p1 - p0 along u and p3 - p0 along v, which
// are the axes a + 1, a + 2 on a + face and a + 2, a + 1 on a - face -- the
// corners sit at (u, v) = (-,-), (+,-), (+,+), (-,+), all at n = +-1/2, so
// both maps between barycentric and cell coordinates are sums of the
// coordinates with unit weights:
//   x_n = +-(y1 + y2 + y3) / 2,
//   k = 0: x_u = (-y1 + y2 + y3) / 2, x_v = (-y1 - y2 + y3) / 2,
//   k = 1: x_u = (-y1 + y2 - y3) / 2, x_v = (-y1 + y2 + y3) / 2,
// and back, with h = |x_n|: y0 = 1 - 2 h,
//   k = 0: (y1, y2, y3) = (h - x_u, x_u - x_v, h + x_v),
//   k = 1: (y1, y2, y3) = (h - x_v, h + x_u, x_v - x_u);
// the point lies on face f's pyramid when |x_a| is the largest coordinate,
// and in tet k = 1 when x_v > x_u (the plane through the centre and the
// diagonal p0 p2 separates the two).
__device__ __forceinline__ void bary_to_cell(int tet, const float* y, float& x0, float& x1, float& x2) {
    const int f = tet >> 1, a = f >> 1;
    const bool plus = f & 1, k1 = tet & 1;
    const float xn = (plus ? 0.5f : -0.5f) * (y[1] + y[2] + y[3]);
    const float xu = 0.5f * (k1 ? (y[2] - y[1] - y[3]) : (y[2] + y[3] - y[1]));
    const float xv = 0.5f * (k1 ? (y[2] + y[3] - y[1]) : (y[3] - y[1] - y[2]));
    const float xp = plus ? xu : xv;  // axis a + 1
    const float xq = plus ? xv : xu;  // axis a + 2
    x0 = a == 0 ? xn : a == 1 ? xq : xp;
    x1 = a == 1 ? xn : a == 2 ? xq : xp;
    x2 = a == 2 ? xn : a == 0 ? xq : xp;
}

__device__ __forceinline__ void cell_to_bary(float x0, float x1, float x2, S32& s) {
    const float a0 = fabsf(x0), a1 = fabsf(x1), a2 = fabsf(x2);
    const bool ax0 = a0 >= a1 && a0 >= a2, ax1 = !ax0 && a1 >= a2;
    const int a = ax0 ? 0 : ax1 ? 1 : 2;
    const float xn = ax0 ? x0 : ax1 ? x1 : x2;
    const float xp = ax0 ? x1 : ax1 ? x2 : x0;  // axis a + 1
    const float xq = ax0 ? x2 : ax1 ? x0 : x1;  // axis a + 2
    const bool plus = xn > 0.f;
    const float h = fabsf(xn);
    const float xu = plus ? xp : xq, xv = plus ? xq : xp;
    const bool k1 = xv > xu;
    s.tet = 4 * a + (plus ? 2 : 0) + (k1 ? 1 : 0);
    s.y[1] = h - (k1 ? xv : xu);
    s.y[2] = k1 ? h + xu : xu - xv;
    s.y[3] = k1 ? xv - xu : h + xv;
    // the centre coordinate as every later reader forms it from the stored
    // three (so a deposit-only pass over the store deposits the same weights)
    s.y[0] = 1.f - s.y[1] - s.y[2] - s.y[3];
}

__device__ __forceinline__ void store_rec(const DSpecies& p, int i, const S32& s, int cell_tet) {
    __stcs(p.tet + i, cell_tet);
    __stcs(p.y32[0] + i, s.y[1]);
    __stcs(p.y32[1] + i, s.y[2]);
    __stcs(p.y32[2] + i, s.y[3]);
    __stcs(p.u32[0] + i, s.U[0]);
    __stcs(p.u32[1] + i, s.U[1]);
    __stcs(p.u32[2] + i, s.U[2]);
}

// Uniform block meshes.  Each block moves one contiguous chunk of the store,
// 256 particles per tile, the next tile's records loaded before the current
// tile is processed.  Every particle is pushed (PICParcel::move) and its
// displaced point followed in normalised cell coordinates: inside the cell
// it takes the tet found by cell_to_bary (tracking inside a cell crosses only
// tet faces, which carry no event); across a cell face into a neighbour the
// point moves one cell over; an absorbing patch removes the particle, a
// floating or circuit patch removes a charged one and keeps its charge
// (PICParcel::hitPatch, PICParcel.C:153-184).  A particle that reaches a
// reflecting patch keeps its start record, gets its pushed velocity written
// back and joins the block's segment of the crossing queue, whose tracker
// repeats its step with the wall's velocity sync.  The in-cell path uses
// selects only (no indexed registers, no calls), so it needs no stack.
template <int PUSHER, bool ATTRS>
__global__ void __launch_bounds__(256, 5) move_cell_kernel_fp32(MoveParams P, int chunk) {
    __shared__ unsigned tri_s[12];
    __shared__ int kind_s[kMaxPatches];
    __shared__ int w0s, qn;
    extern __shared__ unsigned win[];  // kCellWindow * kCellSlots slots (32-bit, carry to global)
    int n_end = P.n, first = P.first, ch = chunk;
    if (P.n_dev) {
        n_end = *P.n_dev;
        first = P.first_dev ? *P.first_dev : 0;
        const long tiles = (long(n_end) - first + 255) / 256;
        ch = int(((tiles + gridDim.x - 1) / gridDim.x) * 256);
        if (ch <= 0) ch = 256;
    }
    const int start = first + blockIdx.x * ch;
    const int end = min(n_end, start + ch);
    if (start >= end) {
        // block-uniform: nothing to move; the crossing tracker reads the count
        if (threadIdx.x == 0) {
            P.xq.count[blockIdx.x] = 0;
            P.xq.start[blockIdx.x] = 0;
        }
        return;
    }
    {
        if (threadIdx.x < 12) tri_s[threadIdx.x] = P.t32->tri[threadIdx.x];
        if (threadIdx.x < kMaxPatches) kind_s[threadIdx.x] = P.t32->kind[threadIdx.x];
        for (int k = threadIdx.x; k < kCellWindow * kCellSlots; k += blockDim.x) win[k] = 0u;
    }
    if (threadIdx.x == 0) {
        int c0 = 0;
        for (int k = start; k < end && k < start + 64; ++k) {
            const int t = P.p.tet[k];
            if (t >= 0) { c0 = t / 12; break; }
        }
        w0s = max(0, c0 - kCellWindow / 16);
        qn = 0;
    }
    __syncthreads();
    const int w0 = w0s;
    unsigned ts = 0, fc = 0, ab = 0;
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
        load_attributes32<ATTRS>(P, ci, s);
        // the outcome: 0 moved, 1 removed, 2 at a reflecting patch (queued).
        // The rare outcomes set flags only, so the common tail below runs
        // once for the warp, whatever its lanes met on the way.
        int fate = 0;
        unsigned faces = 0;
        if (P.solve_movement) {
            if (P.charged && s.zf != 0.f) push32<PUSHER>(P, tri_s, s, P.dt_f);
            if (!(s.U[0] * s.U[0] + s.U[1] * s.U[1] + s.U[2] * s.U[2] < float(kC) * float(kC))) {
                atomicMax(&P.counters->error, int(PICGPU_SPEED_OF_LIGHT));
                fate = 1;
            }
            // the displacement U dt in normalised cell units, followed in
            // the cell frame (empty axes: the centre plane)
            float d0 = s.U[0] * P.dth[0], d1 = s.U[1] * P.dth[1], d2 = s.U[2] * P.dth[2];
            float e0 = 0.f, e1 = 0.f, e2 = 0.f;
            if (fate == 0) {
                float x0, x1, x2;
                bary_to_cell(s.tet, s.y, x0, x1, x2);
                x0 *= P.keep[0];
                x1 *= P.keep[1];
                x2 *= P.keep[2];
                e0 = x0 + d0;
                e1 = x1 + d1;
                e2 = x2 + d2;
                const bool out0 = fabsf(e0) > 0.5f, out1 = fabsf(e1) > 0.5f, out2 = fabsf(e2) > 0.5f;
                if (int(out0) + int(out1) + int(out2) == 1 && fmaxf(fabsf(e0), fmaxf(fabsf(e1), fabsf(e2))) <= 1.5f) {
                    // through one face and no further than the neighbour: into
                    // the neighbour, whose frame is this one shifted by a cell
                    // along the axis; a patch decides without the crossing
                    // time.  A longer step along one axis takes the loop below.
                    const int ax = out0 ? 0 : out1 ? 1 : 2;
                    const float ea = out0 ? e0 : out1 ? e1 : e2;
                    const int nb = __ldg(P.m.nbr + 6 * s.cell + 2 * ax + (ea > 0.f ? 1 : 0));
                    faces = 1;
                    if (nb >= 0) {
                        s.cell = nb;
                        const float shift = ea > 0.f ? 1.f : -1.f;
                        e0 = out0 ? e0 - shift : e0;
                        e1 = out1 ? e1 - shift : e1;
                        e2 = out2 ? e2 - shift : e2;
                    } else {
                        const int patch = -nb - 1;
                        const int kind = kind_s[patch];
                        fate = 1;
                        if (kind == PICGPU_PATCH_FLOATING || (kind == PICGPU_PATCH_CIRCUIT && P.q != 0.0))
                            atomicAdd(P.qconv + patch, parcel_charge(P, s));
                        else if (kind != PICGPU_PATCH_ABSORB)
                            fate = 2;
                    }
                } else if (out0 || out1 || out2) {
                    // through cell faces: the first face on the way per axis
                    // (|x_a| <= 1/2 after the clamp, so d_a != 0 where |e_a| > 1/2)
                    x0 = fminf(fmaxf(x0, -0.5f), 0.5f);
                    x1 = fminf(fmaxf(x1, -0.5f), 0.5f);
                    x2 = fminf(fmaxf(x2, -0.5f), 0.5f);
                    e0 = x0 + d0;
                    e1 = x1 + d1;
                    e2 = x2 + d2;
                    int budget = P.max_steps;
                    while (true) {
                        float t = 2.f;
                        int ax = 0;
                        if (fabsf(e0) > 0.5f) t = __fdividef(copysignf(0.5f, e0) - x0, d0);
                        if (fabsf(e1) > 0.5f) {
                            const float ta = __fdividef(copysignf(0.5f, e1) - x1, d1);
                            if (ta < t) { t = ta; ax = 1; }
                        }
                        if (fabsf(e2) > 0.5f) {
                            const float ta = __fdividef(copysignf(0.5f, e2) - x2, d2);
                            if (ta < t) { t = ta; ax = 2; }
                        }
                        t = fminf(fmaxf(t, 0.f), 1.f);
                        const float ea = ax == 0 ? e0 : ax == 1 ? e1 : e2;
                        const float face = ea > 0.f ? 0.5f : -0.5f;
                        x0 = ax == 0 ? face : fminf(fmaxf(x0 + t * d0, -0.5f), 0.5f);
                        x1 = ax == 1 ? face : fminf(fmaxf(x1 + t * d1, -0.5f), 0.5f);
                        x2 = ax == 2 ? face : fminf(fmaxf(x2 + t * d2, -0.5f), 0.5f);
                        const float rest = 1.f - t;
                        d0 *= rest;
                        d1 *= rest;
                        d2 *= rest;
                        ++faces;
                        const int nb = __ldg(P.m.nbr + 6 * s.cell + 2 * ax + (ea > 0.f ? 1 : 0));
                        if (nb < 0) {
                            const int patch = -nb - 1;
                            const int kind = kind_s[patch];
                            fate = 1;
                            if (kind == PICGPU_PATCH_FLOATING || (kind == PICGPU_PATCH_CIRCUIT && P.q != 0.0))
                                atomicAdd(P.qconv + patch, parcel_charge(P, s));
                            else if (kind != PICGPU_PATCH_ABSORB)
                                fate = 2;
                            break;
                        }
                        // the neighbour: the point sits on its opposite face
                        s.cell = nb;
                        x0 = ax == 0 ? -face : x0;
                        x1 = ax == 1 ? -face : x1;
                        x2 = ax == 2 ? -face : x2;
                        e0 = x0 + d0;
                        e1 = x1 + d1;
                        e2 = x2 + d2;
                        if (fmaxf(fabsf(e0), fmaxf(fabsf(e1), fabsf(e2))) <= 0.5f) break;
                        if (--budget <= 0) {
                            atomicMax(&P.counters->error, int(PICGPU_TRACK_LOOP_CAP));
                            fate = 1;
                            break;
                        }
                    }
                }
            }
            if (fate == 0) {
                cell_to_bary(e0, e1, e2, s);
                ++ts;
                store_rec(P.p, ci, s, 12 * s.cell + s.tet);
            } else if (fate == 1) {
                P.p.tet[ci] = -1;
                ++ab;
            } else {
                // a reflecting patch: the crossing tracker repeats this step
                // from the start record with the pushed velocity
                __stcs(P.p.u32[0] + ci, s.U[0]);
                __stcs(P.p.u32[1] + ci, s.U[1]);
                __stcs(P.p.u32[2] + ci, s.U[2]);
                P.xq.queue[start + atomicAdd(&qn, 1)] = ci;
            }
            fc += faces;
        }
        if (fate == 0) deposit_cell32(P, tri_s, s, w0, win);
    }
    __syncthreads();
    if (P.has_value) {
        const int nslot = min(kCellWindow, P.m.n_cells - w0) * 9;
        unsigned long long* g = P.acc9 + 9 * size_t(w0);
        for (int k = threadIdx.x; k < nslot; k += blockDim.x) {
            const int rel = k / 9, j = k - 9 * rel;
            const unsigned* a = win + kCellSlots * rel;
            unsigned long long v = 0;
            if (j == 0) {
#pragma unroll
                for (int q = 0; q < kCellSub; ++q) v += a[q];
            } else {
                v = a[kCellSub - 1 + j];
            }
            if (v) atomicAdd(g + k, v);
        }
    }
    if (threadIdx.x == 0) {
        P.xq.count[blockIdx.x] = qn;
        P.xq.start[blockIdx.x] = start;
    }
    warp_add_counter<float>(&P.counters->tet_steps, ts);
    warp_add_counter<float>(&P.counters->faces, fc);
    warp_add_counter<float>(&P.counters->absorbed, ab);
}

// Charge deposit straight into the global accumulators.
__device__ __forceinline__ void deposit_global32(const MoveParams& P, const unsigned* tri_of, const S32& s) {
    if (!P.has_value) return;
    deposit_heavy32(P, tri_of, s);
}

// The particles the in-cell mover queued, block b of this grid taking block
// b's segment: barycentric tracking from the start position with the pushed
// velocity (PICParcel::moveForward: cell faces, patches, velocity sync),
// then store and deposit.
template <int PUSHER, bool ATTRS>
__global__ void __launch_bounds__(256) track_queue_kernel_fp32(MoveParams P) {
    __shared__ Tables32 T;
    const int cnt = P.xq.count[blockIdx.x];
    if (cnt <= 0) return;  // block-uniform
    const int qs = P.xq.start[blockIdx.x];
    {
        const unsigned* src = reinterpret_cast<const unsigned*>(P.t32);
        unsigned* dst = reinterpret_cast<unsigned*>(&T);
        for (int k = threadIdx.x; k < int(sizeof(Tables32) / 4); k += blockDim.x) dst[k] = src[k];
    }
    __syncthreads();
    unsigned ts = 0, fc = 0, wl = 0, ab = 0;
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
        const int i = P.xq.queue[qs + k];
        const Rec r = load_rec(P.p, i);
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
        load_attributes32<ATTRS>(P, i, s);
        Tally td{0u, 0u, 0u, true};
        track32<PUSHER>(P, T, s, td);
        ts += td.tet_steps;
        fc += td.faces;
        wl += td.walls;
        if (!td.keep) {
            P.p.tet[i] = -1;
            ++ab;
            continue;
        }
        store_rec(P.p, i, s, 12 * s.cell + s.tet);
        deposit_global32(P, T.tri, s);
    }
    warp_add_counter<float>(&P.counters->tet_steps, ts);
    warp_add_counter<float>(&P.counters->faces, fc);
    warp_add_counter<float>(&P.counters->walls, wl);
    warp_add_counter<float>(&P.counters->absorbed, ab);
}

template <int PUSHER, bool ATTRS>
int launch_kernels(const MoveParams& P, int blocks, int chunk, bool cell, cudaStream_t s) {
    const size_t smem = size_t(kWindow) * 9 * sizeof(unsigned);
    if (!cell) {
        move_kernel_fp32<PUSHER, ATTRS><<<blocks, 256, smem, s>>>(P, chunk);
        return 1;
    }
    const size_t cell_smem = size_t(kCellWindow) * kCellSlots * sizeof(unsigned);
    move_cell_kernel_fp32<PUSHER, ATTRS><<<blocks, 256, cell_smem, s>>>(P, chunk);
    if (!P.solve_movement || !P.reflecting) return 1;
    track_queue_kernel_fp32<PUSHER, ATTRS><<<blocks, 256, 0, s>>>(P);
    return 2;
}

// Stores with per-parcel attributes take the kernels that read them.
template <int PUSHER>
int launch_pusher(const MoveParams& P, int blocks, int chunk, bool cell, cudaStream_t s) {
    return P.p.nw ? launch_kernels<PUSHER, true>(P, blocks, chunk, cell, s)
                  : launch_kernels<PUSHER, false>(P, blocks, chunk, cell, s);
}

}  // namespace

// grid: the number of resident blocks to use (5 per SM); each block takes one
// contiguous chunk (a multiple of 256 particles) of [P.first, P.n).  With
// P.n_dev set the counts are read on the device and all grid blocks launch.
// Uniform block meshes with a crossing queue run the in-cell mover and the
// crossing tracker; other meshes the general kernel.  Returns the number of
// kernels launched.
int launch_move_fp32(const MoveParams& P, int grid, cudaStream_t s) {
    int blocks, chunk;
    if (P.n_dev) {
        // device-resident counts: the kernel sizes its chunks; grid fixed
        blocks = grid;
        chunk = 0;
    } else {
        const long work = long(P.n) - P.first;
        if (work <= 0) return 0;
        const long tiles = (work + 255) / 256;
        const long per = (tiles + grid - 1) / grid;
        chunk = int(per * 256);
        blocks = int((work + chunk - 1) / chunk);
    }
    const bool cell = P.cell_mover && P.xq.queue && blocks <= P.xq.capacity;
    switch (P.pusher) {
        case PICGPU_PUSHER_BORIS: return launch_pusher<PICGPU_PUSHER_BORIS>(P, blocks, chunk, cell, s);
        case PICGPU_PUSHER_BORIS_NR: return launch_pusher<PICGPU_PUSHER_BORIS_NR>(P, blocks, chunk, cell, s);
        case PICGPU_PUSHER_VAY: return launch_pusher<PICGPU_PUSHER_VAY>(P, blocks, chunk, cell, s);
        case PICGPU_PUSHER_HIGUERA_CARY: return launch_pusher<PICGPU_PUSHER_HIGUERA_CARY>(P, blocks, chunk, cell, s);
        default: return launch_pusher<PICGPU_PUSHER_NONE>(P, blocks, chunk, cell, s);
    }
}

}  // namespace pgd
