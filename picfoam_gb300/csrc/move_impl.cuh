// move_impl.cuh -- fused push + barycentric track + charge deposit.
//
// One thread moves one particle through one time step, the work of
// PICParcel::move / moveForward (PICMCCFVM/parcels/Templates/PICParcel/PICParcel.C:38-144)
// with the selected ParticlePusher, FieldWeigthing and ChargeDistribution
// fused in, then deposits its charge (ChargeDistribution::add,
// submodels/ChargeDistribution/VolumeWeighting/VolumeWeighting.C:105-124) so
// the particle record is read and written once per step.
//
// Instantiated twice: Real = double in move_fp64.cu (built with --fmad=false,
// evaluation order identical to the CPU oracle, so the FP64 form is bit-exact)
// and Real = float in move_fp32.cu (the mixed form).
#pragma once

#include "common.cuh"

namespace pgd {

template <class Real> struct RealTraits;
template <> struct RealTraits<double> {
    static __device__ __forceinline__ double thr() { return 1e-12; }
};
template <> struct RealTraits<float> {
    static __device__ __forceinline__ float thr() { return 1e-6f; }
};

// Per-precision access to the species and field constants.  The FP64 form
// evaluates q dt/2 / m exactly as the oracle does; the FP32 form uses the
// host-rounded float copies.
template <class Real> struct PC;
template <> struct PC<double> {
    static __device__ __forceinline__ double dt(const MoveParams& P) { return P.dt; }
    static __device__ __forceinline__ double B(const MoveParams& P, int a) { return P.B[a]; }
    // the parcel's charge is the species charge times its charge modifier zf
    // (PICCloud.C:368); zf = 1 leaves q dt/2 / m as it is
    static __device__ __forceinline__ double qdm(const MoveParams& P, double half_dt, double zf) {
        return P.q * zf * half_dt / P.mass;
    }
    static __device__ __forceinline__ double centre(const MoveParams& P, int a) { return P.m.mesh_centre[a]; }
    static __device__ __forceinline__ double cc(const MoveParams& P, int c, int a) {
        return P.m.cc[3 * size_t(c) + a];
    }
};
template <> struct PC<float> {
    static __device__ __forceinline__ float dt(const MoveParams& P) { return P.dt_f; }
    static __device__ __forceinline__ float B(const MoveParams& P, int a) { return P.B_f[a]; }
    static __device__ __forceinline__ float qdm(const MoveParams& P, float half_dt, float zf) {
        return P.qm_f * zf * half_dt;
    }
    static __device__ __forceinline__ float centre(const MoveParams& P, int a) { return P.centre_f[a]; }
    static __device__ __forceinline__ float cc(const MoveParams& P, int c, int a) {
        return P.m.cc32[3 * size_t(c) + a];
    }
};

template <class Real>
__device__ __forceinline__ Real dot3(const Real* a, const Real* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
template <class Real>
__device__ __forceinline__ void cross3(const Real* a, const Real* b, Real* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

template <class Real>
struct PState {
    int cell, tet;
    Real y[4];
    Real U[3];
    Real zf;      // charge modifier (1 without per-parcel attributes)
    double nw;    // nParticle (the species weight without per-parcel attributes)
};

// The parcel's charge modifier and weight: per parcel when the store has
// the arrays, else 1 and the species weight.
template <class Real>
__device__ __forceinline__ void load_attributes(const MoveParams& P, int i, PState<Real>& s) {
    if (P.p.nw) {
        s.zf = Real(P.p.zq[i]);
        s.nw = P.p.nw[i];
    } else {
        s.zf = Real(1);
        s.nw = P.weight;
    }
}

template <class Real> __device__ __forceinline__ const Real* e_cell(const MoveParams& P);
template <> __device__ __forceinline__ const double* e_cell<double>(const MoveParams& P) { return P.E; }
template <> __device__ __forceinline__ const float* e_cell<float>(const MoveParams& P) { return P.E32; }
template <class Real> __device__ __forceinline__ const Real* e_point(const MoveParams& P);
template <> __device__ __forceinline__ const double* e_point<double>(const MoveParams& P) { return P.Ept; }
template <> __device__ __forceinline__ const float* e_point<float>(const MoveParams& P) { return P.Ept32; }
template <class Real> __device__ __forceinline__ const Real* tetinv(const DMesh& m);
template <> __device__ __forceinline__ const double* tetinv<double>(const DMesh& m) { return m.tetinv; }
template <> __device__ __forceinline__ const float* tetinv<float>(const DMesh& m) { return m.tetinv32; }
template <class Real> __device__ __forceinline__ const Real* offsets(const DMesh& m);
template <> __device__ __forceinline__ const double* offsets<double>(const DMesh& m) { return m.offset; }
template <> __device__ __forceinline__ const float* offsets<float>(const DMesh& m) { return m.offset32; }
template <class Real> __device__ __forceinline__ const Real* fnormals(const DMesh& m);
template <> __device__ __forceinline__ const double* fnormals<double>(const DMesh& m) { return m.fnormal; }
template <> __device__ __forceinline__ const float* fnormals<float>(const DMesh& m) { return m.fnormal32; }

// FieldWeigthing::getFieldVector: VolumeWeighting (VolumeWeightingFW.C:60-67)
// interpolates cell centre + three triangle points; CellAverage
// (CellAverageFW.C:58-65) returns the cell value.
template <class Real>
__device__ __forceinline__ void field_at(const MoveParams& P, const TetConst& T,
                                         const PState<Real>& s, Real* E) {
    const Real* Ec = e_cell<Real>(P) + 3 * size_t(s.cell);
    if (P.field_weighting == PICGPU_WEIGHTING_CELL_AVERAGE) {
        E[0] = Ec[0]; E[1] = Ec[1]; E[2] = Ec[2];
        return;
    }
    const int* cp = P.m.cell_pt + 8 * size_t(s.cell);
    const Real* Ep = e_point<Real>(P);
    const Real* e1 = Ep + 3 * size_t(cp[T.tri[s.tet][0]]);
    const Real* e2 = Ep + 3 * size_t(cp[T.tri[s.tet][1]]);
    const Real* e3 = Ep + 3 * size_t(cp[T.tri[s.tet][2]]);
#pragma unroll
    for (int a = 0; a < 3; ++a)
        E[a] = Ec[a] * s.y[0] + e1[a] * s.y[1] + e2[a] * s.y[2] + e3[a] * s.y[3];
}

// BorisPusher::updateVelocity (submodels/ParticlePusher/BorisPusher/BorisPusher.C:69-112)
template <class Real>
__device__ __forceinline__ void push_boris(const MoveParams& P, const Real* E, const Real* Bv, Real* U, Real tt,
                                      Real zf) {
    const Real c = Real(kC);
    const Real dt2 = Real(0.5) * tt;
    const Real mU = sqrt(dot3(U, U)) / c;
    const Real g0 = sqrt(Real(1) - mU * mU);
    Real rU[3] = {U[0] / g0, U[1] / g0, U[2] / g0};
    const Real oldrU[3] = {rU[0], rU[1], rU[2]};
    const Real qdm = PC<Real>::qdm(P, dt2, zf);
    const Real rUsm[3] = {qdm * E[0], qdm * E[1], qdm * E[2]};
    rU[0] = rU[0] + rUsm[0]; rU[1] = rU[1] + rUsm[1]; rU[2] = rU[2] + rUsm[2];
    if (P.rotation) {
        const Real a0 = sqrt(dot3(oldrU, oldrU)) / c, a1 = sqrt(dot3(rU, rU)) / c;
        const Real lF = (sqrt(Real(1) + a0 * a0) + sqrt(Real(1) + a1 * a1)) / Real(2);
        const Real t[3] = {qdm * Bv[0] / lF, qdm * Bv[1] / lF, qdm * Bv[2] / lF};
        Real cr[3];
        cross3(rU, t, cr);
        const Real Ud[3] = {rU[0] + cr[0], rU[1] + cr[1], rU[2] + cr[2]};
        const Real den = Real(1) + dot3(t, t);
        const Real sv[3] = {Real(2) * t[0] / den, Real(2) * t[1] / den, Real(2) * t[2] / den};
        cross3(Ud, sv, cr);
        rU[0] = rU[0] + cr[0]; rU[1] = rU[1] + cr[1]; rU[2] = rU[2] + cr[2];
    }
    rU[0] = rU[0] + rUsm[0]; rU[1] = rU[1] + rUsm[1]; rU[2] = rU[2] + rUsm[2];
    const Real mr = sqrt(dot3(rU, rU)) / c;
    const Real g1 = sqrt(Real(1) + mr * mr);
    U[0] = rU[0] / g1; U[1] = rU[1] / g1; U[2] = rU[2] / g1;
}

// BorisNRPusher::updateVelocity (BorisNRPusher.C:69-99)
template <class Real>
__device__ __forceinline__ void push_boris_nr(const MoveParams& P, const Real* E, const Real* Bv, Real* U, Real tt,
                                      Real zf) {
    const Real dt2 = Real(0.5) * tt;
    const Real alpha = PC<Real>::qdm(P, dt2, zf);
    Real W[3] = {U[0] + alpha * E[0], U[1] + alpha * E[1], U[2] + alpha * E[2]};
    if (P.rotation) {
        const Real t[3] = {alpha * Bv[0], alpha * Bv[1], alpha * Bv[2]};
        Real cr[3];
        cross3(W, t, cr);
        const Real Ud[3] = {W[0] + cr[0], W[1] + cr[1], W[2] + cr[2]};
        const Real den = Real(1) + dot3(t, t);
        const Real sv[3] = {Real(2) * t[0] / den, Real(2) * t[1] / den, Real(2) * t[2] / den};
        cross3(Ud, sv, cr);
        W[0] = W[0] + cr[0]; W[1] = W[1] + cr[1]; W[2] = W[2] + cr[2];
    }
    U[0] = W[0] + alpha * E[0]; U[1] = W[1] + alpha * E[1]; U[2] = W[2] + alpha * E[2];
}

// VayPusher::updateVelocity (VayPusher.C:54-100); U x T uses v (VayPusher.C:81).
template <class Real>
__device__ __forceinline__ void push_vay(const MoveParams& P, const Real* E, const Real* Bv, Real* U, Real tt,
                                      Real zf) {
    const Real c = Real(kC);
    const Real dt2 = Real(0.5) * tt;
    const Real mU = sqrt(dot3(U, U)) / c;
    const Real lF = Real(1) / sqrt(Real(1) - mU * mU);
    const Real rU0[3] = {lF * U[0], lF * U[1], lF * U[2]};
    const Real qe = PC<Real>::qdm(P, tt, zf);
    Real Ud[3] = {rU0[0] + qe * E[0], rU0[1] + qe * E[1], rU0[2] + qe * E[2]};
    const Real qb = PC<Real>::qdm(P, dt2, zf);
    Real T[3] = {qb * Bv[0], qb * Bv[1], qb * Bv[2]};
    Real cr[3];
    cross3(U, T, cr);
    Ud[0] = Ud[0] + cr[0]; Ud[1] = Ud[1] + cr[1]; Ud[2] = Ud[2] + cr[2];
    const Real mUd = sqrt(dot3(Ud, Ud)) / c;
    Real alpha = Real(1) + mUd * mUd;
    const Real T2 = dot3(T, T);
    Real s = alpha - T2;
    const Real udt = dot3(Ud, T) / c;
    const Real us2 = udt * udt;
    alpha = Real(1) / sqrt(Real(0.5) * (s + sqrt(s * s + Real(4) * (T2 + us2))));
    T[0] = alpha * T[0]; T[1] = alpha * T[1]; T[2] = alpha * T[2];
    s = Real(1) / (Real(1) + dot3(T, T));
    alpha = dot3(Ud, T);
    cross3(Ud, T, cr);
    Real rU[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) rU[a] = s * ((Ud[a] + alpha * T[a]) + cr[a]);
    const Real mr = sqrt(dot3(rU, rU)) / c;
    const Real g1 = sqrt(Real(1) + mr * mr);
    U[0] = rU[0] / g1; U[1] = rU[1] / g1; U[2] = rU[2] / g1;
}

// HigueraCaryPusher::updateVelocity (HigueraCary.C:69-115)
template <class Real>
__device__ __forceinline__ void push_hc(const MoveParams& P, const Real* E, const Real* Bv, Real* U, Real tt,
                                      Real zf) {
    const Real c = Real(kC);
    const Real dt2 = Real(0.5) * tt;
    const Real mU = sqrt(dot3(U, U)) / c;
    const Real g0 = sqrt(Real(1) - mU * mU);
    Real rU[3] = {U[0] / g0, U[1] / g0, U[2] / g0};
    const Real qdm = PC<Real>::qdm(P, dt2, zf);
    const Real rUsm[3] = {qdm * E[0], qdm * E[1], qdm * E[2]};
    rU[0] = rU[0] + rUsm[0]; rU[1] = rU[1] + rUsm[1]; rU[2] = rU[2] + rUsm[2];
    if (P.rotation) {
        const Real mr0 = sqrt(dot3(rU, rU)) / c;
        const Real gfm2 = Real(1) + mr0 * mr0;
        Real t[3] = {qdm * Bv[0], qdm * Bv[1], qdm * Bv[2]};
        const Real beta2 = dot3(t, t);
        const Real gb = gfm2 - beta2;
        const Real tr = dot3(t, rU);
        const Real iG = Real(1) / sqrt(Real(0.5) * (gb + sqrt(gb * gb + Real(4) * (beta2 + tr * tr))));
        t[0] = iG * t[0]; t[1] = iG * t[1]; t[2] = iG * t[2];
        Real cr[3];
        cross3(rU, t, cr);
        const Real Ud[3] = {rU[0] + cr[0], rU[1] + cr[1], rU[2] + cr[2]};
        const Real den = Real(1) + dot3(t, t);
        const Real sv[3] = {Real(2) * t[0] / den, Real(2) * t[1] / den, Real(2) * t[2] / den};
        cross3(Ud, sv, cr);
        rU[0] = rU[0] + cr[0]; rU[1] = rU[1] + cr[1]; rU[2] = rU[2] + cr[2];
    }
    rU[0] = rU[0] + rUsm[0]; rU[1] = rU[1] + rUsm[1]; rU[2] = rU[2] + rUsm[2];
    const Real mr = sqrt(dot3(rU, rU)) / c;
    const Real g1 = sqrt(Real(1) + mr * mr);
    U[0] = rU[0] / g1; U[1] = rU[1] / g1; U[2] = rU[2] / g1;
}

// The magnetic field the pushers use: the cell value (B[celli], as every
// picFoam pusher reads it, e.g. BorisPusher.C:100) when a per-cell field is
// set, else the uniform one.
template <class Real>
__device__ __forceinline__ void cell_B(const MoveParams& P, int cell, Real* Bv) {
    if (P.Bc) {
#pragma unroll
        for (int a = 0; a < 3; ++a) Bv[a] = Real(P.Bc[3 * size_t(cell) + a]);
    } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) Bv[a] = PC<Real>::B(P, a);
    }
}

template <class Real>
__device__ __forceinline__ void push(const MoveParams& P, const TetConst& T, PState<Real>& s, Real tt) {
    if (P.pusher == PICGPU_PUSHER_NONE) return;
    Real E[3], Bv[3];
    field_at(P, T, s, E);
    cell_B(P, s.cell, Bv);
    switch (P.pusher) {
        case PICGPU_PUSHER_BORIS: push_boris(P, E, Bv, s.U, tt, s.zf); break;
        case PICGPU_PUSHER_BORIS_NR: push_boris_nr(P, E, Bv, s.U, tt, s.zf); break;
        case PICGPU_PUSHER_VAY: push_vay(P, E, Bv, s.U, tt, s.zf); break;
        default: push_hc(P, E, Bv, s.U, tt, s.zf); break;
    }
}

// One tet step: barycentric displacement, first coordinate to reach zero,
// clamp and renormalise.  Returns the hit tet face or -1.
template <class Real>
__device__ __forceinline__ int tet_step(const MoveParams& P, PState<Real>& s, const Real* dx, Real* lam_out) {
    const Real* inv = tetinv<Real>(P.m) + (size_t(P.m.cell_class[s.cell]) * 12 + s.tet) * 9;
    Real dy[4];
    dy[1] = inv[0] * dx[0] + inv[1] * dx[1] + inv[2] * dx[2];
    dy[2] = inv[3] * dx[0] + inv[4] * dx[1] + inv[5] * dx[2];
    dy[3] = inv[6] * dx[0] + inv[7] * dx[1] + inv[8] * dx[2];
    dy[0] = -(dy[1] + dy[2] + dy[3]);
    const Real S = fabs(dy[0]) + fabs(dy[1]) + fabs(dy[2]) + fabs(dy[3]);
    const Real thr = -RealTraits<Real>::thr() * S;
    Real lam = Real(1);
    int hit = -1;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (dy[i] < thr) {
            const Real l = -s.y[i] / dy[i];
            if (l < lam) { lam = l; hit = i; }
        }
    }
    Real y[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) y[i] = s.y[i] + lam * dy[i];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (i == hit) y[i] = Real(0);
#pragma unroll
    for (int i = 0; i < 4; ++i) y[i] = fmax(y[i], Real(0));
    const Real r = Real(1) / (y[0] + y[1] + y[2] + y[3]);
#pragma unroll
    for (int i = 0; i < 4; ++i) s.y[i] = y[i] * r;
    *lam_out = lam;
    return hit;
}

template <class Real>
__device__ __forceinline__ void sync_velocity(const MoveParams& P, const TetConst& T, PState<Real>& s,
                                              Real fraction) {
    if (P.sync && P.charged && s.zf != Real(0)) push(P, T, s, fraction * PC<Real>::dt(P));
}

struct TrackTally {
    unsigned tet_steps, faces, walls;
    bool keep, capped, resync;
};

// PICParcel::hitPatch (PICParcel.C:153-184) for the patch models in scope.
template <class Real>
__device__ __forceinline__ void hit_patch(const MoveParams& P, const TetConst& T, const PatchConst& PCs,
                                          PState<Real>& s, int patch, Real sf, TrackTally& td) {
    const int kind = PCs.kind[patch];
    if (kind == PICGPU_PATCH_ABSORB) { td.keep = false; return; }
    // FloatingPotential deletes every parcel; a circuit electrode
    // (circuitRLC.C:268-288) deletes charged parcels and reflects neutral ones
    if (kind == PICGPU_PATCH_FLOATING || (kind == PICGPU_PATCH_CIRCUIT && P.q != 0.0)) {
        td.keep = false;
        atomicAdd(P.qconv + patch, P.p.nw ? s.nw * (P.q * double(s.zf)) : P.weight * P.q);
        return;
    }
    const int f = s.tet / 2;
    const Real* n = fnormals<Real>(P.m) + size_t(P.m.cell_class[s.cell]) * 18 + 3 * f;
    if (kind == PICGPU_PATCH_WALL || kind == PICGPU_PATCH_CIRCUIT) {
        sync_velocity(P, T, s, sf - Real(0.5));
        td.walls++;
        td.resync = true;
    }
    const Real Un = s.U[0] * n[0] + s.U[1] * n[1] + s.U[2] * n[2];
    if (Un > Real(0)) {
        const Real t = Real(2) * Un;
        s.U[0] = s.U[0] - t * n[0];
        s.U[1] = s.U[1] - t * n[1];
        s.U[2] = s.U[2] - t * n[2];
    }
}

template <class Real>
__device__ __forceinline__ void track_to_and_hit_face(const MoveParams& P, const TetConst& T,
                                                      const PatchConst& PCs, PState<Real>& s,
                                                      const Real* disp, Real f, Real& sf,
                                                      TrackTally& td, int& budget) {
    Real rem = Real(1);
    for (;;) {
        if (--budget < 0) { td.capped = true; sf = Real(1); return; }
        const Real dx[3] = {rem * disp[0], rem * disp[1], rem * disp[2]};
        Real lam;
        const int hit = tet_step(P, s, dx, &lam);
        td.tet_steps++;
        if (hit < 0) { sf = Real(1); return; }
        sf = sf + (f * rem) * lam;
        if (hit > 0) {
            Real y[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int src = T.inner_src[s.tet][hit][j];
                Real v = Real(0);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (q == src) v = s.y[q];
                y[j] = v;
            }
            s.tet = T.inner_next[s.tet][hit];
#pragma unroll
            for (int j = 0; j < 4; ++j) s.y[j] = y[j];
            rem = rem * (Real(1) - lam);
            continue;
        }
        const int face = s.tet / 2;
        const int nb = P.m.nbr[6 * size_t(s.cell) + face];
        td.faces++;
        if (nb >= 0) {
            Real y[4];
            y[0] = Real(0);
#pragma unroll
            for (int j = 1; j < 4; ++j) {
                const int src = T.cross_src[s.tet][j];
                Real v = Real(0);
#pragma unroll
                for (int q = 1; q < 4; ++q)
                    if (q == src) v = s.y[q];
                y[j] = v;
            }
            s.tet = T.cross_next[s.tet];
            s.cell = nb;
#pragma unroll
            for (int j = 0; j < 4; ++j) s.y[j] = y[j];
            return;
        }
        hit_patch(P, T, PCs, s, -nb - 1, sf, td);
        return;
    }
}

template <class Real> __device__ __forceinline__ Real* ybuf(const DSpecies& p, int a);
template <> __device__ __forceinline__ double* ybuf<double>(const DSpecies& p, int a) { return p.y64[a]; }
template <> __device__ __forceinline__ float* ybuf<float>(const DSpecies& p, int a) { return p.y32[a]; }
template <class Real> __device__ __forceinline__ Real* ubuf(const DSpecies& p, int a);
template <> __device__ __forceinline__ double* ubuf<double>(const DSpecies& p, int a) { return p.u64[a]; }
template <> __device__ __forceinline__ float* ubuf<float>(const DSpecies& p, int a) { return p.u32[a]; }

__device__ __forceinline__ void deposit_add(const MoveParams& P, double* dst64, long long* dstfix,
                                            size_t idx, double v) {
    if (P.deposit_mode == PICGPU_DEPOSIT_FIXED_POINT) {
        const long long q = __double2ll_rn(v * P.fix_scale);
        atomicAdd(reinterpret_cast<unsigned long long*>(dstfix + idx), (unsigned long long)q);
    } else {
        atomicAdd(dst64 + idx, v);
    }
}

// ChargeDistribution::add for one particle at its end-of-step position.
__device__ __forceinline__ void deposit(const MoveParams& P, const TetConst& T, const PState<double>& s) {
    // charge x nParticle of the parcel (VolumeWeighting.C:114)
    const double value = P.p.nw ? P.q * s.zf * s.nw : P.value;
    if (value == 0.0) return;
    if (P.charge_distribution == PICGPU_WEIGHTING_CELL_AVERAGE) {
        deposit_add(P, P.cc_data, P.cc_fix, s.cell, value);
        return;
    }
    const int* cp = P.m.cell_pt + 8 * size_t(s.cell);
    deposit_add(P, P.cc_data, P.cc_fix, s.cell, double(s.y[0]) * value);
#pragma unroll
    for (int i = 0; i < 3; ++i)
        deposit_add(P, P.vtx_data, P.vtx_fix, cp[T.tri[s.tet][i]], double(s.y[i + 1]) * value);
}

template <class Real>
__device__ __forceinline__ void warp_add_counter(unsigned long long* dst, unsigned v) {
    unsigned long long x = v;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(dst, x);
}

// The per-particle step.  Returns through the tally; the particle record is
// written back in place (tet = -1 once removed).
template <class Real>
__device__ __forceinline__ void move_one(const MoveParams& P, const TetConst& T, const PatchConst& PCs,
                                         int i, TrackTally& td) {
    int32_t tetg = P.p.tet[i];
    if (tetg < 0) return;
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
    if (P.solve_movement) {
        const Real dt = PC<Real>::dt(P);
        // PICParcel::move pushes charged parcels only (PICParcel.C:55)
        if (P.charged && s.zf != Real(0)) push(P, T, s, dt);
        const Real c = Real(kC);
        if (!(sqrt(dot3(s.U, s.U)) < c)) {
            td.keep = false;
            atomicMax(&P.counters->error, int(PICGPU_SPEED_OF_LIGHT));
        } else {
            Real sf = Real(0);
            int resync = 0;
            int budget = P.max_steps;
            while (td.keep && sf < Real(1)) {
                Real Ut[3] = {s.U[0], s.U[1], s.U[2]};
                Real dev[3] = {Real(0), Real(0), Real(0)};
                if (P.m.any_empty) {
                    const Real* off = offsets<Real>(P.m) + size_t(P.m.cell_class[s.cell]) * 24;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        if (!P.m.empty[a]) continue;
                        Ut[a] = Real(0);
                        const Real x = PC<Real>::cc(P, s.cell, a) + s.y[1] * off[3 * T.tri[s.tet][0] + a] +
                                       s.y[2] * off[3 * T.tri[s.tet][1] + a] +
                                       s.y[3] * off[3 * T.tri[s.tet][2] + a];
                        dev[a] = x - PC<Real>::centre(P, a);
                    }
                }
                const Real f = Real(1) - sf;
                const Real fdt = f * dt;
                const Real disp[3] = {fdt * Ut[0] - dev[0], fdt * Ut[1] - dev[1], fdt * Ut[2] - dev[2]};
                td.resync = false;
                track_to_and_hit_face(P, T, PCs, s, disp, f, sf, td, budget);
                if (td.capped) break;
                if (td.resync && td.keep) {
                    resync++;
                    if (resync > 1) { td.resync = false; continue; }
                    sync_velocity(P, T, s, Real(0.5) - sf);
                    td.resync = false;
                }
            }
            if (td.capped) {
                td.keep = false;
                atomicMax(&P.counters->error, int(PICGPU_TRACK_LOOP_CAP));
            }
        }
    }
    if (!td.keep) {
        P.p.tet[i] = -1;
        return;
    }
    P.p.tet[i] = 12 * s.cell + s.tet;
    ybuf<Real>(P.p, 0)[i] = s.y[1];
    ybuf<Real>(P.p, 1)[i] = s.y[2];
    ybuf<Real>(P.p, 2)[i] = s.y[3];
    ubuf<Real>(P.p, 0)[i] = s.U[0];
    ubuf<Real>(P.p, 1)[i] = s.U[1];
    ubuf<Real>(P.p, 2)[i] = s.U[2];
    deposit(P, T, s);
}

}  // namespace pgd
