// mcc_fp32.cu -- the background electron-neutral MCC of the FP32 store in
// FP32 arithmetic.
//
// The same null-collision step as mcc_kernel in collide.cu
// (ElectronNeutralCollisionModel.C:703-829: candidates with replacement from
// the cell's electrons, a gas partner from the drifting Maxwellian, the
// start-of-step (sigma v)_max in the acceptance test, elastic / excitation /
// ionisation by one uniform, NanbuElectronNeutralCollision.C:60-131 for the
// scattering, the ionisation energy sharing of
// ElectronNeutralCollisionModel.C:655-659), computed in FP32.  GB300 issues
// FP32 at 64 times its FP64 rate, and the FP32 store keeps velocities in
// FP32 anyway; the per-cell remainder and (sigma v)_max stay FP64.
// Where FP32 would lose the quantity, the form is changed, not the physics:
//   * the kinetic energy from gamma - 1 by its series below v^2/c^2 = 1e-3
//     (1 / sqrt(1 - b) rounds to 1 at plasma energies);
//   * Nanbu's cos(chi) = (e + 2 - 2 (1 + e)^R) / e as 1 - 2 t / e with
//     t = expm1(R log1p(e)) (the difference of two numbers near 2 otherwise).
// Collision counts and velocity moments agree with the FP64 kernel
// statistically (tests/test_gpu_statistics.py, 16 seeds).
#include <cuda_runtime.h>

#include "collide.h"

namespace pgd {
namespace {

constexpr float kC2 = float(kC * kC);
constexpr float kTwoPi = 6.283185307f;

struct F3 {
    float x, y, z;
};

__device__ __forceinline__ float uni(Philox& r) { return float(r.u32() >> 8) * (1.f / 16777216.f); }

// Two standard normals (Box-Muller).
__device__ __forceinline__ void normal2(Philox& r, float& a, float& b) {
    const float u1 = 1.f - uni(r), u2 = uni(r);
    const float rad = sqrtf(-2.f * __logf(u1));
    float s, c;
    __sincosf(kTwoPi * u2, &s, &c);
    a = rad * c;
    b = rad * s;
}

__device__ __forceinline__ float norm3(F3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }

// NanbuElectronNeutralCollision::updateVelocity (:97-131) in FP32.
__device__ void nanbu32(float eV, F3& Ue, F3& Un, float ke, float kn, Philox& r) {
    const float phi = kTwoPi * uni(r);
    const float R = uni(r);
    float cosChi, sinChi;
    if (eV < 1e-30f) {
        cosChi = 1.f;
    } else {
        const float t = expm1f(R * log1pf(eV));
        cosChi = 1.f - 2.f * t / eV;
    }
    if (cosChi * cosChi > 1.f) {
        cosChi = copysignf(1.f, cosChi);
        sinChi = 0.f;
    } else {
        sinChi = sqrtf(1.f - cosChi * cosChi);
    }
    const F3 g = {Ue.x - Un.x, Ue.y - Un.y, Ue.z - Un.z};
    const float gm = norm3(g);
    const float gp = sqrtf(g.y * g.y + g.z * g.z);
    float sp, cp;
    __sincosf(phi, &sp, &cp);
    const float igp = 1.f / gp;
    const F3 h = {gp * cp, -(g.y * g.x * cp + gm * g.z * sp) * igp, -(g.z * g.x * cp - gm * g.y * sp) * igp};
    const float oc = 1.f - cosChi;
    const F3 d = {oc * g.x + sinChi * h.x, oc * g.y + sinChi * h.y, oc * g.z + sinChi * h.z};
    Ue = {Ue.x - ke * d.x, Ue.y - ke * d.y, Ue.z - ke * d.z};
    Un = {Un.x + kn * d.x, Un.y + kn * d.y, Un.z + kn * d.z};
}

// The tables share one energy axis: one bracket, every table read at it.
struct Bracket32 {
    int lo, hi, exact;
};
__device__ Bracket32 bracket32(float x, const float* e, int n) {
    if (x <= e[0]) return {0, 0, 0};
    if (x >= e[n - 1]) return {n - 1, n - 1, n - 1};
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (e[mid] <= x) lo = mid; else hi = mid;
    }
    return {lo, hi, e[lo] == x ? lo : -1};
}
__device__ __forceinline__ float at32(const Bracket32& b, float x, const float* e, const float* v) {
    if (b.exact >= 0) return v[b.exact];
    return v[b.lo] + ((x - e[b.lo]) / (e[b.hi] - e[b.lo])) * (v[b.hi] - v[b.lo]);
}

__global__ void __launch_bounds__(256) mcc_fp32_kernel(MccParams M, DSpecies el, Secondary* __restrict__ stage) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells) return;
    const int eC = M.e_start[c + 1] - M.e_start[c];
    const double sv = M.svmax[c];
    const double coll = M.rem[c] + double(eC) * M.n_gas * sv * M.dt;
    const long nC = long(coll);
    M.rem[c] = coll - double(nC);
    if (nC == 0 || eC == 0) return;
    const int* list = M.e_idx + M.e_start[c];
    const int n = M.n_xs;
    const float* E = M.xs32;
    const float* EL = E + n;
    const float* EX = E + 2 * n;
    const float* IZ = E + 3 * n;
    Philox r(M.seed, kStreamMcc, uint32_t(c), M.step_dev ? *M.step_dev : M.step);
    const float svf = float(sv);
    double sv_run = sv;
    const float vth = float(M.vth_gas);
    const F3 drift = {float(M.drift[0]), float(M.drift[1]), float(M.drift[2])};
    const float me = float(M.me), mg = float(M.mg);
    const float ke = mg / (mg + me), kn = me / (mg + me);
    const float ex_th = float(M.ex_th), iz_th = float(M.iz_th);
    const float wEwN = float(M.wEwN), wNwE = float(M.wNwE);
    unsigned long long nel = 0, nex = 0, niz = 0;
    const int base = M.cand_off[c];
    const bool room = long(base) + nC <= M.stage_cap;
    if (!room) {
        // this cell's slots below the capacity stay unused: clear them so
        // that no stale flag is appended
        atomicExch(M.overflow, 1);
        for (long k = base; k < long(base) + nC && k < M.stage_cap; ++k) stage[k].flag = 0;
    }
    for (long i = 0; i < nC; ++i) {
        int j = int(uni(r) * float(eC));
        if (j >= eC) j = eC - 1;
        const int pi = list[j];
        F3 Ue = {el.u32[0][pi], el.u32[1][pi], el.u32[2][pi]};
        float n0, n1, n2, n3;
        normal2(r, n0, n1);
        normal2(r, n2, n3);
        F3 Un = {vth * n0 + drift.x, vth * n1 + drift.y, vth * n2 + drift.z};
        const F3 d = {Ue.x - Un.x, Ue.y - Un.y, Ue.z - Un.z};
        const float c2 = d.x * d.x + d.y * d.y + d.z * d.z;
        const float cR = sqrtf(c2);
        const float b = c2 / kC2;
        const float gm1 = b < 1e-3f ? b * (0.5f + b * (0.375f + b * 0.3125f)) : 1.f / sqrtf(1.f - b) - 1.f;
        float eV = gm1 * M.me_c2_eV;
        const Bracket32 xb = bracket32(eV, E, n);
        const float Qel = at32(xb, eV, E, EL);
        const float Qex = at32(xb, eV, E, EX);
        const float Qiz = at32(xb, eV, E, IZ);
        const float Qt = Qel + Qex + Qiz;
        sv_run = fmax(sv_run, double(Qt * cR));
        // Ru <= Q / sigma_T with sigma_T = (sigma v)_max / c_R
        const float Ru = uni(r);
        const float scale = cR / svf;
        if (Ru <= Qel * scale) {
            nel++;
            nanbu32(eV, Ue, Un, ke, kn, r);
            el.u32[0][pi] = Ue.x; el.u32[1][pi] = Ue.y; el.u32[2][pi] = Ue.z;
        } else if (eV >= ex_th && Ru <= (Qel + Qex) * scale) {
            nex++;
            const float f = sqrtf(1.f - ex_th / eV);
            Ue = {f * Ue.x, f * Ue.y, f * Ue.z};
            eV -= ex_th;
            nanbu32(eV, Ue, Un, ke, kn, r);
            el.u32[0][pi] = Ue.x; el.u32[1][pi] = Ue.y; el.u32[2][pi] = Ue.z;
        } else if (eV >= iz_th && Ru <= Qt * scale) {
            const float E0 = 2.f - 100.f / (eV + 10.f);
            const float E1 = 0.5f * (eV - iz_th) - E0;
            const float alpha = 10.3f;
            const float a0 = atanf(E0 / alpha);
            const float Ep = E0 + alpha * tanf(uni(r) * (atanf(E1 / alpha) + a0) - a0);
            const F3 preUe = Ue, preUn = Un;
            const float f = sqrtf(fmaxf(1.f - (iz_th + Ep) / eV, 0.f));
            Ue = {f * Ue.x, f * Ue.y, f * Ue.z};
            eV -= iz_th + Ep;
            nanbu32(eV, Ue, Un, ke, kn, r);
            const float rndU = uni(r);
            Secondary sc{};
            const bool make = rndU <= wEwN;
            if (make && M.create_i) {
                sc.flag |= 2;
                sc.ui[0] = Un.x; sc.ui[1] = Un.y; sc.ui[2] = Un.z;
                niz++;
            }
            if (rndU > wNwE) Ue = preUe;
            el.u32[0][pi] = Ue.x; el.u32[1][pi] = Ue.y; el.u32[2][pi] = Ue.z;
            if (make && M.create_e) {
                const float sp = sqrtf(2.f * Ep * float(1.602176634e-19 / M.me));
                const float mp = norm3(preUe);
                F3 ne = {sp * (preUe.x / mp), sp * (preUe.y / mp), sp * (preUe.z / mp)};
                F3 un2 = preUn;
                nanbu32(Ep, ne, un2, ke, kn, r);
                sc.flag |= 1;
                sc.ue[0] = ne.x; sc.ue[1] = ne.y; sc.ue[2] = ne.z;
            }
            if (sc.flag) {
                sc.tet = el.tet[pi];
                sc.y[0] = el.y32[0][pi]; sc.y[1] = el.y32[1][pi]; sc.y[2] = el.y32[2][pi];
                sc.tet_i = sc.tet;
                for (int a = 0; a < 3; ++a) sc.y_i[a] = sc.y[a];
            }
            if (room) stage[base + i] = sc;
            continue;
        }
        if (room) stage[base + i].flag = 0;
    }
    if (sv_run > sv) M.svmax[c] = sv_run;
    if (M.iz_cell && niz) M.iz_cell[c] += niz;
    atomicAdd(M.counts + 0, (unsigned long long)nC);
    if (nel) atomicAdd(M.counts + 1, nel);
    if (nex) atomicAdd(M.counts + 2, nex);
    if (niz) atomicAdd(M.counts + 3, niz);
}

}  // namespace

void launch_mcc_fp32(const MccParams& M, const DSpecies& el, Secondary* stage, int block, cudaStream_t s) {
    mcc_fp32_kernel<<<(M.n_cells + block - 1) / block, block, 0, s>>>(M, el, stage);
}

}  // namespace pgd
