// oracle.cpp -- CPU restatement of the picFoam per-time-step hot path.
//
// TEST INFRASTRUCTURE ONLY (the checker for the CUDA library and the timed
// CPU baseline); nothing in the product links it.  Parity against picFoam
// binaries is unpinned: picFoam needs OpenFOAM-9 to build and ships no test
// vectors, so this restatement is pinned by analytic known-answer tests.
//
// Structure follows the reference: parcels are records kept in insertion
// order (PICParcel in an IDLList), each time step runs PICCloud::evolve
// (PICMCCFVM/clouds/Templates/PICCloud/PICCloud.C:1426-1471) as a sequence
// of whole-cloud passes.  File:line citations below are relative to the
// picFoam source tree (PICMCCFVM/ abbreviated as PIC/, PIC/submodels as SM/).
//
// The OpenFOAM-9 pieces picFoam calls into (barycentric tet tracking,
// interpolationCellPoint, fvm::laplacian + PCG, fvc::grad) are restated from
// their published descriptions, not from OpenFOAM source.
//
// Floating point: compiled with -ffp-contract=off; every expression below is
// written in the evaluation order the CUDA kernels use so that the FP64 form
// agrees bit for bit.

#include "oracle.h"
#include "collisions.hpp"
#include "picgpu_init.h"
#include "omesh.hpp"
#include "oboundary.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

using HexMesh = om::Mesh;
using om::PatchTriangles;
using om::patch_triangles;

// CODATA constants (values used throughout the project).
constexpr double kC = 299792458.0;
constexpr double kPi = 3.14159265358979323846;
constexpr double kMu0 = 4.0 * kPi * 1e-7;
const double kEps0 = 1.0 / (kMu0 * kC * kC);

struct V3 { double x, y, z; };
inline V3 v3(double a, double b, double c) { return V3{a, b, c}; }
inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 smul(double s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 sdiv(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
inline double dotv(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double magv(V3 a) { return std::sqrt(dotv(a, a)); }
inline V3 crossv(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

struct Parcel {
    int cell = 0;
    int tet = 0;         // local tet 0..11
    double y[4] = {1, 0, 0, 0};
    V3 U{0, 0, 0};
    bool alive = true;
    // PICParcel nParticle_ (negative: the species weight, as addNewParcel
    // sets it, PICCloud.C:707-723) and chargeModifier_ (PICParcel.H:182-195)
    double nw = -1.0;
    int zq = 1;
};

// Deterministic reduction: the fixed order the CUDA kernels reduce in (256
// threads, kItems = 4 strided items per thread; lane l adds threads l, l+32,
// ..., l+224 in turn, then a 32-lane xor-tree).
double tree_block(const double* acc /*256*/) {
    double a[32];
    for (int l = 0; l < 32; ++l) {
        a[l] = acc[l];
        for (int j = 1; j < 8; ++j) a[l] = a[l] + acc[l + 32 * j];
    }
    for (int off = 16; off >= 1; off >>= 1)
        for (int l = 0; l < off; ++l) a[l] = a[l] + a[l + off];
    return a[0];
}

// det_sum with the GPU's fused accumulation s = fma(a_i, b_i, s).
double det_dot(long n, const double* a, const double* b) {
    const int items = 4;
    const long chunk = 256 * items;
    const long nb = (n + chunk - 1) / chunk;
    std::vector<double> part(std::max<long>(nb, 1), 0.0);
    double acc[256];
    for (long blk = 0; blk < nb; ++blk) {
        for (int t = 0; t < 256; ++t) {
            double s = 0.0;
            for (int j = 0; j < items; ++j) {
                const long i = blk * chunk + long(j) * 256 + t;
                if (i < n) s = std::fma(a[i], b[i], s);
            }
            acc[t] = s;
        }
        part[blk] = tree_block(acc);
    }
    for (int t = 0; t < 256; ++t) {
        double s = 0.0;
        for (long i = t; i < nb; i += 256) s = s + part[i];
        acc[t] = s;
    }
    return tree_block(acc);
}

template <class F>
double det_sum(long n, F term) {
    const int items = 4;
    const long chunk = 256 * items;
    const long nb = (n + chunk - 1) / chunk;
    std::vector<double> part(std::max<long>(nb, 1), 0.0);
    double acc[256];
    for (long b = 0; b < nb; ++b) {
        for (int t = 0; t < 256; ++t) {
            double s = 0.0;
            for (int j = 0; j < items; ++j) {
                const long i = b * chunk + long(j) * 256 + t;
                if (i < n) s = s + term(i);
            }
            acc[t] = s;
        }
        part[b] = tree_block(acc);
    }
    for (int t = 0; t < 256; ++t) {
        double s = 0.0;
        for (long i = t; i < nb; i += 256) s = s + part[i];
        acc[t] = s;
    }
    return tree_block(acc);
}

struct Oracle {
    picgpu_config cfg{};
    HexMesh m;
    int nthreads = 1;
    int precond = ORACLE_PRECOND_JACOBI;
    std::string err;
    std::vector<std::vector<Parcel>> cloud;  // per species, insertion order
    // fields
    std::vector<double> phi, rho, E, Ept, Eb;
    std::vector<double> ccData, vtxData;     // VolumeWeighting accumulators
    std::vector<long long> ccFix, vtxFix;    // fixed-point accumulators
    double fixScale = 1.0;
    std::vector<double> Mdiag, Moff, dinv;   // SPD Poisson operator -laplacian
    std::vector<double> sigma, gradBC, Qconv; // per patch floating state
    std::vector<double> rlcK;                 // per patch RLCBoundary a0 epsilon A
    // circuit model (circuitRLC / IdealVoltageSource / IdealCurrentSource)
    ob::RlcCoeffs rlc;
    double circuitI = 0.0;
    std::vector<int> cathodeFaces;
    ob::CircuitState circuit{};
    bool rotation = false;
    std::vector<double> Bcell;   // per-cell magnetic field (3 per cell); empty: the uniform cfg.B
    // parcels of the step's cell occupancy per species (the slots before the
    // collision secondaries; neutral parcels deleted on the way come off)
    std::vector<long> occ_n;
    // Perez ionisation tables per species (inactive: limit < 0)
    struct PerezTab {
        int atomic = 0, limit = -1;
        std::vector<double> cs, te, le;   // [Zstar][100]: cross section, transferred and lost energy
    };
    std::vector<PerezTab> perez;
    double move_seconds = 0;
    long long step_index = 0;
    // collision state
    std::vector<double> svmax, remainder;
    std::vector<double> psvmax, premainder;  // electron - neutral parcels
    std::vector<double> ipsvmax, ipremainder;  // ion - neutral parcels
    std::vector<double> isvmax, iremainder;  // ion-neutral
    int last_pcg_iter = 0;
    double last_res_l2 = 0, last_res_of = 0;
    picgpu_step_stats acc{};
    ocoll::Tables xs, ixs;
    // SimpleInjection boundary models
    struct Injector {
        picgpu_injection cfg{};
        double remainder[PICGPU_MAX_SPECIES] = {};
        PatchTriangles tri;
    };
    std::vector<Injector> injectors;
    // FreeStream boundary models
    struct FreeStream {
        picgpu_freestream cfg{};
        ob::FreeStreamFaces F;
        std::vector<double> acc;   // n_faces * n_species
    };
    std::vector<FreeStream> freestreams;
    // EmissionModels
    struct Emitter {
        picgpu_emission cfg{};
        PatchTriangles tri;
        double j = 0.0, remainder = 0.0;
        std::vector<int> faces;
    };
    std::vector<Emitter> emitters;
    // BinaryCollisionModel state per cell
    std::vector<double> bsmax, brem, bbgrem;
};

// ------------------------------------------------------------ pushers -----
// E at the particle: FieldWeigthing (SM/FieldWeigthing).
// VolumeWeighting (VolumeWeightingFW.C:60-67 -> interpolationCellPoint):
//   E = y0 E_cell + y1 E_pt[tri0] + y2 E_pt[tri1] + y3 E_pt[tri2].
// CellAverage (CellAverageFW.C:58-65): E = E_cell.
// A parcel's nParticle and charge (species charge x chargeModifier,
// PICCloud.C:368).
double pweight(const Oracle& o, const Parcel& p, int s) { return p.nw < 0.0 ? o.cfg.species[s].weight : p.nw; }
double pcharge(const Oracle& o, const Parcel& p, int s) { return o.cfg.species[s].charge * double(p.zq); }

V3 field_at(const Oracle& o, const Parcel& p) {
    const HexMesh& m = o.m;
    const double* Ec = &o.E[3 * size_t(p.cell)];
    if (o.cfg.field_weighting == PICGPU_WEIGHTING_CELL_AVERAGE) return v3(Ec[0], Ec[1], Ec[2]);
    const int* cp = &m.cell_pt[8 * size_t(p.cell)];
    const double* e1 = &o.Ept[3 * size_t(cp[m.tt.tri[p.tet][0]])];
    const double* e2 = &o.Ept[3 * size_t(cp[m.tt.tri[p.tet][1]])];
    const double* e3 = &o.Ept[3 * size_t(cp[m.tt.tri[p.tet][2]])];
    double r[3];
    for (int a = 0; a < 3; ++a)
        r[a] = Ec[a] * p.y[0] + e1[a] * p.y[1] + e2[a] * p.y[2] + e3[a] * p.y[3];
    return v3(r[0], r[1], r[2]);
}

// The magnetic field of a parcel's cell: the per-cell field when one was
// set, else the uniform one.
V3 cell_B(const Oracle& o, int cell) {
    if (o.Bcell.empty()) return v3(o.cfg.B[0], o.cfg.B[1], o.cfg.B[2]);
    return v3(o.Bcell[3 * size_t(cell)], o.Bcell[3 * size_t(cell) + 1], o.Bcell[3 * size_t(cell) + 2]);
}

// BorisPusher::updateVelocity (SM/ParticlePusher/BorisPusher/BorisPusher.C:69-112)
void push_boris(const Oracle& o, Parcel& p, double q, double mass, double trackTime) {
    const V3 E = field_at(o, p);
    const V3 B = cell_B(o, p.cell);  // B[celli] (BorisPusher.C:100)
    const double dt2 = 0.5 * trackTime;
    const double mU = magv(p.U) / kC;
    V3 rU = sdiv(p.U, std::sqrt(1.0 - mU * mU));
    const V3 oldrU = rU;
    const double qdm = q * dt2 / mass;
    const V3 rUsm = smul(qdm, E);
    rU = add(rU, rUsm);
    if (o.rotation) {
        const double a0 = magv(oldrU) / kC, a1 = magv(rU) / kC;
        const double lF = (std::sqrt(1.0 + a0 * a0) + std::sqrt(1.0 + a1 * a1)) / 2.0;
        const V3 t = sdiv(smul(qdm, B), lF);
        const V3 Udash = add(rU, crossv(rU, t));
        const double den = 1.0 + dotv(t, t);
        const V3 s = sdiv(smul(2.0, t), den);
        rU = add(rU, crossv(Udash, s));
    }
    rU = add(rU, rUsm);
    const double mr = magv(rU) / kC;
    p.U = sdiv(rU, std::sqrt(1.0 + mr * mr));
}

// BorisNRPusher::updateVelocity (SM/ParticlePusher/BorisNRPusher/BorisNRPusher.C:69-99)
void push_boris_nr(const Oracle& o, Parcel& p, double q, double mass, double trackTime) {
    const V3 E = field_at(o, p);
    const V3 B = cell_B(o, p.cell);
    const double dt2 = 0.5 * trackTime;
    const double alpha = q * dt2 / mass;
    V3 U = add(p.U, smul(alpha, E));
    if (o.rotation) {
        const V3 t = smul(alpha, B);
        const V3 Udash = add(U, crossv(U, t));
        const double den = 1.0 + dotv(t, t);
        U = add(U, crossv(Udash, sdiv(smul(2.0, t), den)));
    }
    p.U = add(U, smul(alpha, E));
}

// VayPusher::updateVelocity (SM/ParticlePusher/VayPusher/VayPusher.C:54-100);
// the rotation term uses the velocity v, not u (VayPusher.C:81).
void push_vay(const Oracle& o, Parcel& p, double q, double mass, double trackTime) {
    const V3 E = field_at(o, p);
    const V3 B = cell_B(o, p.cell);
    const double dt2 = 0.5 * trackTime;
    const double mU = magv(p.U) / kC;
    const double lF = 1.0 / std::sqrt(1.0 - mU * mU);
    V3 rU = smul(lF, p.U);
    V3 Ud = add(rU, smul(q * trackTime / mass, E));
    V3 T = smul(q * dt2 / mass, B);
    Ud = add(Ud, crossv(p.U, T));
    const double mUd = magv(Ud) / kC;
    double alpha = 1.0 + mUd * mUd;
    const double T2 = dotv(T, T);
    double s = alpha - T2;
    const double udt = dotv(Ud, T) / kC;
    const double us2 = udt * udt;
    alpha = 1.0 / std::sqrt(0.5 * (s + std::sqrt(s * s + 4.0 * (T2 + us2))));
    T = smul(alpha, T);
    s = 1.0 / (1.0 + dotv(T, T));
    alpha = dotv(Ud, T);
    rU = smul(s, add(add(Ud, smul(alpha, T)), crossv(Ud, T)));
    const double mr = magv(rU) / kC;
    p.U = sdiv(rU, std::sqrt(1.0 + mr * mr));
}

// HigueraCaryPusher::updateVelocity (SM/ParticlePusher/HigueraCary/HigueraCary.C:69-115)
void push_hc(const Oracle& o, Parcel& p, double q, double mass, double trackTime) {
    const V3 E = field_at(o, p);
    const V3 B = cell_B(o, p.cell);
    const double dt2 = 0.5 * trackTime;
    const double mU = magv(p.U) / kC;
    V3 rU = sdiv(p.U, std::sqrt(1.0 - mU * mU));
    const double qdm = q * dt2 / mass;
    const V3 rUsm = smul(qdm, E);
    rU = add(rU, rUsm);
    if (o.rotation) {
        const double mr0 = magv(rU) / kC;
        const double gfm2 = 1.0 + mr0 * mr0;
        V3 t = smul(qdm, B);
        const double beta2 = dotv(t, t);
        const double gb = gfm2 - beta2;
        const double tr = dotv(t, rU);
        const double iG = 1.0 / std::sqrt(0.5 * (gb + std::sqrt(gb * gb + 4.0 * (beta2 + tr * tr))));
        t = smul(iG, t);
        const V3 Udash = add(rU, crossv(rU, t));
        const double den = 1.0 + dotv(t, t);
        rU = add(rU, crossv(Udash, sdiv(smul(2.0, t), den)));
    }
    rU = add(rU, rUsm);
    const double mr = magv(rU) / kC;
    p.U = sdiv(rU, std::sqrt(1.0 + mr * mr));
}

// ParticlePusher::updateVelocity dispatch (ParticlePusher.H:131-134)
void push(const Oracle& o, Parcel& p, int species, double trackTime) {
    const double q = pcharge(o, p, species), mass = o.cfg.species[species].mass;
    switch (o.cfg.pusher) {
        case PICGPU_PUSHER_BORIS: push_boris(o, p, q, mass, trackTime); break;
        case PICGPU_PUSHER_BORIS_NR: push_boris_nr(o, p, q, mass, trackTime); break;
        case PICGPU_PUSHER_VAY: push_vay(o, p, q, mass, trackTime); break;
        case PICGPU_PUSHER_HIGUERA_CARY: push_hc(o, p, q, mass, trackTime); break;
        default: break;  // "none" (NoPush)
    }
}

// ------------------------------------------------------------ tracking ----
struct TrackData {
    bool keep = true;
    bool requireResync = false;
    long long tet_steps = 0, faces = 0, walls = 0;
    bool capped = false;
    bool superluminal = false;
    double* qconv = nullptr;   // floating-patch charge accumulator of this thread
};

V3 position_of(const Oracle& o, const Parcel& p) {
    double x[3];
    om::position(o.m, 12LL * p.cell + p.tet, &p.y[1], x);
    return v3(x[0], x[1], x[2]);
}

// One tet step of barycentric tracking (the OpenFOAM-5+ algorithm: map the
// displacement into barycentric space, take the first coordinate to reach
// zero, clamp round-off, renormalise).  Returns the hit tet face (-1: the
// displacement is used up) and the fraction lambda of the displacement moved.
int tet_step(const Oracle& o, Parcel& p, const double* dx, double* lambda) {
    const double* inv = &o.m.cls_tetinv[(size_t(o.m.cell_class[p.cell]) * 12 + p.tet) * 9];
    double dy[4];
    dy[1] = inv[0] * dx[0] + inv[1] * dx[1] + inv[2] * dx[2];
    dy[2] = inv[3] * dx[0] + inv[4] * dx[1] + inv[5] * dx[2];
    dy[3] = inv[6] * dx[0] + inv[7] * dx[1] + inv[8] * dx[2];
    dy[0] = -(dy[1] + dy[2] + dy[3]);
    const double S = std::fabs(dy[0]) + std::fabs(dy[1]) + std::fabs(dy[2]) + std::fabs(dy[3]);
    const double thr = -1e-12 * S;
    double lam = 1.0;
    int hit = -1;
    for (int i = 0; i < 4; ++i) {
        if (dy[i] < thr) {
            const double l = -p.y[i] / dy[i];
            if (l < lam) { lam = l; hit = i; }
        }
    }
    double y[4];
    for (int i = 0; i < 4; ++i) y[i] = p.y[i] + lam * dy[i];
    if (hit >= 0) y[hit] = 0.0;
    for (int i = 0; i < 4; ++i) y[i] = std::fmax(y[i], 0.0);
    const double r = 1.0 / (y[0] + y[1] + y[2] + y[3]);
    for (int i = 0; i < 4; ++i) p.y[i] = y[i] * r;
    *lambda = lam;
    return hit;
}

// PICParcel::syncVelocityAtBoundary (PIC/parcels/Templates/PICParcel/PICParcel.C:220-227)
void sync_velocity(const Oracle& o, Parcel& p, int species, double fraction) {
    if (o.cfg.sync_velocity_at_boundary && pcharge(o, p, species) != 0.0)
        push(o, p, species, fraction * o.cfg.dt);
}

// PICParcel::hitPatch (PICParcel.C:153-184) with the patch models in scope:
// NoInflow (SM/BoundaryModel/NoInflow/NoInflow.C:56-61) and FloatingPotential
// (SM/BoundaryModel/FloatingPotential/FloatingPotential.C:119-127) delete the
// parcel; a wall without a model reflects (SpecularReflection.C:53-67) and
// asks for a velocity resync.
void hit_patch(Oracle& o, Parcel& p, int species, int patch, double sf, TrackData& td) {
    const picgpu_patch& P = o.m.patches[patch].p;
    if (P.kind == PICGPU_PATCH_ABSORB) {
        td.keep = false;
        return;
    }
    // a circuit electrode (circuitRLC.C:268-288) deletes charged parcels and
    // reflects neutral ones
    const bool charged = o.cfg.species[species].charge != 0.0;
    if (P.kind == PICGPU_PATCH_FLOATING || (P.kind == PICGPU_PATCH_CIRCUIT && charged)) {
        td.keep = false;
        td.qconv[patch] += pweight(o, p, species) * pcharge(o, p, species);
        return;
    }
    const int f = p.tet / 2;
    const double* n = &o.m.cls_fnormal[size_t(o.m.cell_class[p.cell]) * 18 + 3 * f];
    if (P.kind == PICGPU_PATCH_WALL || P.kind == PICGPU_PATCH_CIRCUIT) {
        sync_velocity(o, p, species, sf - 0.5);
        td.walls++;
        td.requireResync = true;
    }
    // specular reflection (also used for a stray hit of an empty patch)
    const double Un = p.U.x * n[0] + p.U.y * n[1] + p.U.z * n[2];
    if (Un > 0.0) {
        const double t = 2.0 * Un;
        p.U = v3(p.U.x - t * n[0], p.U.y - t * n[1], p.U.z - t * n[2]);
    }
}

// trackToAndHitFace: tet steps inside the cell until the displacement is used
// up or a cell face is reached; then cross into the neighbour (internal or
// cyclic face) or interact with the patch.
void track_to_and_hit_face(Oracle& o, Parcel& p, int species, const double* disp, double f,
                           double& sf, TrackData& td, int& budget) {
    const HexMesh& m = o.m;
    double rem = 1.0;
    for (;;) {
        if (--budget < 0) { td.capped = true; sf = 1.0; return; }
        double dx[3] = {rem * disp[0], rem * disp[1], rem * disp[2]};
        double lam;
        const int hit = tet_step(o, p, dx, &lam);
        td.tet_steps++;
        if (hit < 0) { sf = 1.0; return; }
        sf += (f * rem) * lam;
        if (hit > 0) {
            const int nt = m.tt.inner_next[p.tet][hit];
            double y[4];
            for (int j = 0; j < 4; ++j) {
                const int s = m.tt.inner_src[p.tet][hit][j];
                y[j] = s < 0 ? 0.0 : p.y[s];
            }
            std::memcpy(p.y, y, sizeof y);
            p.tet = nt;
            rem = rem * (1.0 - lam);
            continue;
        }
        // cell face
        const int face = p.tet / 2;
        const int nb = m.nbr[6 * size_t(p.cell) + face];
        td.faces++;
        if (nb >= 0) {
            const int nt = m.tt.cross_next[p.tet];
            double y[4];
            y[0] = 0.0;
            for (int j = 1; j < 4; ++j) y[j] = p.y[m.tt.cross_src[p.tet][j]];
            std::memcpy(p.y, y, sizeof y);
            p.tet = nt;
            p.cell = nb;
            return;
        }
        hit_patch(o, p, species, -nb - 1, sf, td);
        return;
    }
}

// PICParcel::move + moveForward (PICParcel.C:38-144)
void move_parcel(Oracle& o, Parcel& p, int species, TrackData& td) {
    const picgpu_species& sp = o.cfg.species[species];
    if (!sp.solve_movement) return;
    // the particle store holds three barycentric coordinates; the centre one
    // is re-derived at the start of every step
    p.y[0] = 1.0 - p.y[1] - p.y[2] - p.y[3];
    if (pcharge(o, p, species) != 0.0) push(o, p, species, o.cfg.dt);
    if (!(magv(p.U) < kC)) { td.keep = false; td.superluminal = true; return; }
    const HexMesh& m = o.m;
    double sf = 0.0;
    int resync = 0;
    int budget = o.cfg.track_max_steps > 0 ? o.cfg.track_max_steps : 4096;
    const double dt = o.cfg.dt;
    while (td.keep && sf < 1.0) {
        // Utracking constrained to the solution directions and the deviation
        // from the mesh centre in the empty ones (PICParcel.C:119-126)
        double Ut[3] = {p.U.x, p.U.y, p.U.z};
        double dev[3] = {0, 0, 0};
        bool reduced = false;
        for (int a = 0; a < 3; ++a) if (m.empty[a]) { Ut[a] = 0.0; reduced = true; }
        if (reduced) {
            const V3 x = position_of(o, p);
            const double xa[3] = {x.x, x.y, x.z};
            for (int a = 0; a < 3; ++a) if (m.empty[a]) dev[a] = xa[a] - m.mesh_centre[a];
        }
        const double f = 1.0 - sf;
        const double fdt = f * dt;
        const double disp[3] = {fdt * Ut[0] - dev[0], fdt * Ut[1] - dev[1], fdt * Ut[2] - dev[2]};
        td.requireResync = false;
        track_to_and_hit_face(o, p, species, disp, f, sf, td, budget);
        if (td.capped) return;
        if (td.requireResync && td.keep) {
            resync++;
            if (resync > 1) { td.requireResync = false; continue; }
            sync_velocity(o, p, species, 0.5 - sf);
            td.requireResync = false;
        }
    }
}

// ----------------------------------------------------- charge and fields --
void reset_charge(Oracle& o) {
    std::fill(o.ccData.begin(), o.ccData.end(), 0.0);
    std::fill(o.vtxData.begin(), o.vtxData.end(), 0.0);
    std::fill(o.ccFix.begin(), o.ccFix.end(), 0LL);
    std::fill(o.vtxFix.begin(), o.vtxFix.end(), 0LL);
}

// ChargeDistribution::add: VolumeWeighting (VolumeWeighting.C:105-124),
// CellAverage (CellAverage.C:53-60).
void deposit(Oracle& o, const Parcel& p, int species) {
    const double value = pcharge(o, p, species) * pweight(o, p, species);
    if (value == 0.0) return;
    const HexMesh& m = o.m;
    const bool fixed = o.cfg.deposit_mode == PICGPU_DEPOSIT_FIXED_POINT;
    if (o.cfg.charge_distribution == PICGPU_WEIGHTING_CELL_AVERAGE) {
        if (fixed) o.ccFix[p.cell] += std::llrint(value * o.fixScale);
        else o.ccData[p.cell] += value;
        return;
    }
    const int* cp = &m.cell_pt[8 * size_t(p.cell)];
    if (fixed) {
        o.ccFix[p.cell] += std::llrint((p.y[0] * value) * o.fixScale);
        for (int i = 0; i < 3; ++i)
            o.vtxFix[cp[m.tt.tri[p.tet][i]]] += std::llrint((p.y[i + 1] * value) * o.fixScale);
    } else {
        o.ccData[p.cell] += p.y[0] * value;
        for (int i = 0; i < 3; ++i) o.vtxData[cp[m.tt.tri[p.tet][i]]] += p.y[i + 1] * value;
    }
}

// ChargeDistribution::update (VolumeWeighting.C:138-164, CellAverage.C:63-68)
// and the spaceCharge addition (PICCloud.C:687-690).
void update_charge(Oracle& o) {
    const HexMesh& m = o.m;
    const bool fixed = o.cfg.deposit_mode == PICGPU_DEPOSIT_FIXED_POINT;
    for (int c = 0; c < m.n_cells; ++c) {
        const double V = m.vol[c];
        const double ccv = fixed ? double(o.ccFix[c]) / o.fixScale : o.ccData[c];
        double r = 0.0;
        if (o.cfg.charge_distribution == PICGPU_WEIGHTING_CELL_AVERAGE) {
            r = ccv / V;
        } else {
            r = r + ccv / V;
            for (int q = 0; q < 8; ++q) {
                const int pt = m.cell_pt[8 * size_t(c) + q];
                const double vv = fixed ? double(o.vtxFix[pt]) / o.fixScale : o.vtxData[pt];
                r = r + (m.vw_weight[8 * size_t(c) + q] * vv) / V;
            }
        }
        o.rho[c] = r + o.cfg.space_charge;
    }
}

// FloatingPotential::preUpdate_Boundary (FloatingPotential.C:89-100)
void floating_pre_update(Oracle& o) {
    for (size_t pa = 0; pa < o.m.patches.size(); ++pa) {
        if (o.m.patches[pa].p.kind != PICGPU_PATCH_FLOATING) continue;
        o.sigma[pa] += o.Qconv[pa] / o.m.patches[pa].area;
        o.gradBC[pa] = o.sigma[pa] / kEps0;
        o.Qconv[pa] = 0.0;
    }
}

// Circuit models around the field solve (PICCloud.C:1457-1464), with the
// source and averaging factor of the step and the cathode-face sum in the
// device's lane order.
double circuit_src(const Oracle& o) {
    if (o.cfg.circuit.model != PICGPU_CIRCUIT_RLC) return 0.0;
    return ob::circuit_source(o.cfg.circuit, double(o.step_index + 1) * o.cfg.dt);
}

void circuit_pre_update(Oracle& o) {
    const picgpu_circuit& cc = o.cfg.circuit;
    if (cc.model == PICGPU_CIRCUIT_NONE) return;
    ob::circuit_pre_update(cc.model, cc.cathode_patch, o.rlc.a, o.m.patches[cc.cathode_patch].area, o.circuitI,
                           o.cfg.dt, kEps0, circuit_src(o), o.Qconv.data(), o.gradBC.data(), o.circuit);
}

void circuit_post_update(Oracle& o) {
    const picgpu_circuit& cc = o.cfg.circuit;
    if (cc.model == PICGPU_CIRCUIT_NONE) return;
    const HexMesh& m = o.m;
    const int nf = int(o.cathodeFaces.size());
    double sum = 0.0;
    if (cc.model == PICGPU_CIRCUIT_RLC) {
        sum = ob::lane_sum(nf, [&](int i) {
            const om::BFace& B = m.bfaces[o.cathodeFaces[i]];
            return ob::face_value(ob::kRuleRlc, 0.0, 0.0, o.rlc.k, B.delta, o.phi[B.cell]);
        });
    } else if (cc.model == PICGPU_CIRCUIT_IDEAL_CURRENT) {
        sum = ob::lane_sum(nf, [&](int i) {
            const om::BFace& B = m.bfaces[o.cathodeFaces[i]];
            return B.area * o.phi[B.cell];
        });
    }
    const double t = double(o.step_index + 1) * o.cfg.dt;
    ob::circuit_post_update(cc.model, cc.anode_patch, cc.cathode_patch, nf, o.rlc.a,
                            m.patches[cc.cathode_patch].area, o.cfg.dt, circuit_src(o), o.cfg.dt / t, sum,
                            o.Qconv.data(), o.circuit);
}

// Right-hand side of -laplacian(phi) = rho/eps0 in integral form (the
// fvm::laplacian(phiE) + rhoCharge/epsilon0 system of ElectroStaticSolver.C:61-64):
// Dirichlet faces add a |S|/delta phi_b, circuitBoundary faces add |S| g
// (circuitBoundaryFvPatchField.C:157-175).
void assemble_rhs(const Oracle& o, const double* rho, std::vector<double>& b) {
    const HexMesh& m = o.m;
    b.resize(m.n_cells);
    for (int c = 0; c < m.n_cells; ++c) {
        double t = (rho[c] / kEps0) * m.vol[c];
        for (int f = 0; f < 6; ++f) {
            const int bf = m.cell_bface[6 * size_t(c) + f];
            if (bf < 0) continue;
            const om::BFace& B = m.bfaces[bf];
            const picgpu_patch& P = m.patches[B.patch].p;
            const int rule = ob::face_rule(P.kind, P.phi_bc);
            if (rule != ob::kRuleNone)
                t = t + ob::face_rhs(rule, P.phi, o.gradBC[B.patch], o.rlcK[B.patch], B.area, B.delta);
        }
        b[c] = t;
    }
    if (!m.has_dirichlet) {
        // singular (fully periodic / Neumann) system: project out the mean
        const double mean = det_sum(m.n_cells, [&](long i) { return b[i]; }) / double(m.n_cells);
        for (int c = 0; c < m.n_cells; ++c) b[c] = b[c] - mean;
    }
}

void apply_M(const Oracle& o, const std::vector<double>& x, std::vector<double>& y) {
    const HexMesh& m = o.m;
    for (int c = 0; c < m.n_cells; ++c) {
        double s = o.Mdiag[c] * x[c];
        for (int f = 0; f < 6; ++f) {
            const int nb = m.nbr[6 * size_t(c) + f];
            if (nb >= 0) s = std::fma(o.Moff[6 * size_t(c) + f], x[nb], s);
        }
        y[c] = s;
    }
}

// OpenFOAM-normalised residual: sum|b - Ax| / (sum(|Ax - A xRef| + |b - A xRef|) + 1e-20)
// with xRef the mean of x.
double of_residual(const Oracle& o, const std::vector<double>& b, const std::vector<double>& x) {
    const HexMesh& m = o.m;
    std::vector<double> Ax(m.n_cells);
    apply_M(o, x, Ax);
    double mean = 0;
    for (int c = 0; c < m.n_cells; ++c) mean += x[c];
    mean /= m.n_cells;
    double num = 0, den = 0;
    for (int c = 0; c < m.n_cells; ++c) {
        double rowsum = o.Mdiag[c];
        for (int f = 0; f < 6; ++f)
            if (m.nbr[6 * size_t(c) + f] >= 0) rowsum += o.Moff[6 * size_t(c) + f];
        const double Axr = rowsum * mean;
        num += std::fabs(b[c] - Ax[c]);
        den += std::fabs(Ax[c] - Axr) + std::fabs(b[c] - Axr);
    }
    return num / (den + 1e-20);
}

// PCG with the Jacobi preconditioner, reductions in the GPU's fixed order.
// Jacobi-preconditioned CG in the Chronopoulos-Gear form the GPU runs (one
// reduction point per iteration), with the GPU's operation order, fused
// multiply-adds and reduction tree, so both produce the same bits.  The iterates equal those
// of the textbook PCG of lduMatrix in exact arithmetic.
int pcg_jacobi(Oracle& o, const std::vector<double>& b, std::vector<double>& x, double tol,
               int maxit, double* res) {
    const long n = o.m.n_cells;
    std::vector<double> r(n), u(n), w(n), p(n), s(n);
    apply_M(o, x, w);
    for (long i = 0; i < n; ++i) {
        r[i] = b[i] - w[i];
        u[i] = o.dinv[i] * r[i];
    }
    double g = det_dot(n, r.data(), u.data());
    double rr = det_dot(n, r.data(), r.data());
    const double bb = det_dot(n, b.data(), b.data());
    apply_M(o, u, w);
    double d = det_dot(n, w.data(), u.data());
    const double lim = (tol * tol) * bb;
    double alpha = g / d, beta = 0.0;
    int it = 0;
    if (!(rr <= lim)) {
        for (int k = 0;;) {
            for (long i = 0; i < n; ++i) {
                if (k == 0) {
                    p[i] = u[i];
                    s[i] = w[i];
                } else {
                    p[i] = std::fma(beta, p[i], u[i]);
                    s[i] = std::fma(beta, s[i], w[i]);
                }
                x[i] = std::fma(alpha, p[i], x[i]);
                r[i] = std::fma(-alpha, s[i], r[i]);
                u[i] = o.dinv[i] * r[i];
            }
            const double gn = det_dot(n, r.data(), u.data());
            rr = det_dot(n, r.data(), r.data());
            apply_M(o, u, w);
            d = det_dot(n, w.data(), u.data());
            ++k;
            if (rr <= lim) { it = k; break; }
            if (k >= maxit) { it = -maxit; break; }
            beta = gn / g;
            alpha = gn / (d - beta * gn / alpha);
            g = gn;
        }
    }
    *res = bb > 0 ? std::sqrt(rr / bb) : 0.0;
    return it;
}

// OpenFOAM PCG with the DIC preconditioner (tutorial system/fvSolution) on
// the internal faces in upper-triangular order; coupled cyclic faces are
// interfaces the preconditioner leaves out.
int pcg_dic(Oracle& o, const std::vector<double>& b, std::vector<double>& x, double tol,
            int maxit, double* res) {
    const HexMesh& m = o.m;
    const long n = m.n_cells;
    struct F { int l, u; double a; };
    std::vector<F> faces;
    for (int c = 0; c < n; ++c)
        for (int f = 1; f < 6; f += 2) {  // + faces: owner c, neighbour higher
            const int nb = m.nbr[6 * size_t(c) + f];
            if (nb > c && !(m.cell_ijk[3 * size_t(c) + f / 2] == m.n[f / 2] - 1))
                faces.push_back({c, nb, o.Moff[6 * size_t(c) + f]});
        }
    std::sort(faces.begin(), faces.end(), [](const F& a, const F& b2) {
        return a.l != b2.l ? a.l < b2.l : a.u < b2.u;
    });
    std::vector<double> rD(o.Mdiag);
    for (const F& f : faces) rD[f.u] -= f.a * f.a / rD[f.l];
    for (long i = 0; i < n; ++i) rD[i] = 1.0 / rD[i];
    auto prec = [&](const std::vector<double>& r, std::vector<double>& w) {
        for (long i = 0; i < n; ++i) w[i] = rD[i] * r[i];
        for (const F& f : faces) w[f.u] -= rD[f.u] * f.a * w[f.l];
        for (auto it = faces.rbegin(); it != faces.rend(); ++it) w[it->l] -= rD[it->l] * it->a * w[it->u];
    };
    std::vector<double> r(n), z(n), p(n), q(n);
    apply_M(o, x, q);
    double rr = 0, bb = 0;
    for (long i = 0; i < n; ++i) { r[i] = b[i] - q[i]; rr += r[i] * r[i]; bb += b[i] * b[i]; }
    const double lim = tol * tol * bb;
    int it = 0;
    if (!(rr <= lim)) {
        prec(r, z);
        double rz = 0;
        for (long i = 0; i < n; ++i) rz += r[i] * z[i];
        p = z;
        for (it = 1; it <= maxit; ++it) {
            apply_M(o, p, q);
            double pq = 0;
            for (long i = 0; i < n; ++i) pq += p[i] * q[i];
            const double alpha = rz / pq;
            rr = 0;
            for (long i = 0; i < n; ++i) {
                x[i] += alpha * p[i];
                r[i] -= alpha * q[i];
                rr += r[i] * r[i];
            }
            if (rr <= lim) break;
            prec(r, z);
            double rzn = 0;
            for (long i = 0; i < n; ++i) rzn += r[i] * z[i];
            const double beta = rzn / rz;
            rz = rzn;
            for (long i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        }
        if (it > maxit) it = -maxit;
    }
    *res = bb > 0 ? std::sqrt(rr / bb) : 0.0;
    return it;
}

// E = -fvc::grad(phi) (Gauss linear) with corrected boundary values, then the
// point field (FieldWeigthing::update, VolumeWeightingFW.C:70-75).
void compute_E(Oracle& o) {
    const HexMesh& m = o.m;
    for (int c = 0; c < m.n_cells; ++c) {
        const int cl = m.cell_class[c];
        double g[3] = {0, 0, 0};
        for (int f = 0; f < 6; ++f) {
            const int nb = m.nbr[6 * size_t(c) + f];
            double pf;
            if (nb >= 0) {
                const double w = m.ip_weight[6 * size_t(c) + f];
                pf = w * o.phi[c] + (1.0 - w) * o.phi[nb];
            } else {
                const int bf = m.cell_bface[6 * size_t(c) + f];
                if (bf < 0) continue;  // empty
                const om::BFace& B = m.bfaces[bf];
                const picgpu_patch& P = m.patches[B.patch].p;
                pf = ob::face_value(ob::face_rule(P.kind, P.phi_bc), P.phi, o.gradBC[B.patch], o.rlcK[B.patch],
                                    B.delta, o.phi[c]);
            }
            const double area = m.cls_farea[size_t(cl) * 6 + f];
            const double* n = &m.cls_fnormal[size_t(cl) * 18 + 3 * f];
            for (int a = 0; a < 3; ++a) g[a] = g[a] + pf * (n[a] * area);
        }
        for (int a = 0; a < 3; ++a) o.E[3 * size_t(c) + a] = -(g[a] / m.vol[c]);
    }
    for (size_t b = 0; b < m.bfaces.size(); ++b) {
        const om::BFace& B = m.bfaces[b];
        const picgpu_patch& P = m.patches[B.patch].p;
        const double* Ec = &o.E[3 * size_t(B.cell)];
        const double sn = ob::face_sn_grad(ob::face_rule(P.kind, P.phi_bc), P.phi, o.gradBC[B.patch],
                                           o.rlcK[B.patch], B.delta, o.phi[B.cell]);
        const double En = Ec[0] * B.normal[0] + Ec[1] * B.normal[1] + Ec[2] * B.normal[2];
        for (int a = 0; a < 3; ++a)
            o.Eb[3 * b + a] = (Ec[a] - En * B.normal[a]) - sn * B.normal[a];
    }
    for (int p = 0; p < m.n_points; ++p) {
        double e[3] = {0, 0, 0};
        for (int k = m.pi_start[p]; k < m.pi_start[p + 1]; ++k) {
            const int s = m.pi_src[k];
            const double* src = s >= 0 ? &o.E[3 * size_t(s)] : &o.Eb[3 * size_t(-s - 1)];
            for (int a = 0; a < 3; ++a) e[a] = e[a] + m.pi_w[k] * src[a];
        }
        for (int a = 0; a < 3; ++a) o.Ept[3 * size_t(p) + a] = e[a];
    }
}

void set_applied_field(Oracle& o) {
    for (int c = 0; c < o.m.n_cells; ++c)
        for (int a = 0; a < 3; ++a) o.E[3 * size_t(c) + a] = o.cfg.E_applied[a];
    for (int p = 0; p < o.m.n_points; ++p)
        for (int a = 0; a < 3; ++a) o.Ept[3 * size_t(p) + a] = o.cfg.E_applied[a];
}

int solve_fields(Oracle& o, picgpu_step_stats* st) {
    if (o.cfg.maxwell_solver != PICGPU_MAXWELL_ELECTROSTATIC) { set_applied_field(o); return 0; }
    std::vector<double> b;
    assemble_rhs(o, o.rho.data(), b);
    double res = 0;
    double r0 = 0, bb = 0;
    for (int i = 0; i < o.m.n_cells; ++i) {
        double ax = o.Mdiag[i] * o.phi[i];
        for (int k = 0; k < 6; ++k) {
            const int j = o.m.nbr[6 * size_t(i) + k];
            if (j >= 0) ax += o.Moff[6 * size_t(i) + k] * o.phi[j];
        }
        r0 += (b[i] - ax) * (b[i] - ax);
        bb += b[i] * b[i];
    }
    const int maxit = o.cfg.pcg_max_iter > 0 ? o.cfg.pcg_max_iter : 10000;
    const double tol = o.cfg.pcg_tol > 0 ? o.cfg.pcg_tol : 1e-10;
    int it = o.precond == ORACLE_PRECOND_DIC ? pcg_dic(o, b, o.phi, tol, maxit, &res)
                                              : pcg_jacobi(o, b, o.phi, tol, maxit, &res);
    o.last_pcg_iter = it < 0 ? -it : it;
    o.last_res_l2 = res;
    o.last_res_of = of_residual(o, b, o.phi);
    if (st) {
        st->pcg_iterations = o.last_pcg_iter;
        st->pcg_iterations_total += o.last_pcg_iter;
        st->pcg_residual_l2 = res;
        st->pcg_residual_of = o.last_res_of;
        st->pcg_residual_initial = bb > 0 ? std::sqrt(r0 / bb) : 0.0;
    }
    compute_E(o);
    return it < 0 ? PICGPU_PCG_NOT_CONVERGED : 0;
}

void calculate_fields(Oracle& o) {
    reset_charge(o);
    for (size_t s = 0; s < o.cloud.size(); ++s)
        for (const Parcel& p : o.cloud[s]) deposit(o, p, int(s));
    update_charge(o);
}

// Cloud::move over all parcels; parcels are independent, so threads take
// contiguous ranges (the oracle's host-thread decomposition mode).
int move_all(Oracle& o, picgpu_step_stats* st) {
    const auto t0 = std::chrono::steady_clock::now();
    int status = 0;
    for (size_t s = 0; s < o.cloud.size(); ++s) {
        auto& cl = o.cloud[s];
        const size_t n = cl.size();
        const int nt = std::max(1, std::min<int>(o.nthreads, int(n / 1024) + 1));
        std::vector<TrackData> tds(nt);
        std::vector<std::vector<double>> qconv(nt, std::vector<double>(o.Qconv.size(), 0.0));
        auto work = [&](int ti) {
            const size_t lo = n * ti / nt, hi = n * (ti + 1) / nt;
            for (size_t i = lo; i < hi; ++i) {
                TrackData td;
                td.qconv = qconv[ti].data();
                move_parcel(o, cl[i], int(s), td);
                cl[i].alive = td.keep && !td.capped && !td.superluminal;
                tds[ti].tet_steps += td.tet_steps;
                tds[ti].faces += td.faces;
                tds[ti].walls += td.walls;
                tds[ti].capped |= td.capped;
                tds[ti].superluminal |= td.superluminal;
            }
        };
        if (nt == 1) {
            work(0);
        } else {
            std::vector<std::thread> th;
            for (int ti = 0; ti < nt; ++ti) th.emplace_back(work, ti);
            for (auto& t : th) t.join();
        }
        // floating-patch charge, summed in thread order
        for (int ti = 0; ti < nt; ++ti)
            for (size_t pa = 0; pa < o.Qconv.size(); ++pa) o.Qconv[pa] += qconv[ti][pa];
        size_t w = 0;
        long long absorbed = 0;
        for (size_t i = 0; i < n; ++i) {
            if (cl[i].alive) cl[w++] = cl[i];
            else absorbed++;
        }
        cl.resize(w);
        for (auto& td : tds) {
            if (td.capped) status = PICGPU_TRACK_LOOP_CAP;
            if (td.superluminal) status = PICGPU_SPEED_OF_LIGHT;
            if (st) {
                st->tet_steps += td.tet_steps;
                st->face_crossings += td.faces;
                st->wall_hits += td.walls;
            }
        }
        if (st) st->n_absorbed[s] += absorbed;
    }
    o.move_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return status;
}

// ------------------------------------------------------------ collisions --
constexpr double kBoltzmann = 1.380649e-23;
constexpr double kPlanck = 6.62607015e-34;

V3 normal3(ocoll::Philox& r) {
    const double a = r.normal(), b = r.normal(), c = r.normal();
    return v3(a, b, c);
}

// Nanbu scattering against a partner of mass mN (NanbuElectronNeutralCollision.C:97-131):
// cos(chi) = (eV + 2 - 2 (1 + eV)^R) / eV, azimuth 2 pi R.
void nanbu_scatter(double eV, V3& Ue, V3& Un, double mE, double mN, ocoll::Philox& r) {
    const double phi = 2.0 * kPi * r.uniform();
    double cosChi;
    if (eV < 1e-30) cosChi = 1.0;
    else cosChi = 1.0 / eV * (eV + 2.0 - 2.0 * std::pow(1.0 + eV, r.uniform()));
    double sinChi;
    if (cosChi * cosChi > 1.0) { cosChi = 1.0; sinChi = 0.0; }
    else sinChi = std::sqrt(1.0 - cosChi * cosChi);
    const V3 g = sub(Ue, Un);
    const double gm = magv(g);
    const double gp = std::sqrt(g.y * g.y + g.z * g.z);
    const double cp = std::cos(phi), sp = std::sin(phi);
    const V3 h = v3(gp * cp, -1.0 * (g.y * g.x * cp + gm * g.z * sp) / gp,
                    -1.0 * (g.z * g.x * cp - gm * g.y * sp) / gp);
    const V3 d = add(smul(1.0 - cosChi, g), smul(sinChi, h));
    Ue = sub(Ue, smul(mN / (mN + mE), d));
    Un = add(Un, smul(mE / (mN + mE), d));
}

// Relativistic centre-of-momentum frame of two particles and the rotation of
// the momentum in it by (chi, eps), shared by
// RelativisticElectronNeutralCollision.C:161-242 and PerezRelativisticCollision.C:60-192.
struct CoM {
    double gP, gQ, gc, gcv, gPc, gQc, mag_pc;
    V3 vc, pc;
};

bool com_frame(const V3& UP, const V3& UQ, double mP, double mQ, CoM& f) {
    const double aP = magv(UP) / kC, aQ = magv(UQ) / kC;
    f.gP = 1.0 / std::sqrt(1.0 - aP * aP);
    f.gQ = 1.0 / std::sqrt(1.0 - aQ * aQ);
    const V3 pP = smul(mP * f.gP, UP);
    const V3 pQ = smul(mQ * f.gQ, UQ);
    f.vc = sdiv(add(pP, pQ), mP * f.gP + mQ * f.gQ);
    const double vc2 = dotv(f.vc, f.vc);
    if (vc2 == 0.0) {
        f.gc = 1.0;
        f.gcv = 0.5;
        f.pc = pP;
        f.gPc = f.gP;
        f.gQc = f.gQ;
    } else {
        f.gc = 1.0 / std::sqrt(1.0 - vc2 / (kC * kC));
        f.gcv = (f.gc - 1.0) / vc2;
        f.pc = add(pP, smul((f.gcv * dotv(f.vc, UP) - f.gc) * mP * f.gP, f.vc));
        f.gPc = (1.0 - dotv(f.vc, UP) / (kC * kC)) * f.gP * f.gc;
        f.gQc = (1.0 - dotv(f.vc, UQ) / (kC * kC)) * f.gQ * f.gc;
    }
    f.mag_pc = magv(f.pc);
    return f.mag_pc != 0.0;
}

void com_rotate(const CoM& f, double cosChi, double sinChi, double eps, double mP, double mQ, V3& UP, V3& UQ) {
    const double sce = sinChi * std::cos(eps), sse = sinChi * std::sin(eps);
    const V3& p = f.pc;
    const double pperp = std::sqrt(p.x * p.x + p.y * p.y);
    V3 np;
    if (pperp > 1.e-10 * f.mag_pc) {
        const double ip = 1.0 / pperp;
        np = v3((p.x * p.z * sce - p.y * f.mag_pc * sse) * ip + p.x * cosChi,
                (p.y * p.z * sce + p.x * f.mag_pc * sse) * ip + p.y * cosChi, -pperp * sce + p.z * cosChi);
    } else {
        np = v3(f.mag_pc * sce, f.mag_pc * sse, f.mag_pc * cosChi);
    }
    const V3 npP = add(np, smul(f.gcv * dotv(f.vc, np) + mP * f.gPc * f.gc, f.vc));
    const double aP = magv(npP) / (mP * kC);
    const double ngP = std::sqrt(1.0 + aP * aP);
    const V3 mnp = smul(-1.0, np);
    const V3 npQ = add(mnp, smul(f.gcv * dotv(f.vc, mnp) + mQ * f.gQc * f.gc, f.vc));
    const double aQ = magv(npQ) / (mQ * kC);
    const double ngQ = std::sqrt(1.0 + aQ * aQ);
    UP = sdiv(npP, mP * ngP);
    UQ = sdiv(npQ, mQ * ngQ);
}

// RelativisticElectronNeutralCollision::updateVelocity (:161-242): draws
// cos(chi) first, then the azimuth.
void relativistic_scatter(double eV, V3& Ue, V3& Un, double mE, double mN, ocoll::Philox& r) {
    CoM f;
    if (!com_frame(Ue, Un, mE, mN, f)) return;
    double cosChi;
    if (eV < 1e-30) cosChi = 1.0;
    else cosChi = 1.0 / eV * (eV + 2.0 - 2.0 * std::pow(1.0 + eV, r.uniform()));
    const double sinChi = std::sqrt(1.0 - cosChi * cosChi);
    const double eps = 2.0 * kPi * r.uniform();
    com_rotate(f, cosChi, sinChi, eps, mE, mN, Ue, Un);
}

void electron_scatter(const Oracle& o, double eV, V3& Ue, V3& Un, double mE, double mN, ocoll::Philox& r) {
    if (o.cfg.mcc.scatter == 1) relativistic_scatter(eV, Ue, Un, mE, mN, r);
    else nanbu_scatter(eV, Ue, Un, mE, mN, r);
}

// ElectronNeutralCollisionModel::performBackgroundCollisions
// (ElectronNeutralCollisionModel.C:703-829) with the event kinematics of
// :532-544 (elastic), :567-585 (excitation), :645-700 (ionisation).
void mcc_background(Oracle& o, std::vector<std::vector<int>>& occ, picgpu_step_stats* st) {
    const picgpu_mcc& mc = o.cfg.mcc;
    const int es = o.cfg.electron_species;
    const double me = o.cfg.species[es].mass;
    const double mg = mc.gas_mass;
    const double dt = o.cfg.dt;
    const double vth = std::sqrt(kBoltzmann * mc.gas_temperature / mg);
    auto& el = o.cloud[es];
    std::vector<Parcel> new_e, new_i;
    long long cand = 0, nel = 0, nex = 0, niz = 0;
    for (int c = 0; c < o.m.n_cells; ++c) {
        const std::vector<int>& list = occ[c];
        const long eC = long(list.size());
        const double sv = o.svmax[c];
        const double coll = o.remainder[c] + double(eC) * mc.gas_density * sv * dt;
        const long nC = long(coll);
        o.remainder[c] = coll - double(nC);
        if (nC == 0 || eC == 0) continue;
        ocoll::Philox r(o.cfg.seed, ocoll::kStreamMcc, uint32_t(c), uint32_t(o.step_index));
        cand += nC;
        for (long i = 0; i < nC; ++i) {
            long j = long(r.uniform() * double(eC));
            if (j >= eC) j = eC - 1;
            Parcel& e = el[list[j]];
            const V3 nrm = normal3(r);
            V3 Un = v3(vth * nrm.x + mc.gas_velocity[0], vth * nrm.y + mc.gas_velocity[1],
                       vth * nrm.z + mc.gas_velocity[2]);
            const double cR = magv(sub(e.U, Un));
            const double gamma = 1.0 / std::sqrt(1.0 - (cR * cR) / (kC * kC));
            double eV = (gamma - 1.0) * me * kC * kC / ocoll::kEcharge;
            const double sigmaT = sv / cR;
            const double Qel = ocoll::interp_xs(eV, o.xs.e, o.xs.el);
            const double Qex = ocoll::interp_xs(eV, o.xs.e, o.xs.ex);
            const double Qiz = ocoll::interp_xs(eV, o.xs.e, o.xs.iz);
            const double Qt = Qel + Qex + Qiz;
            if (Qt * cR > o.svmax[c]) o.svmax[c] = Qt * cR;
            const double R = r.uniform();
            if (R <= Qel / sigmaT) {
                nel++;
                electron_scatter(o, eV, e.U, Un, me, mg, r);
            } else if (eV >= mc.ex_threshold && R <= (Qel + Qex) / sigmaT) {
                nex++;
                e.U = smul(std::sqrt(1.0 - mc.ex_threshold / eV), e.U);
                eV -= mc.ex_threshold;
                electron_scatter(o, eV, e.U, Un, me, mg, r);
            } else if (eV >= mc.iz_threshold && R <= Qt / sigmaT) {
                const double th = mc.iz_threshold;
                const double E0 = 2.0 - 100.0 / (eV + 10.0);
                const double E1 = (eV - th) / 2.0 - E0;
                const double alpha = 10.3;
                const double Ep = E0 + alpha * std::tan(r.uniform() * (std::atan(E1 / alpha) + std::atan(E0 / alpha)) -
                                                        std::atan(E0 / alpha));
                const V3 preUe = e.U;
                const V3 preUn = Un;
                e.U = smul(std::sqrt(1.0 - (th + Ep) / eV), e.U);
                eV -= (th + Ep);
                const double wE = o.cfg.species[es].weight, wN = mc.gas_weight;
                const double wEwN = wE / wN, wNwE = 1.0 / wEwN;
                electron_scatter(o, eV, e.U, Un, me, mg, r);
                const double rndU = r.uniform();
                bool created = false;
                if (rndU <= wEwN && mc.create_ion && mc.ion_species >= 0) {
                    Parcel ion = e;
                    ion.U = Un;
                    new_i.push_back(ion);
                    created = true;
                }
                if (rndU > wNwE) e.U = preUe;
                if (rndU <= wEwN && mc.create_electron) {
                    Parcel ne = e;
                    const double sp = std::sqrt(2.0 * Ep * ocoll::kEcharge / me);
                    ne.U = smul(sp, sdiv(preUe, magv(preUe)));
                    V3 un2 = preUn;
                    electron_scatter(o, Ep, ne.U, un2, me, mg, r);
                    new_e.push_back(ne);
                }
                if (created) niz++;
            }
        }
    }
    for (auto& p : new_e) el.push_back(p);
    if (mc.ion_species >= 0)
        for (auto& p : new_i) o.cloud[mc.ion_species].push_back(p);
    if (st) {
        st->mcc_candidates += cand;
        st->mcc_elastic += nel;
        st->mcc_excitation += nex;
        st->mcc_ionization += niz;
    }
}

// ElectronNeutralCollisionModel::performCollisions
// (ElectronNeutralCollisionModel.C:833-1009): collisions with the neutral
// parcels of the cell (NTC candidates eC nC w_max (sigma_T c_R)_max dt / V,
// a random neutral and a random electron each), with the events of the
// background model and the parcel as partner (:489-645); an ionised neutral
// is deleted unless deleteNeutral is off.
void mcc_parcels(Oracle& o, std::vector<std::vector<std::vector<int>>>& occ, picgpu_step_stats* st) {
    const picgpu_mcc& mc = o.cfg.mcc;
    const int es = o.cfg.electron_species, ns = mc.neutral_species;
    const double me = o.cfg.species[es].mass, mn = o.cfg.species[ns].mass;
    const double wE = o.cfg.species[es].weight, wN = o.cfg.species[ns].weight;
    const double wmax = std::max(wE, wN);
    const double dt = o.cfg.dt;
    const bool update_neutral = !mc.keep_neutral_velocity, delete_neutral = !mc.keep_neutrals;
    auto& el = o.cloud[es];
    auto& neu = o.cloud[ns];
    std::vector<Parcel> new_e, new_i;
    long long cand = 0, nel = 0, nex = 0, niz = 0;
    for (int c = 0; c < o.m.n_cells; ++c) {
        const std::vector<int>& elist = occ[es][c];
        std::vector<int>& nlist = occ[ns][c];
        const long eC = long(elist.size());
        long nC = long(nlist.size());
        const double sv = o.psvmax[c];
        if (!(sv > 0.0) || nC == 0 || eC == 0) continue;
        const double selected = o.premainder[c] + double(int(eC) * int(nC)) * wmax * sv * dt / o.m.vol[c];
        const long nCand = long(selected);
        o.premainder[c] = selected - double(nCand);
        cand += nCand;
        if (nCand == 0) continue;
        ocoll::Philox r(o.cfg.seed, ocoll::kStreamMcc | 1u, uint32_t(c), uint32_t(o.step_index));
        for (long i = 0; i < nCand; ++i) {
            long jn = long(r.uniform() * double(nC));
            if (jn >= nC) jn = nC - 1;
            long je = long(r.uniform() * double(eC));
            if (je >= eC) je = eC - 1;
            Parcel& n = neu[nlist[jn]];
            Parcel& e = el[elist[je]];
            V3 Un = n.U;
            const double cR = magv(sub(e.U, Un));
            const double gamma = 1.0 / std::sqrt(1.0 - (cR * cR) / (kC * kC));
            double eV = (gamma - 1.0) * me * kC * kC / ocoll::kEcharge;
            const double Qel = ocoll::interp_xs(eV, o.xs.e, o.xs.el);
            const double Qex = ocoll::interp_xs(eV, o.xs.e, o.xs.ex);
            const double Qiz = ocoll::interp_xs(eV, o.xs.e, o.xs.iz);
            const double Qt = Qel + Qex + Qiz;
            if (Qt * cR > o.psvmax[c]) o.psvmax[c] = Qt * cR;
            const double R = r.uniform();
            if (R <= Qel * cR / sv) {
                nel++;
                electron_scatter(o, eV, e.U, Un, me, mn, r);
                if (update_neutral) n.U = Un;
            } else if (eV >= mc.ex_threshold && R <= (Qel + Qex) * cR / sv) {
                nex++;
                e.U = smul(std::sqrt(1.0 - mc.ex_threshold / eV), e.U);
                eV -= mc.ex_threshold;
                electron_scatter(o, eV, e.U, Un, me, mn, r);
                if (update_neutral) n.U = Un;
            } else if (eV >= mc.iz_threshold && R <= Qt * cR / sv) {
                const double th = mc.iz_threshold;
                const double E0 = 2.0 - 100.0 / (eV + 10.0);
                const double E1 = (eV - th) / 2.0 - E0;
                const double alpha = 10.3;
                const double Ep = E0 + alpha * std::tan(r.uniform() * (std::atan(E1 / alpha) + std::atan(E0 / alpha)) -
                                                        std::atan(E0 / alpha));
                const V3 preUe = e.U;
                const V3 preUn = Un;
                e.U = smul(std::sqrt(1.0 - (th + Ep) / eV), e.U);
                eV -= (th + Ep);
                const double wEwN = wE / wN, wNwE = 1.0 / wEwN;
                electron_scatter(o, eV, e.U, Un, me, mn, r);
                const double rndU = r.uniform();
                bool created = false;
                if (rndU <= wEwN && mc.create_ion) {
                    Parcel ion = n;          // at the neutral's position, with its scattered velocity
                    ion.U = Un;
                    new_i.push_back(ion);
                    created = true;
                }
                if (rndU > wNwE) e.U = preUe;
                if (rndU <= wEwN && mc.create_electron) {
                    Parcel ne = e;
                    const double sp = std::sqrt(2.0 * Ep * ocoll::kEcharge / me);
                    ne.U = smul(sp, sdiv(preUe, magv(preUe)));
                    V3 un2 = preUn;
                    electron_scatter(o, Ep, ne.U, un2, me, mn, r);
                    new_e.push_back(ne);
                }
                if (update_neutral) n.U = Un;
                if (created) {
                    niz++;
                    if (delete_neutral) {
                        n.alive = false;
                        nlist.erase(nlist.begin() + jn);
                        --nC;
                        if (nC < 1) break;
                    }
                }
            }
        }
    }
    // deleted neutrals leave the cloud in order; the cell lists, which the
    // ion - neutral parcel step reads next (picFoam's sortedCellOccupancy
    // holds parcel pointers), follow the parcels to their new indices
    size_t w = 0;
    std::vector<int> moved(neu.size(), -1);
    for (size_t k = 0; k < neu.size(); ++k)
        if (neu[k].alive) {
            moved[k] = int(w);
            neu[w++] = neu[k];
        }
    if (size_t(ns) < o.occ_n.size()) o.occ_n[ns] -= long(neu.size() - w);
    neu.resize(w);
    for (auto& list : occ[ns])
        for (int& idx : list) idx = moved[idx];
    for (auto& p : new_e) el.push_back(p);
    if (mc.ion_species >= 0 && mc.create_ion)
        for (auto& p : new_i) o.cloud[mc.ion_species].push_back(p);
    if (st) {
        st->mcc_parcel_candidates += cand;
        st->mcc_parcel_elastic += nel;
        st->mcc_parcel_excitation += nex;
        st->mcc_parcel_ionization += niz;
    }
}

void weight_correct_pair(int model, double wP, double wQ, double mP, double mQ, const V3& preP, const V3& preQ,
                         V3& UP, V3& UQ, ocoll::Philox& r);

// IonNeutralCollisionModel::performCollisions (IonNeutralCollisionModel.C:
// 579-707): ions with the neutral parcels of the cell, isotropic elastic
// scattering of the pair (neutral P, ion Q; IonIsotropicScattering.C:60-100)
// or the charge-exchange identity switch (:401-413).
void ion_parcels(Oracle& o, std::vector<std::vector<std::vector<int>>>& occ, picgpu_step_stats* st) {
    const picgpu_ion_mcc& im = o.cfg.ion_mcc;
    const int is = im.ion_species, ns = im.neutral_species;
    const double mi = o.cfg.species[is].mass, mn = o.cfg.species[ns].mass;
    const double wI = o.cfg.species[is].weight, wN = o.cfg.species[ns].weight;
    const double wmax = std::max(wN, wI), dt = o.cfg.dt, mt = mn + mi;
    const bool update_neutral = !im.keep_neutral_velocity;
    auto& ions = o.cloud[is];
    auto& neu = o.cloud[ns];
    long long cand = 0, nel = 0, ncx = 0;
    for (int c = 0; c < o.m.n_cells; ++c) {
        const std::vector<int>& ilist = occ[is][c];
        const std::vector<int>& nlist = occ[ns][c];
        const long iC = long(ilist.size()), nC = long(nlist.size());
        if (nC == 0 || iC == 0) continue;
        const double sv = o.ipsvmax[c];
        const double selected = o.ipremainder[c] + double(int(nC) * int(iC)) * wmax * sv * dt / o.m.vol[c];
        const long nCand = long(selected);
        o.ipremainder[c] = selected - double(nCand);
        cand += nCand;
        if (nCand == 0) continue;
        ocoll::Philox r(o.cfg.seed, ocoll::kStreamIonMcc | 1u, uint32_t(c), uint32_t(o.step_index));
        for (long k = 0; k < nCand; ++k) {
            long jp = long(r.uniform() * double(nC));
            if (jp >= nC) jp = nC - 1;
            long jq = long(r.uniform() * double(iC));
            if (jq >= iC) jq = iC - 1;
            Parcel& P = neu[nlist[jp]];
            Parcel& Q = ions[ilist[jq]];
            const double cR = magv(sub(Q.U, P.U));
            const double gamma = 1.0 / std::sqrt(1.0 - (cR * cR) / (kC * kC));
            const double eV = (gamma - 1.0) * mi * kC * kC / ocoll::kEcharge;
            const double Qel = ocoll::interp_xs(eV, o.ixs.e, o.ixs.el);
            const double Qcx = ocoll::interp_xs(eV, o.ixs.e, o.ixs.ex);
            const double Qt = Qel + Qcx;
            if (Qt * cR > o.ipsvmax[c]) o.ipsvmax[c] = Qt * cR;
            const double rndU = r.uniform();
            if (rndU <= Qel * cR / sv) {
                nel++;
                const V3 preUP = P.U;
                const V3 preUQ = Q.U;
                const V3 Ucm = v3((mn * P.U.x + mi * Q.U.x) / mt, (mn * P.U.y + mi * Q.U.y) / mt,
                                  (mn * P.U.z + mi * Q.U.z) / mt);
                const double cr = magv(sub(P.U, Q.U));
                const double cosT = 2.0 * r.uniform() - 1.0;
                const double sinT = std::sqrt(1.0 - cosT * cosT);
                const double phi = 2.0 * kPi * r.uniform();
                const V3 rel = v3(cr * cosT, cr * (sinT * std::cos(phi)), cr * (sinT * std::sin(phi)));
                P.U = v3(Ucm.x + rel.x * mi / mt, Ucm.y + rel.y * mi / mt, Ucm.z + rel.z * mi / mt);
                Q.U = v3(Ucm.x - rel.x * mn / mt, Ucm.y - rel.y * mn / mt, Ucm.z - rel.z * mn / mt);
                // weightCorrection_->correctVelocity(pP, pQ, preUp, preUq)
                // (IonNeutralCollisionModel.C:443-444), before the
                // updateNeutralVelocity reset
                weight_correct_pair(im.weight_correction, wN, wI, mn, mi, preUP, preUQ, P.U, Q.U, r);
                if (!update_neutral) P.U = preUP;
            } else if (eV >= im.cx_threshold && rndU <= Qt * cR / sv) {
                ncx++;
                const double u = r.uniform();
                const V3 tmpP = P.U;
                if (u <= wI / wN) P.U = Q.U;
                if (u <= wN / wI) Q.U = tmpP;
                if (!update_neutral) P.U = tmpP;
            }
        }
    }
    if (st) {
        st->ion_parcel_candidates += cand;
        st->ion_parcel_elastic += nel;
        st->ion_parcel_charge_exchange += ncx;
    }
}

// IonNeutralCollisionModel::performBackgroundCollisions
// (IonNeutralCollisionModel.C:453-577): IsotropicScattering elastic
// (IonIsotropicScattering.C:103-143) or charge exchange (:419-426).
void ion_mcc_background(Oracle& o, std::vector<std::vector<int>>& occ, picgpu_step_stats* st) {
    const picgpu_ion_mcc& im = o.cfg.ion_mcc;
    const picgpu_mcc& gas = o.cfg.mcc;
    const int is = im.ion_species;
    const double mi = o.cfg.species[is].mass;
    const double mg = gas.gas_mass;
    const double dt = o.cfg.dt;
    const double vth = std::sqrt(kBoltzmann * gas.gas_temperature / mg);
    auto& ions = o.cloud[is];
    long long cand = 0, nel = 0, ncx = 0;
    for (int c = 0; c < o.m.n_cells; ++c) {
        const std::vector<int>& list = occ[c];
        const long nI = long(list.size());
        const double sv = o.isvmax[c];
        const double coll = o.iremainder[c] + double(nI) * gas.gas_density * sv * dt;
        const long nC = long(coll);
        o.iremainder[c] = coll - double(nC);
        if (nC == 0 || nI == 0) continue;
        ocoll::Philox r(o.cfg.seed, ocoll::kStreamIonMcc, uint32_t(c), uint32_t(o.step_index));
        cand += nC;
        for (long i = 0; i < nC; ++i) {
            long j = long(r.uniform() * double(nI));
            if (j >= nI) j = nI - 1;
            Parcel& p = ions[list[j]];
            const V3 nrm = normal3(r);
            V3 Un = v3(vth * nrm.x + gas.gas_velocity[0], vth * nrm.y + gas.gas_velocity[1],
                       vth * nrm.z + gas.gas_velocity[2]);
            const double cR = magv(sub(p.U, Un));
            const double gamma = 1.0 / std::sqrt(1.0 - (cR * cR) / (kC * kC));
            const double eV = (gamma - 1.0) * mi * kC * kC / ocoll::kEcharge;
            const double sigmaT = sv / cR;
            const double Qel = ocoll::interp_xs(eV, o.ixs.e, o.ixs.el);
            const double Qcx = ocoll::interp_xs(eV, o.ixs.e, o.ixs.ex);
            const double Qt = Qel + Qcx;
            if (Qt * cR > o.isvmax[c]) o.isvmax[c] = Qt * cR;
            const double R = r.uniform();
            if (R <= Qel / sigmaT) {
                nel++;
                // isotropic scattering in the centre-of-mass frame
                const V3 Ucm = sdiv(add(smul(mi, p.U), smul(mg, Un)), mi + mg);
                const double cosT = 2.0 * r.uniform() - 1.0;
                const double sinT = std::sqrt(1.0 - cosT * cosT);
                const double phi = 2.0 * kPi * r.uniform();
                const V3 rel = smul(cR, v3(cosT, sinT * std::cos(phi), sinT * std::sin(phi)));
                p.U = add(Ucm, sdiv(smul(mg, rel), mi + mg));
            } else if (eV >= im.cx_threshold && R <= Qt / sigmaT) {
                ncx++;
                p.U = Un;  // identity swap with the background neutral
            }
        }
    }
    if (st) {
        st->ion_mcc_candidates += cand;
        st->ion_mcc_elastic += nel;
        st->ion_mcc_charge_exchange += ncx;
    }
}

// NanbuCollision::calculate_cosChi (NanbuCollision.C:137-161), also
// PerezRelativisticCollision::calculate_cosChi.
double nanbu_cos_chi(double s, ocoll::Philox& r) {
    double U = r.uniform();
    if (s < 0.1) {
        if (U < 0.0001) U = 0.0001;
        return 1.0 + s * std::log(U);
    }
    if (s < 3.0) {
        const double invA = 0.00569578 + (0.95602 + (-0.508139 + (0.479139 + (-0.12789 + 0.0238957 * s) * s) * s) * s) * s;
        const double A = 1.0 / invA;
        return invA * std::log(std::exp(-A) + 2.0 * U * std::sinh(A));
    }
    if (s < 6.0) {
        const double A = 3.0 * std::exp(-s);
        return (1.0 / A) * std::log(std::exp(-A) + 2.0 * U * std::sinh(A));
    }
    return 2.0 * U - 1.0;
}

// NanbuWeightCorrectionModel::correctVelocity (NanbuCorrection.C:50-66): one
// draw; each partner keeps its new velocity with probability w_other/w_self.
// Sentoku-Kemp weight corrections (SentokuKempNonRelCorrection.C:50-125,
// SentokuKempCorrection.C:50-169): the parcel of the larger weight gets the
// weight-averaged velocity (momentum) plus an orthogonal kick restoring the
// weight-averaged kinetic (total) energy, at a uniform azimuth.
void sk_basis(const V3& a, double amag, V3& e2, V3& e3) {
    e2 = v3(0.0, 1.0, 0.0);
    e3 = v3(0.0, 0.0, 1.0);
    const double up = std::sqrt(a.y * a.y + a.z * a.z);
    if (up > 1.0e-300) {  // VSMALL
        e2 = v3(0.0, a.z / up, -a.y / up);
        const double den = amag * up;
        e3 = v3((up * up) / den, -(a.x * a.y) / den, -(a.x * a.z) / den);
    }
}

void sentoku_kemp_nr(double mass, double wr, const V3& pre, V3& U, ocoll::Philox& r) {
    const V3 after = v3((1.0 - wr) * pre.x + wr * U.x, (1.0 - wr) * pre.y + wr * U.y, (1.0 - wr) * pre.z + wr * U.z);
    const double afterE = (1.0 - wr) * 0.5 * mass * dotv(pre, pre) + wr * 0.5 * mass * dotv(U, U);
    const double dE = afterE - 0.5 * mass * dotv(after, after);
    if (!(dE > 0.0)) return;
    V3 e2, e3;
    sk_basis(after, std::sqrt(dotv(after, after)), e2, e3);
    const double eps = 6.283185307179586 * r.uniform();  // twoPi * scalar01
    const double sp = std::sqrt(dE * 2.0 / mass), ce = std::cos(eps), se = std::sin(eps);
    U = v3(after.x + sp * (e2.x * ce + e3.x * se), after.y + sp * (e2.y * ce + e3.y * se),
           after.z + sp * (e2.z * ce + e3.z * se));
}

void sentoku_kemp(double mass, double dw, const V3& pre, V3& U, ocoll::Philox& r) {
    const double c = kC;
    const double mpre = std::sqrt(dotv(pre, pre)) / c, mpost = std::sqrt(dotv(U, U)) / c;
    const double g0 = 1.0 / std::sqrt(1.0 - mpre * mpre), g1 = 1.0 / std::sqrt(1.0 - mpost * mpost);
    const V3 p0 = v3(mass * g0 * pre.x, mass * g0 * pre.y, mass * g0 * pre.z);
    const V3 p1 = v3(mass * g1 * U.x, mass * g1 * U.y, mass * g1 * U.z);
    const double mc = mass * c;
    const double e0 = c * std::sqrt(dotv(p0, p0) + mc * mc), e1 = c * std::sqrt(dotv(p1, p1) + mc * mc);
    const double aE = (1.0 - dw) * e0 + dw * e1;
    const V3 aM = v3((1.0 - dw) * p0.x + dw * p1.x, (1.0 - dw) * p0.y + dw * p1.y, (1.0 - dw) * p0.z + dw * p1.z);
    const double aMm = std::sqrt(dotv(aM, aM));
    const double ge = aE / (mass * (c * c));
    const double gq = aMm / mc;
    const double gp = std::sqrt(1.0 + gq * gq);
    if (!(gp < ge)) return;
    const double dp = mass * c * std::sqrt(ge * ge - gp * gp);
    V3 e2, e3;
    sk_basis(aM, aMm, e2, e3);
    const double eps = 6.283185307179586 * r.uniform();
    const double ce = std::cos(eps), se = std::sin(eps);
    const V3 ps = v3(aM.x + dp * (e2.x * ce + e3.x * se), aM.y + dp * (e2.y * ce + e3.y * se),
                     aM.z + dp * (e2.z * ce + e3.z * se));
    const double gs0 = std::sqrt(dotv(ps, ps)) / mc;
    const double gs = std::sqrt(1.0 + gs0 * gs0);
    U = v3(ps.x / (mass * gs), ps.y / (mass * gs), ps.z / (mass * gs));
}

// WeightCorrection: none, Nanbu (NanbuCorrection.C:50-66), SentokuKempNR,
// SentokuKemp.
void weight_correct(Oracle& o, Parcel& P, int sp, Parcel& Q, int sq, const V3& preP, const V3& preQ,
                    ocoll::Philox& r) {
    const int wc = o.cfg.coulomb.weight_correction;
    const double wP = pweight(o, P, sp), wQ = pweight(o, Q, sq);
    if (wc == 1) {
        const double u = r.uniform();
        if (u > wP / wQ) Q.U = preQ;
        if (u > wQ / wP) P.U = preP;
    } else if (wc == 2 || wc == 3) {
        if (wP > wQ) {
            if (wc == 3) sentoku_kemp(o.cfg.species[sp].mass, wQ / wP, preP, P.U, r);
            else sentoku_kemp_nr(o.cfg.species[sp].mass, wQ / wP, preP, P.U, r);
        } else if (wP < wQ) {
            if (wc == 3) sentoku_kemp(o.cfg.species[sq].mass, wP / wQ, preQ, Q.U, r);
            else sentoku_kemp_nr(o.cfg.species[sq].mass, wP / wQ, preQ, Q.U, r);
        }
    }
}

// NanbuCollision::collide (NanbuCollision.C:60-135).
void nanbu_collide(Oracle& o, Parcel& P, int sp, Parcel& Q, int sq, double lD, double nP, double nQ,
                   double nPQ, ocoll::Philox& r) {
    const double mP = o.cfg.species[sp].mass, qP = pcharge(o, P, sp);
    const double mQ = o.cfg.species[sq].mass, qQ = pcharge(o, Q, sq);
    const double reMass = mP * mQ / (mP + mQ);
    const V3 g = sub(P.U, Q.U);
    const double gm = magv(g);
    double cl = o.cfg.coulomb.coulomb_log;
    if (cl == 0.0) {
        double b0 = qP * qQ / (2.0 * kPi * kEps0 * reMass * gm * gm);
        if (o.cfg.coulomb.calculate_bmin) b0 = std::fmax(kPlanck / (2.0 * (gm * reMass)), std::fabs(b0));
        cl = std::fmax(2.0, 0.5 * std::log(1.0 + (lD * lD) / (b0 * b0)));
    }
    const double A = qP * qQ / (kEps0 * reMass);
    const double s = cl / (4.0 * kPi) * (A * A) * (nQ * nP / nPQ) * (1.0 / (gm * gm * gm)) * o.cfg.dt;
    const double cosChi = nanbu_cos_chi(s, r);
    const double sinChi = std::sqrt(1.0 - cosChi * cosChi);
    const double gp = std::sqrt(g.y * g.y + g.z * g.z);
    const double eps = 2.0 * kPi * r.uniform();
    const double ce = std::cos(eps), se = std::sin(eps);
    const V3 h = v3(gp * ce, -1.0 * (g.y * g.x * ce + gm * g.z * se) / gp,
                    -1.0 * (g.z * g.x * ce - gm * g.y * se) / gp);
    const V3 d = add(smul(1.0 - cosChi, g), smul(sinChi, h));
    const V3 preP = P.U, preQ = Q.U;
    P.U = sub(P.U, smul(mQ / (mP + mQ), d));
    Q.U = add(Q.U, smul(mP / (mP + mQ), d));
    weight_correct(o, P, sp, Q, sq, preP, preQ, r);
}

// PerezRelativisticCollision::collide (PerezRelativisticCollision.C:60-192).
void perez_collide(Oracle& o, Parcel& P, int sp, Parcel& Q, int sq, double lD, double nP, double nQ,
                   double nPQ, ocoll::Philox& r) {
    const double mP = o.cfg.species[sp].mass, qP = pcharge(o, P, sp);
    const double mQ = o.cfg.species[sq].mass, qQ = pcharge(o, Q, sq);
    CoM f;
    if (!com_frame(P.U, Q.U, mP, mQ, f)) return;
    const double mgsum = mP * f.gP + mQ * f.gQ;
    const double c2 = kC * kC;
    const double pc2 = f.mag_pc * f.mag_pc;
    double cl = o.cfg.coulomb.coulomb_log;
    if (cl == 0.0) {
        double b0 = qP * qQ / (4.0 * kPi * kEps0 * c2) * f.gc / mgsum * (1.0 + mP * f.gPc * mQ * f.gQc * c2 / pc2);
        if (o.cfg.coulomb.calculate_bmin) b0 = std::fmax(kPlanck / (2 * f.mag_pc), std::fabs(b0));
        cl = std::fmax(2.0, 0.5 * std::log(1.0 + (lD * lD) / (b0 * b0)));
    }
    const double t1 = f.gc * f.mag_pc / mgsum;
    const double t2b = 1.0 + mP * f.gPc * mQ * f.gQc * c2 / pc2;
    const double t2 = t2b * t2b;
    const double qq = qP * qQ;
    double s = (nP * nQ / nPQ) * o.cfg.dt * cl * (qq * qq) /
               (4.0 * kPi * (kEps0 * kEps0) * (c2 * c2) * mP * f.gP * mQ * f.gQ) * t1 * t2;
    const double v_rel = f.mag_pc * mgsum / (mP * f.gPc * mQ * f.gQc * f.gc);
    const double s_max = std::pow(4.0 * kPi / 3.0, 1.0 / 3.0) * (nP * nQ / nPQ) * o.cfg.dt * (mP + mQ) /
                         std::fmax(mP * std::pow(nP, 2.0 / 3.0), mQ * std::pow(nQ, 2.0 / 3.0)) * v_rel;
    s = std::fmin(s_max, s);
    const double cosChi = nanbu_cos_chi(s, r);
    const double sinChi = std::sqrt(1.0 - cosChi * cosChi);
    const double eps = 2.0 * kPi * r.uniform();
    const V3 preP = P.U, preQ = Q.U;
    com_rotate(f, cosChi, sinChi, eps, mP, mQ, P.U, Q.U);
    weight_correct(o, P, sp, Q, sq, preP, preQ, r);
}

// ---- PerezIonizationModel (CoulombCollisionModel/IonizationModel/
// PerezIonizationModel/PerezIonizationModel.C) ------------------------------

// IonizationData::calculateIonizationCrossSection (PerezIonizationModel.C:
// 405-484): per charge state the orbital-summed cross section, and the mean
// energies transferred to the new electron and lost by the colliding one
// (in m_e c^2), on 100 log-spaced energies 1 eV - 10 MeV; binding energies
// after Carlson (bindingEnergy, :395-399).
Oracle::PerezTab perez_tables(const picgpu_perez_ion& in) {
    Oracle::PerezTab T;
    const int A = in.atomic_number;
    T.atomic = A;
    T.limit = in.ionization_limit < 0 ? A : std::min(in.ionization_limit, A);
    T.cs.assign(size_t(A) * 100, 0.0);
    T.te.assign(size_t(A) * 100, 0.0);
    T.le.assign(size_t(A) * 100, 0.0);
    auto binding = [&](int Z, int k) {
        return in.ionization_energy[Z] - in.binding_energy[A - Z - 1] + in.binding_energy[k];
    };
    const double r_e = 2.8179403227e-15;
    const double step = 99.0 / std::log(1e7 / 1.0);
    for (int Z = 0; Z < A; ++Z)
        for (int i = 0; i < 100; ++i) {
            const double E = std::exp(double(i) / step);
            int N = 1;
            double cs = 0.0, te = 0.0, le = 0.0;
            for (int k = 0; k < A - Z; ++k) {
                const double Bk = binding(Z, k);
                if (k < A - Z - 1 && Bk == binding(Z, k + 1)) {
                    N++;
                    continue;
                }
                const double eps = E / Bk;
                if (eps > 1.0) {
                    const double b_dash = Bk / 510997.37;
                    const double eps_dash = E / 510997.37;
                    const double u_dash = b_dash;
                    const double beta_eps2 = 1.0 - 1.0 / ((1.0 + eps_dash) * (1.0 + eps_dash));
                    const double beta_b2 = 1.0 - 1.0 / ((1.0 + b_dash) * (1.0 + b_dash));
                    const double beta_u2 = 1.0 - 1.0 / ((1.0 + u_dash) * (1.0 + u_dash));
                    const double sigma0 = 2.0 * kPi * r_e * r_e * N / (b_dash * (beta_eps2 + beta_b2 + beta_u2));
                    double ediv2 = 1.0 + eps_dash * 0.5;
                    ediv2 *= ediv2;
                    const double A1 = 1.0 / (1.0 + eps) * (1.0 + 2 * eps_dash) / ediv2;
                    const double A2 = (eps - 1.0) / 2.0 * b_dash * b_dash / ediv2;
                    const double A3 = std::log(beta_eps2 / (1.0 - beta_eps2)) - beta_eps2 - std::log(2.0 * b_dash);
                    const double sk = sigma0 * (0.5 * A3 * (1.0 - 1.0 / (eps * eps)) + 1.0 - 1.0 / eps + A2 -
                                                A1 * std::log(eps));
                    const double wk = sigma0 * (0.5 * A3 * (eps - 1.0) * (eps - 1.0) / (eps * (eps - 1.0)) +
                                                2.0 * std::log((eps + 1.0) * 0.5) - std::log(eps) +
                                                A2 * (eps - 1.0) * 0.25 -
                                                A1 * (std::log(eps) - (eps + 1.0) * std::log(0.5 * (eps + 1.0))));
                    const double ek = sk + wk;
                    cs += sk;
                    te += wk * b_dash;
                    le += ek * b_dash;
                }
                N = 1;
            }
            if (cs > 0.0) {
                te /= cs;
                le /= cs;
            }
            T.cs[size_t(Z) * 100 + i] = cs;
            T.te[size_t(Z) * 100 + i] = te;
            T.le[size_t(Z) * 100 + i] = le;
        }
    return T;
}

// The model's state between the calls of one species pair (the members
// np_, ne_, nei_ of PerezIonizationModel): initIonization (:129-137) and
// prepareNumberDensities (:140-195).
struct Ionizer {
    double np = 0.0, ne = 0.0, nei = 0.0;
    std::vector<Parcel> electrons;   // parcels added by addNewParcel, appended after the step
};

bool perez_active(const Oracle& o, int s) { return size_t(s) < o.perez.size() && o.perez[s].limit >= 0 && o.perez[s].atomic > 0; }

void perez_init(const Oracle& o, Ionizer& I, int p, int q, double nP, double nQ) {
    I.ne = 0.0;
    I.nei = 0.0;
    if (p == o.cfg.electron_species) I.np = nQ;
    else if (q == o.cfg.electron_species) I.np = nP;
}

// the electron's kinetic energy [eV] from its Lorentz factor
double electron_eV(const Oracle& o, const Parcel& e) {
    const double m = o.cfg.species[o.cfg.electron_species].mass;
    const double b = magv(e.U) / kC;
    const double gamma = 1.0 / std::sqrt(1.0 - b * b);
    return (gamma - 1.0) * m * kC * kC / ocoll::kEcharge;
}

void perez_prepare_densities(const Oracle& o, Ionizer& I, const Parcel& P, int sp, const Parcel& Q, int sq) {
    const int es = o.cfg.electron_species;
    const Parcel* e;
    const Parcel* ion;
    int si;
    if (sp == es) { e = &P; ion = &Q; si = sq; }
    else if (sq == es) { e = &Q; ion = &P; si = sp; }
    else return;
    if (!perez_active(o, si) || ion->zq >= o.perez[si].limit) return;
    double x = 6.142165 * std::log(electron_eV(o, *e));
    if (x < 0.0) x = 0.0;
    else if (x > 99.0) x = 99.0;
    const double cs = o.perez[si].cs[size_t(ion->zq) * 100 + size_t(int(x))];
    if (cs > 0.0) {
        const double We = pweight(o, *e, es), Wi = pweight(o, *ion, si);
        I.ne += We;
        I.nei += We < Wi ? We : Wi;
    }
}

// prepareIonization (:198-234): the pair's electron and ion when the ion
// species ionises, its charge state is below the limit and nei > 0.
bool perez_prepare(const Oracle& o, const Ionizer& I, int sp, const Parcel& P, int sq, const Parcel& Q) {
    const int es = o.cfg.electron_species;
    int si;
    const Parcel* ion;
    if (sp == es && perez_active(o, sq)) { si = sq; ion = &Q; }
    else if (sq == es && perez_active(o, sp)) { si = sp; ion = &P; }
    else return false;
    if (ion->zq >= o.perez[si].limit) return false;
    return I.nei > 0.0;
}

// ionize (:237-385) for the electron e and ion of species si after their
// Coulomb collision; random numbers from the stream of the collision
// ordinal.  Returns whether the charge state rose.
bool perez_ionize(Oracle& o, Ionizer& I, Parcel& e, Parcel& ion, int si, int cell, long ordinal) {
    const int es = o.cfg.electron_species;
    const Oracle::PerezTab& T = o.perez[si];
    const int atomicNumber = T.atomic;
    int Zstar = ion.zq;
    const int initialZstar = Zstar;
    const double c = kC, c2 = kC * kC;
    double gammaE = 1.0 / std::sqrt(1.0 - (magv(e.U) / c) * (magv(e.U) / c));
    const double gammaP = 1.0 / std::sqrt(1.0 - (magv(ion.U) / c) * (magv(ion.U) / c));
    const double massE = o.cfg.species[es].mass, massP = o.cfg.species[si].mass;
    const double deltaT = o.cfg.dt;
    const double wE = pweight(o, e, es), wP = pweight(o, ion, si);
    const double wEwP = wE / wP;
    const double wPwE = 1.0 / wEwP;
    double gamma_s = gammaP * gammaE * (1.0 - magv(ion.U) * magv(e.U) / c2);
    if (gamma_s <= 1.0) return false;
    ocoll::Philox r = ocoll::ionize_stream(o.cfg.seed, uint32_t(cell), uint32_t(o.step_index), ordinal);
    const double ionCoeff_s = c * std::sqrt(gamma_s * gamma_s - 1.0) / gammaP * (I.np * I.ne / I.nei) * deltaT;
    const double eVkin_s = (gamma_s - 1.0) * massE * c * c / ocoll::kEcharge;
    const double rndU = r.uniform();
    const int ionizationMax = T.limit - Zstar - 1;
    std::vector<double> rate(atomicNumber, 0.0), rate_inv(atomicNumber, 0.0), prop(atomicNumber, 0.0);
    double com = 0.0;
    for (int k = 0; k <= ionizationMax; ++k) {
        const double s = 6.142165 * std::log(eVkin_s);
        if (s < 0.0) break;
        const double* cs = &T.cs[size_t(Zstar) * 100];
        const double* te = &T.te[size_t(Zstar) * 100];
        const double* le = &T.le[size_t(Zstar) * 100];
        double crossSection, transferred, lost;
        if (s < 99.0) {
            const int l = int(s);
            const double d = s - double(l);
            crossSection = (cs[l + 1] - cs[l]) * d + cs[l];
            transferred = (te[l + 1] - te[l]) * d + te[l];
            lost = (le[l + 1] - le[l]) * d + le[l];
        } else {
            const double d = s - 99.0;
            crossSection = (cs[99] - cs[98]) * d + cs[99];
            transferred = te[99];
            lost = le[99];
        }
        if (crossSection <= 0.0) break;
        if (lost > gamma_s - 1.0) break;
        rate[k] = ionCoeff_s * crossSection / gammaE;
        rate_inv[k] = 1.0 / rate[k];
        prop[k] = std::exp(-rate[k]);
        if (k == 0) {
            com = prop[k];
        } else {
            for (int x = 0; x < k; ++x) {
                double cp = 1.0 - rate[k] * rate_inv[x];
                for (int b = 0; b < x; ++b) cp *= 1.0 - rate[x] * rate_inv[b];
                for (int b = x + 1; b < k; ++b) cp *= 1.0 - rate[x] * rate_inv[b];
                if (k < ionizationMax) com += (prop[k] - prop[x]) / cp;
                else com += (1.0 - prop[k] + rate[k] * rate_inv[x] * (prop[x] - 1.0)) / cp;
            }
        }
        if (rndU < com) break;
        const V3 pOld = v3(e.U.x * gammaE * massE, e.U.y * gammaE * massE, e.U.z * gammaE * massE);
        const V3 pI = v3(ion.U.x * gammaP * massP, ion.U.y * gammaP * massP, ion.U.z * gammaP * massP);
        const double p2 = gamma_s * gamma_s - 1.0;
        const double rndU2 = r.uniform();
        if (rndU2 < wEwP) {
            ion.zq++;
            const double gammaW = transferred + 1.0;
            const double alpha_w = std::sqrt((gammaW * gammaW - 1.0) / p2);
            const double f = gammaW - alpha_w * gamma_s;
            const V3 pNew = v3(alpha_w * pOld.x + f * pI.x * massE / massP, alpha_w * pOld.y + f * pI.y * massE / massP,
                               alpha_w * pOld.z + f * pI.z * massE / massP);
            const double gNew = std::sqrt(1.0 + std::pow(magv(pNew) / (massE * c), 2));
            Parcel ne = e;
            ne.nw = wP;
            ne.zq = 1;
            ne.U = sdiv(pNew, massE * gNew);
            I.electrons.push_back(ne);
        }
        if (rndU2 < wPwE) {
            const double alpha_e = std::sqrt((std::pow(gamma_s - lost, 2) - 1.0) / p2);
            const double f = (1.0 - alpha_e) * gamma_s - lost;
            const V3 pLost = v3(alpha_e * pOld.x + f * pI.x * massE / massP, alpha_e * pOld.y + f * pI.y * massE / massP,
                                alpha_e * pOld.z + f * pI.z * massE / massP);
            const double gLost = std::sqrt(1.0 + std::pow(magv(pLost) / (massE * c), 2));
            e.U = sdiv(pLost, massE * gLost);
            gammaE += ((1.0 - alpha_e) * gamma_s - lost) * gammaP;
            gamma_s -= lost;
        }
        Zstar++;
    }
    return Zstar != initialZstar;
}

// One Coulomb collision with the random stream of its ordinal in cell c
// (ord counts the cell's collisions in the sequential pairing order); with
// an ionisation model, prepareIonization before and ionize after it.
void coulomb_collide(Oracle& o, Parcel& P, int sp, Parcel& Q, int sq, double lD, double nP, double nQ,
                     double nPQ, int c, long& ord, Ionizer* I = nullptr, long long* ionized = nullptr) {
    const long k = ord;
    const bool ionize = I && perez_prepare(o, *I, sp, P, sq, Q);
    ocoll::Philox r = ocoll::coulomb_pair_stream(o.cfg.seed, uint32_t(c), uint32_t(o.step_index), ord++);
    if (o.cfg.coulomb.collide == 1) perez_collide(o, P, sp, Q, sq, lD, nP, nQ, nPQ, r);
    else nanbu_collide(o, P, sp, Q, sq, lD, nP, nQ, nPQ, r);
    if (ionize) {
        const int es = o.cfg.electron_species;
        const bool pe = sp == es;
        if (perez_ionize(o, *I, pe ? P : Q, pe ? Q : P, pe ? sq : sp, c, k) && ionized) ++*ionized;
    }
}

void shuffle(std::vector<int>& a, ocoll::Philox& r) {
    for (long k = long(a.size()) - 1; k > 0; --k) {
        long j = long(r.uniform() * double(k + 1));
        if (j > k) j = k;
        std::swap(a[k], a[j]);
    }
}

// CoulombCollisionModel::debyeLength (CoulombCollisionModel.C:249-309) over
// the colliding species.
double debye_length(const Oracle& o, const std::vector<int>& charged,
                    std::vector<std::vector<std::vector<int>>>& occ, int c) {
    double debye = 0.0, n_max = 0.0;
    for (int s : charged) {
        const double mass = o.cfg.species[s].mass;
        // the per-species sums (CoulombCollisionModel.C:270-277, per parcel
        // nParticle and charge) in the lane order of the device's warp
        const std::vector<int>& L = occ[s][c];
        const long cnt = long(L.size());
        const auto& cl = o.cloud[s];
        auto w = [&](long t) { return pweight(o, cl[L[t]], s); };
        double vSqr = ocoll::warp_sum(cnt, [&](long t) { return dotv(cl[L[t]].U, cl[L[t]].U) * w(t); });
        double charge = ocoll::warp_sum(cnt, [&](long t) { return pcharge(o, cl[L[t]], s) * w(t); });
        V3 v = v3(ocoll::warp_sum(cnt, [&](long t) { return w(t) * cl[L[t]].U.x; }),
                  ocoll::warp_sum(cnt, [&](long t) { return w(t) * cl[L[t]].U.y; }),
                  ocoll::warp_sum(cnt, [&](long t) { return w(t) * cl[L[t]].U.z; }));
        double n = ocoll::warp_sum(cnt, [&](long t) { return w(t); });
        if (n <= 0.0) continue;
        v = sdiv(v, n);
        charge /= n;
        vSqr /= n;
        n /= o.m.vol[c];
        if (n > n_max) n_max = n;
        const double vd2 = o.cfg.coulomb.debye_drift ? dotv(v, v) : 0.0;
        const double T = mass / (3.0 * kBoltzmann) * (vSqr - vd2);
        if (T <= 0.0) continue;
        debye += n * charge * charge / kEps0 * 1.0 / (T * kBoltzmann);
    }
    if (debye <= 0.0) return 0.0;
    const double r_min = std::pow(4.0 * kPi * n_max / 3.0, -1.0 / 3.0);
    return std::fmax(r_min, std::sqrt(1 / debye));
}

// NanbuYonemuraPairing::pairANDcollide (NanbuYonemuraPairing.C:56-325) and
// TakizukaAbePairing::pairANDcollide (TakizukaAbePairing.C:60-341).
void coulomb_pairs(Oracle& o, std::vector<std::vector<std::vector<int>>>& occ, picgpu_step_stats* st) {
    std::vector<int> charged;
    for (int s = 0; s < o.cfg.n_species; ++s)
        if (o.cfg.species[s].charge != 0.0 && o.cfg.species[s].solve_movement) charged.push_back(s);
    const bool ta = o.cfg.coulomb.pairing == 1;
    const bool need_debye = o.cfg.coulomb.coulomb_log == 0.0;
    long long pairs = 0, ionized = 0;
    Ionizer ionizer;
    Ionizer* I = o.cfg.perez.enabled ? &ionizer : nullptr;
    for (int c = 0; c < o.m.n_cells; ++c) {
        const double V = o.m.vol[c];
        // the shuffles draw from the cell's stream in order, each collision
        // from the counter range of its ordinal
        ocoll::Philox r(o.cfg.seed, ocoll::kStreamCoulomb, uint32_t(c), uint32_t(o.step_index));
        long ord = 0;
        const double lD = need_debye ? debye_length(o, charged, occ, c) : 0.0;
        for (size_t i = 0; i < charged.size(); ++i) {
            for (size_t jj = charged.size(); jj-- > 0;) {
                if (jj < i) break;
                const int a = charged[i], b = charged[jj];
                std::vector<int>& LA = occ[a][c];
                std::vector<int>& LB = occ[b][c];
                const long nA = long(LA.size()), nB = long(LB.size());
                const double wA = o.cfg.species[a].weight;
                auto& ca = o.cloud[a];
                auto& cb = o.cloud[b];
                // NanbuYonemuraPairing.C:96-113: the real particles of each
                // species, parcel by parcel
                double sA = 0.0, sB = 0.0;
                for (long t = 0; t < nA; ++t) sA += pweight(o, ca[LA[t]], a);
                if (a != b)
                    for (long t = 0; t < nB; ++t) sB += pweight(o, cb[LB[t]], b);
                auto pw = [&](const std::vector<Parcel>& cl, const std::vector<int>& L, int k, int sp) {
                    return pweight(o, cl[L[k]], sp);
                };
                if (a == b && nA > 1) {
                    if (!o.cfg.coulomb.allow_intra) continue;
                    std::vector<int> sel(nA);
                    for (long k = 0; k < nA; ++k) sel[k] = int(k);
                    shuffle(sel, r);
                    if (ta) {
                        const double n = double(nA) * wA / V;
                        if (nA % 2 != 0) {
                            const double n12 = (double(nA) + 3.0) * wA / V;
                            Parcel& P = ca[LA[sel[0]]];
                            Parcel& Q = ca[LA[sel[1]]];
                            Parcel& R = ca[LA[sel[2]]];
                            coulomb_collide(o, P, a, Q, a, lD, n, n, n12, c, ord);
                            coulomb_collide(o, Q, a, R, a, lD, n, n, n12, c, ord);
                            coulomb_collide(o, P, a, R, a, lD, n, n, n12, c, ord);
                            for (long x = 3; x < nA - 1; x += 2)
                                coulomb_collide(o, ca[LA[sel[x]]], a, ca[LA[sel[x + 1]]], a, lD, n, n, n12, c, ord);
                            pairs += 2 + nA / 2;
                        } else {
                            for (long x = 0; x < nA - 1; x += 2)
                                coulomb_collide(o, ca[LA[sel[x]]], a, ca[LA[sel[x + 1]]], a, lD, n, n, n, c, ord);
                            pairs += nA / 2;
                        }
                        continue;
                    }
                    const double n = sA / V;
                    if (nA % 2 != 0) {
                        // the extra (last, first) pair first (NanbuYonemuraPairing.C:128-141)
                        double nAA = 0.0;
                        nAA += 2.0 * std::fmin(pw(ca, LA, sel[nA - 1], a), pw(ca, LA, sel[0], a));
                        for (long x = 0; x < nA - 2; x += 2)
                            nAA += 2.0 * std::fmin(pw(ca, LA, sel[x], a), pw(ca, LA, sel[x + 1], a));
                        const double n12 = nAA / V;
                        for (long x = 0; x < nA - 2; x += 2)
                            coulomb_collide(o, ca[LA[sel[x]]], a, ca[LA[sel[x + 1]]], a, lD, n, n, n12, c, ord);
                        coulomb_collide(o, ca[LA[sel[nA - 1]]], a, ca[LA[sel[0]]], a, lD, n, n, n12, c, ord);
                        pairs += 1 + nA / 2;
                    } else {
                        double nAA = 0.0;
                        for (long x = 0; x < nA - 1; x += 2)
                            nAA += 2.0 * std::fmin(pw(ca, LA, sel[x], a), pw(ca, LA, sel[x + 1], a));
                        const double n12 = nAA / V;
                        for (long x = 0; x < nA - 1; x += 2)
                            coulomb_collide(o, ca[LA[sel[x]]], a, ca[LA[sel[x + 1]]], a, lD, n, n, n12, c, ord);
                        pairs += nA / 2;
                    }
                } else if (a != b && std::min(nA, nB) != 0) {
                    if (nA == nB) {
                        std::vector<int> sel(nA);
                        for (long k = 0; k < nA; ++k) sel[k] = int(k);
                        shuffle(sel, r);
                        double nP, nQ, nPQ;
                        if (ta) {
                            nP = double(nA) * wA / V;
                            nQ = double(nB) * wA / V;
                            nPQ = nP;
                        } else {
                            nP = sA / V;
                            nQ = sB / V;
                        }
                        // initIonization + prepareNumberDensities over the pairs
                        // (NanbuYonemuraPairing.C:198-208, TakizukaAbePairing.C:165-180)
                        if (I) perez_init(o, *I, a, b, nP, nQ);
                        double nAB = 0.0;
                        for (long k = 0; k < nA; ++k) {
                            if (!ta) nAB += std::fmin(pw(ca, LA, sel[k], a), pw(cb, LB, sel[nA - k - 1], b));
                            if (I) perez_prepare_densities(o, *I, ca[LA[sel[k]]], a, cb[LB[sel[nA - k - 1]]], b);
                        }
                        if (!ta) nPQ = nAB / V;
                        for (long k = 0; k < nA; ++k)
                            coulomb_collide(o, ca[LA[sel[k]]], a, cb[LB[sel[nA - k - 1]]], b, lD, nP, nQ, nPQ, c, ord,
                                            I, &ionized);
                        pairs += nA;
                    } else {
                        const int minS = nA < nB ? a : b, maxS = nA > nB ? a : b;
                        std::vector<int>& Lmin = nA < nB ? LA : LB;
                        std::vector<int>& Lmax = nA < nB ? LB : LA;
                        const long nMax = std::max(nA, nB), nMin = std::min(nA, nB);
                        std::vector<int> smin(nMin), smax(nMax);
                        for (long k = 0; k < nMax; ++k) { smax[k] = int(k); if (k < nMin) smin[k] = int(k); }
                        shuffle(smin, r);
                        shuffle(smax, r);
                        auto& cmin = o.cloud[minS];
                        auto& cmax = o.cloud[maxS];
                        if (ta) {
                            const double nMinS = double(nMin) * wA / V, nMaxS = double(nMax) * wA / V;
                            const long delta = nMax / nMin;
                            const double delta_r = double(nMax % nMin) / double(nMin);
                            const long g1min = long(delta_r * double(nMin));
                            const long g1max = long(double(delta + 1) * delta_r * double(nMin));
                            const long g2min = long((1.0 - delta_r) * double(nMin));
                            const long g2max = long(double(delta) * (1.0 - delta_r) * double(nMin));
                            long s1 = 0, s2 = 0;
                            if (g1min > 0) {
                                if (I) {
                                    perez_init(o, *I, minS, maxS, nMinS, nMaxS);
                                    for (long g = 0, q1 = 0; g < g1max; ++g, ++q1) {
                                        if (q1 >= g1min) q1 = 0;
                                        perez_prepare_densities(o, *I, cmin[Lmin[smin[q1]]], minS, cmax[Lmax[smax[g]]],
                                                                maxS);
                                    }
                                }
                                for (long g = 0; g < g1max; ++g) {
                                    if (s1 >= g1min) s1 = 0;
                                    coulomb_collide(o, cmax[Lmax[smax[s2]]], maxS, cmin[Lmin[smin[s1]]], minS, lD, nMaxS,
                                                    nMinS, nMaxS, c, ord, I, &ionized);
                                    ++s1;
                                    ++s2;
                                }
                            }
                            if (I) {
                                perez_init(o, *I, minS, maxS, nMinS, nMaxS);
                                for (long g = 0, q1 = g1min; g < g2max; ++g, ++q1) {
                                    if (q1 >= g2min + g1min) q1 = g1min;
                                    perez_prepare_densities(o, *I, cmin[Lmin[smin[q1]]], minS, cmax[Lmax[smax[g1max + g]]],
                                                            maxS);
                                }
                            }
                            s1 = g1min;
                            s2 = g1max;
                            for (long g = 0; g < g2max; ++g) {
                                if (s1 >= g2min + g1min) s1 = g1min;
                                coulomb_collide(o, cmax[Lmax[smax[s2]]], maxS, cmin[Lmin[smin[s1]]], minS, lD, nMaxS,
                                                nMinS, nMaxS, c, ord, I, &ionized);
                                ++s1;
                                ++s2;
                            }
                            pairs += g1max + g2max;
                            continue;
                        }
                        const double nMaxS = (maxS == a ? sA : sB) / V;
                        const double nMinS = (maxS == a ? sB : sA) / V;
                        if (I) perez_init(o, *I, minS, maxS, nMinS, nMaxS);
                        double nAB = 0.0;
                        for (long l = 0, k = 0; l < nMax; ++l, ++k) {
                            if (k >= nMin) k = 0;
                            nAB += std::fmin(pw(cmin, Lmin, smin[k], minS), pw(cmax, Lmax, smax[l], maxS));
                            if (I) perez_prepare_densities(o, *I, cmin[Lmin[smin[k]]], minS, cmax[Lmax[smax[l]]], maxS);
                        }
                        const double n12 = nAB / V;
                        long k = 0;
                        for (long l = 0; l < nMax; ++l) {
                            if (k >= nMin) k = 0;
                            coulomb_collide(o, cmax[Lmax[smax[l]]], maxS, cmin[Lmin[smin[k]]], minS, lD, nMaxS, nMinS,
                                            n12, c, ord, I, &ionized);
                            ++k;
                        }
                        pairs += nMax;
                    }
                }
            }
        }
    }
    if (st) {
        st->coulomb_pairs += pairs;
        st->coulomb_ionizations += ionized;
        st->coulomb_ionization_electrons += (long long)ionizer.electrons.size();
    }
    // the electrons added by ionisations join the cloud after the step
    // (addNewParcel; not in this step's cell lists)
    if (I)
        for (const Parcel& p : ionizer.electrons) o.cloud[o.cfg.electron_species].push_back(p);
}

// PICCloud::buildCellOccupancy (PICCloud.C:327-354) + collisions() (PICCloud.C:526-539):
// Coulomb, then electron-neutral, then ion-neutral.
// BinaryCollisionModel::performCollisions (BinaryCollisionModel.C:229-373):
// per cell, the parcels of the neutral species (species order, then parcel
// order) are split into octant sub-cells around the cell centre; the NTC
// count rem + nC (nC - 1) / 2 * w_max (sigma_T c_r)_max dt / V of
// candidates picks P at random and Q from P's sub-cell when it holds another
// parcel (else from the cell); acceptance sigma_T c_r / (sigma_T c_r)_max
// with the cell's value at the start, the maximum updated as it is exceeded;
// IsotropicScattering (IsotropicScattering.C:67-100) and the weight
// correction.  performBackgroundCollisions (:375-515): rem + nN n_bg
// (sigma_T c_r)_max dt candidates against background velocities
// sqrt(kT/m) N(0,1)^3 + drift (uniformBackground.C:121-127).
double sigma_tcr(const picgpu_binary& bc, double dP, double dQ, double omP, double omQ, double mP, double mQ,
                 double G, const V3& UP, const V3& UQ) {
    const double dPQ = 0.5 * (dP + dQ);
    const V3 g = sub(UP, UQ);
    const double cR = std::sqrt(dotv(g, g));
    if (cR < 1.0e-300) return 0.0;  // vSmall
    double sig;
    if (bc.cross_section == PICGPU_XS_VARIABLE_HARD_SPHERE) {
        const double omPQ = 0.5 * (omP + omQ);
        const double mR = mP * mQ / (mP + mQ);
        sig = kPi * dPQ * dPQ * std::pow(2.0 * kBoltzmann * bc.tref / (mR * cR * cR), omPQ - 0.5) / G;
    } else {
        sig = kPi * dPQ * dPQ;
    }
    return sig * cR;
}

void iso_scatter(double mP, double mQ, V3& UP, V3& UQ, ocoll::Philox& r) {
    const double M = mP + mQ;
    const V3 Ucm = v3((mP * UP.x + mQ * UQ.x) / M, (mP * UP.y + mQ * UQ.y) / M, (mP * UP.z + mQ * UQ.z) / M);
    const V3 g = sub(UP, UQ);
    const double cR = std::sqrt(dotv(g, g));
    const double cosT = 2.0 * r.uniform() - 1.0;
    const double sinT = std::sqrt(1.0 - cosT * cosT);
    const double phi = 6.283185307179586 * r.uniform();
    const V3 pr = v3(cR * cosT, cR * (sinT * std::cos(phi)), cR * (sinT * std::sin(phi)));
    UP = v3(Ucm.x + pr.x * mQ / M, Ucm.y + pr.y * mQ / M, Ucm.z + pr.z * mQ / M);
    UQ = v3(Ucm.x - pr.x * mP / M, Ucm.y - pr.y * mP / M, Ucm.z - pr.z * mP / M);
}

void weight_correct_pair(int model, double wP, double wQ, double mP, double mQ, const V3& preP, const V3& preQ,
                         V3& UP, V3& UQ, ocoll::Philox& r) {
    if (model == 1) {
        const double u = r.uniform();
        if (u > wP / wQ) UQ = preQ;
        if (u > wQ / wP) UP = preP;
    } else if (model == 2 || model == 3) {
        if (wP > wQ) {
            if (model == 3) sentoku_kemp(mP, wQ / wP, preP, UP, r);
            else sentoku_kemp_nr(mP, wQ / wP, preP, UP, r);
        } else if (wP < wQ) {
            if (model == 3) sentoku_kemp(mQ, wP / wQ, preQ, UQ, r);
            else sentoku_kemp_nr(mQ, wP / wQ, preQ, UQ, r);
        }
    }
}

void binary_collisions(Oracle& o, const std::vector<std::vector<std::vector<int>>>& occ, picgpu_step_stats* st) {
    const picgpu_binary& bc = o.cfg.binary;
    const HexMesh& m = o.m;
    const int nc = m.n_cells;
    std::vector<int> ns;
    for (int s = 0; s < o.cfg.n_species; ++s)
        if (o.cfg.species[s].charge == 0.0) ns.push_back(s);
    if (ns.empty()) return;
    if (o.bsmax.empty()) {
        double smax = bc.sigma_tcr_max_init;
        if (!(smax > 0)) {
            const int sp = bc.background_species >= 0 ? bc.background_species : ns[0];
            const double T = bc.init_temperature > 0 ? bc.init_temperature : 293.15;
            const double d = bc.diameter[sp];
            smax = kPi * d * d * std::sqrt(2.0 * kBoltzmann * T / o.cfg.species[sp].mass);
        }
        o.bsmax.assign(nc, smax);
        o.brem.resize(nc);
        o.bbgrem.resize(nc);
        for (int c = 0; c < nc; ++c) {
            ocoll::Philox r0(o.cfg.seed, ocoll::kStreamBinaryRemainder, uint32_t(c), 0u);
            o.brem[c] = r0.uniform();
            ocoll::Philox r1(o.cfg.seed, ocoll::kStreamBinaryBgRemainder, uint32_t(c), 0u);
            o.bbgrem[c] = r1.uniform();
        }
    }
    const int K = int(ns.size());
    double G[PICGPU_MAX_SPECIES][PICGPU_MAX_SPECIES], Gbg[PICGPU_MAX_SPECIES];
    for (int a = 0; a < K; ++a)
        for (int b = 0; b < K; ++b) G[a][b] = std::exp(std::lgamma(2.5 - 0.5 * (bc.omega[ns[a]] + bc.omega[ns[b]])));
    const int bs = bc.background_species;
    const bool bg = bs >= 0 && o.cfg.mcc.gas_density > 0;
    for (int a = 0; a < K; ++a) Gbg[a] = bg ? std::exp(std::lgamma(2.5 - 0.5 * (bc.omega[ns[a]] + bc.omega[bs]))) : 1.0;
    long long tested = 0, collided = 0, btested = 0, bcollided = 0;
    const double dt = o.cfg.dt;
    for (int c = 0; c < nc; ++c) {
        std::vector<std::pair<int, int>> list;  // (neutral species k, parcel index)
        double wmax = 0.0;
        for (int a = 0; a < K; ++a) {
            for (int i : occ[ns[a]][c]) list.emplace_back(a, i);
            if (!occ[ns[a]][c].empty() && o.cfg.species[ns[a]].weight > wmax) wmax = o.cfg.species[ns[a]].weight;
        }
        const int nC = int(list.size());
        auto vel = [&](int j) -> V3& { return o.cloud[ns[list[j].first]][list[j].second].U; };
        if (nC > 1) {
            std::vector<int> sub[8], which(nC);
            for (int j = 0; j < nC; ++j) {
                const Parcel& p = o.cloud[ns[list[j].first]][list[j].second];
                const double* off = &m.cls_offset[size_t(m.cell_class[c]) * 24];
                double rel[3];
                for (int q = 0; q < 3; ++q)
                    rel[q] = p.y[1] * off[3 * m.tt.tri[p.tet][0] + q] + p.y[2] * off[3 * m.tt.tri[p.tet][1] + q] +
                             p.y[3] * off[3 * m.tt.tri[p.tet][2] + q];
                const int oc = (rel[0] >= 0.0 ? 1 : 0) + (rel[1] >= 0.0 ? 2 : 0) + (rel[2] >= 0.0 ? 4 : 0);
                sub[oc].push_back(j);
                which[j] = oc;
            }
            const double smax0 = o.bsmax[c];
            const double sel = o.brem[c] + 0.5 * double(nC) * double(nC - 1) * wmax * smax0 * dt / m.vol[c];
            const long long nCand = (long long)sel;
            o.brem[c] = sel - double(nCand);
            ocoll::Philox r(o.cfg.seed, ocoll::kStreamBinary, uint32_t(c), uint32_t(o.step_index));
            for (long long q = 0; q < nCand; ++q) {
                const int P = int(r.uniform() * double(nC));
                const std::vector<int>& S = sub[which[P]];
                const int nSC = int(S.size());
                int Q = P;
                for (int it = 0; it < 1000 && Q == P; ++it) {
                    if (nSC > 1) Q = S[int(r.uniform() * double(nSC))];
                    else Q = int(r.uniform() * double(nC));
                }
                if (Q == P) continue;
                const int a = list[P].first, b = list[Q].first;
                const int sa = ns[a], sb = ns[b];
                V3& UP = vel(P);
                V3& UQ = vel(Q);
                const double mP = o.cfg.species[sa].mass, mQ = o.cfg.species[sb].mass;
                const double sTcR = sigma_tcr(bc, bc.diameter[sa], bc.diameter[sb], bc.omega[sa], bc.omega[sb], mP,
                                              mQ, G[a][b], UP, UQ);
                ++tested;
                if (sTcR > o.bsmax[c]) o.bsmax[c] = sTcR;
                if (sTcR / smax0 > r.uniform()) {
                    const V3 preP = UP, preQ = UQ;
                    iso_scatter(mP, mQ, UP, UQ, r);
                    weight_correct_pair(bc.weight_correction, o.cfg.species[sa].weight, o.cfg.species[sb].weight,
                                        mP, mQ, preP, preQ, UP, UQ, r);
                    ++collided;
                }
            }
        }
        if (bg && nC > 0) {
            const double smaxb = o.bsmax[c];
            const double coll = o.bbgrem[c] + double(nC) * o.cfg.mcc.gas_density * smaxb * dt;
            const long long nCand = (long long)coll;
            o.bbgrem[c] = coll - double(nCand);
            ocoll::Philox r(o.cfg.seed, ocoll::kStreamBinaryBg, uint32_t(c), uint32_t(o.step_index));
            const double mb = o.cfg.species[bs].mass;
            const double vth = std::sqrt(kBoltzmann * o.cfg.mcc.gas_temperature / mb);
            for (long long q = 0; q < nCand; ++q) {
                const int P = int(r.uniform() * double(nC));
                const int a = list[P].first, sa = ns[a];
                V3& UP = vel(P);
                const double n0 = r.normal(), n1 = r.normal(), n2 = r.normal();
                V3 Ub = v3(vth * n0 + o.cfg.mcc.gas_velocity[0], vth * n1 + o.cfg.mcc.gas_velocity[1],
                           vth * n2 + o.cfg.mcc.gas_velocity[2]);
                const double mP = o.cfg.species[sa].mass;
                const double sTcR = sigma_tcr(bc, bc.diameter[sa], bc.diameter[bs], bc.omega[sa], bc.omega[bs], mP,
                                              mb, Gbg[a], UP, Ub);
                ++btested;
                if (sTcR > o.bsmax[c]) o.bsmax[c] = sTcR;
                if (sTcR / smaxb > r.uniform()) {
                    iso_scatter(mP, mb, UP, Ub, r);
                    ++bcollided;
                }
            }
        }
    }
    if (st) {
        st->binary_candidates += tested;
        st->binary_collisions += collided;
        st->binary_background_candidates += btested;
        st->binary_background_collisions += bcollided;
    }
}

void collisions(Oracle& o, picgpu_step_stats* st) {
    if (!o.cfg.mcc.enabled && !o.cfg.coulomb.enabled && !o.cfg.ion_mcc.enabled && !o.cfg.binary.enabled) return;
    std::vector<std::vector<std::vector<int>>> occ(o.cfg.n_species,
                                                   std::vector<std::vector<int>>(o.m.n_cells));
    for (int s = 0; s < o.cfg.n_species; ++s)
        for (size_t i = 0; i < o.cloud[s].size(); ++i) occ[s][o.cloud[s][i].cell].push_back(int(i));
    if (o.cfg.coulomb.enabled) coulomb_pairs(o, occ, st);
    if (o.cfg.mcc.enabled && o.cfg.mcc.neutral_parcels) mcc_parcels(o, occ, st);
    if (o.cfg.mcc.enabled) mcc_background(o, occ[o.cfg.electron_species], st);
    if (o.cfg.ion_mcc.enabled && o.cfg.ion_mcc.neutral_parcels) ion_parcels(o, occ, st);
    if (o.cfg.ion_mcc.enabled) ion_mcc_background(o, occ[o.cfg.ion_mcc.ion_species], st);
    if (o.cfg.binary.enabled) binary_collisions(o, occ, st);
}


// PairMerging::mergeParticles (PIC/submodels/ParticleMerging/PairMerging/
// PairMerging.C:71-259), cell by cell for each listed species, over the
// parcels of the step's cell occupancy.  Kept as picFoam has it: the speeds
// in the acceptance tests are those of the LIST positions pId1 / pId2 (not
// of the parcels they select, and not shifted after a merge), a pair whose
// velocities are closer in angle than angleDifference is rejected, and the
// merged parcel (addNewParcel) gets charge modifier 1.  The speed order is
// made total by the list position (std::sort's order of equal speeds is
// unspecified); the parcel draw sampleAB(0, N) takes floor(u N) from the
// stream (seed, merge-list entry, cell, step).
void merge_parcels(Oracle& o, picgpu_step_stats* st) {
    const picgpu_merging& mg = o.cfg.merging;
    const double cos_angle = std::cos(mg.angle_difference * kPi / 180.0);
    long long merged_total = 0, checked_total = 0;
    double kin_total = 0.0;
    for (int li = 0; li < mg.n_species; ++li) {
        const int s = mg.species[li];
        auto& cl = o.cloud[s];
        const double wS = o.cfg.species[s].weight, mass = o.cfg.species[s].mass;
        const long nocc = std::min<long>(size_t(s) < o.occ_n.size() ? o.occ_n[s] : 0, long(cl.size()));
        std::vector<std::vector<int>> occ(o.m.n_cells);
        for (long i = 0; i < nocc; ++i) occ[cl[i].cell].push_back(int(i));
        std::vector<char> dead(cl.size(), 0);
        std::vector<Parcel> added;
        auto pw = [&](int i) { return cl[i].nw < 0.0 ? wS : cl[i].nw; };
        for (int c = 0; c < o.m.n_cells; ++c) {
            const std::vector<int>& L = occ[c];
            int N = int(L.size());
            if (N <= mg.cell_parcels_max) continue;
            int nTarget = int(double(N) * mg.reduction_factor);
            if (N - nTarget > mg.merge_maximum_per_cell) nTarget = N - mg.merge_maximum_per_cell;
            std::vector<double> speed(N);
            std::vector<int> sel(N);
            for (int k = 0; k < N; ++k) {
                speed[k] = magv(cl[L[k]].U);
                sel[k] = k;
            }
            std::sort(sel.begin(), sel.end(),
                      [&](int a, int b) { return speed[a] < speed[b] || (speed[a] == speed[b] && a < b); });
            ocoll::Philox rng(o.cfg.seed, ocoll::kStreamMerge | uint32_t(li), uint32_t(c), uint32_t(o.step_index));
            int checks = 0;
            while (N > nTarget) {
                int pId1 = int(rng.uniform() * double(N));
                if (pId1 >= N) pId1 = N - 1;
                const int i1 = L[sel[pId1]];
                int pId2 = pId1 - mg.n_check_neighbors / 2;
                if (pId2 < 0) pId2 = 0;
                if (pId2 + mg.n_check_neighbors > N - 1) pId2 = N - mg.n_check_neighbors - 1;
                if (pId2 < 0) pId2 = 0;
                int found = -1;
                for (int k = 0; k < mg.n_check_neighbors; ++k) {
                    if (pId2 == pId1) pId2++;
                    if (pId2 >= N) break;
                    const int i2 = L[sel[pId2]];
                    checked_total++;
                    if (mg.n_deviation[li] - std::fabs(pw(i2) - pw(i1)) < 0.0) { pId2++; continue; }
                    if (cl[i2].zq != cl[i1].zq) { pId2++; continue; }
                    const V3 U1 = cl[i1].U, U2 = cl[i2].U;
                    if (U2.x * U1.x + U2.y * U1.y + U2.z * U1.z > speed[pId2] * speed[pId1] * cos_angle) {
                        pId2++;
                        continue;
                    }
                    double ratio = speed[pId2] / speed[pId1];
                    if (ratio > 1.0) ratio = 1.0 / ratio;
                    if (ratio < mg.velocity_ratio) { pId2++; continue; }
                    found = pId2;
                    break;
                }
                if (found >= 0) {
                    pId2 = found;
                    const int i2 = L[sel[pId2]];
                    const double n1 = pw(i1), n2 = pw(i2), nSum = n1 + n2;
                    const V3 x1 = position_of(o, cl[i1]), x2 = position_of(o, cl[i2]);
                    const V3 U1 = cl[i1].U, U2 = cl[i2].U;
                    const double com[3] = {(n1 * x1.x + n2 * x2.x) / nSum, (n1 * x1.y + n2 * x2.y) / nSum,
                                           (n1 * x1.z + n2 * x2.z) / nSum};
                    const V3 nU = v3((n1 * U1.x + n2 * U2.x) / nSum, (n1 * U1.y + n2 * U2.y) / nSum,
                                     (n1 * U1.z + n2 * U2.z) / nSum);
                    const double pre = 0.5 * mass *
                                       ((U1.x * U1.x + U1.y * U1.y + U1.z * U1.z) * n1 +
                                        (U2.x * U2.x + U2.y * U2.y + U2.z * U2.z) * n2);
                    const double post = 0.5 * mass * (nU.x * nU.x + nU.y * nU.y + nU.z * nU.z) * nSum;
                    kin_total += post - pre;
                    Parcel p;
                    double y[3];
                    const long long tg = om::locate_in_cell(o.m, c, com, y);
                    p.cell = int(tg / 12);
                    p.tet = int(tg % 12);
                    p.y[1] = y[0];
                    p.y[2] = y[1];
                    p.y[3] = y[2];
                    p.y[0] = 1.0 - y[0] - y[1] - y[2];
                    p.U = nU;
                    p.nw = nSum;
                    p.zq = 1;
                    added.push_back(p);
                    dead[i1] = dead[i2] = 1;
                    merged_total++;
                    const int minPos = std::min(pId1, pId2), maxPos = std::max(pId1, pId2);
                    for (int k = minPos; k < N - 2; ++k) sel[k] = k >= maxPos - 1 ? sel[k + 2] : sel[k + 1];
                    N -= 2;
                }
                checks++;
                if (checks > mg.max_checks) break;
            }
        }
        size_t w = 0;
        for (size_t i = 0; i < cl.size(); ++i)
            if (!dead[i]) cl[w++] = cl[i];
        cl.resize(w);
        for (const Parcel& p : added) cl.push_back(p);
    }
    if (st) {
        st->merged_parcels += merged_total;
        st->merge_checks += checked_total;
        st->merge_kinetic_energy_error += kin_total;
    }
}

void fill_counts(const Oracle& o, picgpu_step_stats* st) {
    if (!st) return;
    for (size_t s = 0; s < o.cloud.size(); ++s) st->n_particles[s] = (long long)o.cloud[s].size();
    for (size_t pa = 0; pa < o.m.patches.size() && pa < PICGPU_MAX_BOXES + 6; ++pa)
        st->floating_charge[pa] = o.sigma[pa] * o.m.patches[pa].area;
    if (o.cfg.circuit.model != PICGPU_CIRCUIT_NONE) {
        st->circuit_voltage = o.circuit.voltage;
        st->circuit_current = o.circuit.current;
        st->circuit_cathode_current = o.circuit.cathode_current;
        st->circuit_charge = o.circuit.charge;
    }
}

}  // namespace

// ------------------------------------------------ initial conditions -----
// picInitialise (preProcess/picInitialise/picInitialise.C:30-319) with the
// InitializationModel sub-models Equipartition
// (EquipartitionInitialization.C:65-141), Maxwellian
// (MaxwellianInitialization.C:73-126), Isotropization
// (IsotropizationInitialization.C:52-123), QuasineutralPlasma
// (QuasineutralPlasmaInitialization.C:38-175) and UniformDisplacement
// (UniformInitialization.C:51-127).  Within a species the particles are added
// in picFoam's order (cell, tet, particle; or cell, particle; or the lattice
// order i, j, k).  picFoam draws every number from one sequential
// Foam::Random; here each tet (cell, lattice point) of each species has its
// own Philox stream, so the CUDA kernels can place the particles in parallel
// and still draw the same numbers.  Normal variates: Marsaglia's polar
// method; the logarithm and the sine are evaluated in fixed FP64 operations
// (atanh series after frexp, Taylor series after reduction by pi) so that no
// math library enters the result.  Points in a tet: the cube-folding method
// of Rocchini & Cignoni (J. Graphics Tools 5(4), 2000).
namespace oinit {

double det_log(double x) {
    int e;
    double m = std::frexp(x, &e);
    if (m < 0.70710678118654752440) {
        m = m * 2.0;
        e = e - 1;
    }
    const double z = (m - 1.0) / (m + 1.0);
    const double w = z * z;
    const double inv_odd[11] = {1.0 / 23.0, 1.0 / 21.0, 1.0 / 19.0, 1.0 / 17.0, 1.0 / 15.0, 1.0 / 13.0,
                                1.0 / 11.0, 1.0 / 9.0,  1.0 / 7.0,  1.0 / 5.0,  1.0 / 3.0};
    double p = inv_odd[0];
    for (int i = 1; i < 11; ++i) p = p * w + inv_odd[i];
    const double lm = 2.0 * z + 2.0 * z * (w * p);
    return double(e) * 0.69314718055994530942 + lm;
}

double det_sin(double x) {
    const double pi_hi = 3.141592653589793116, pi_lo = 1.2246467991473532e-16;
    const double k = std::rint(x / pi_hi);
    const double r = (x - k * pi_hi) - k * pi_lo;
    const double w = r * r;
    // -1/23!, 1/21!, ..., -1/3!
    const double c[11] = {-1.0 / 25852016738884976640000.0, 1.0 / 51090942171709440000.0,
                          -1.0 / 121645100408832000.0,      1.0 / 355687428096000.0,
                          -1.0 / 1307674368000.0,           1.0 / 6227020800.0,
                          -1.0 / 39916800.0,                1.0 / 362880.0,
                          -1.0 / 5040.0,                    1.0 / 120.0,
                          -1.0 / 6.0};
    double p = c[0];
    for (int i = 1; i < 11; ++i) p = p * w + c[i];
    const double s = r + r * (w * p);
    return ((long long)k & 1) ? -s : s;
}

double det_exp(double x) {
    const double ln2_hi = 0.6931471805599452862, ln2_lo = 2.3190468138462996e-17;
    const double k = std::rint(x / ln2_hi);
    const double r = (x - k * ln2_hi) - k * ln2_lo;
    // 1/17!, 1/16!, ..., 1/2!, 1/1!, 1/0!
    const double c[18] = {1.0 / 355687428096000.0, 1.0 / 20922789888000.0, 1.0 / 1307674368000.0,
                          1.0 / 87178291200.0,     1.0 / 6227020800.0,     1.0 / 479001600.0,
                          1.0 / 39916800.0,        1.0 / 3628800.0,        1.0 / 362880.0,
                          1.0 / 40320.0,           1.0 / 5040.0,           1.0 / 720.0,
                          1.0 / 120.0,             1.0 / 24.0,             1.0 / 6.0,
                          0.5,                     1.0,                    1.0};
    double p = c[0];
    for (int i = 1; i < 18; ++i) p = p * r + c[i];
    return std::ldexp(p, int(k));
}

void polar_pair(ocoll::Philox& r, double& n1, double& n2) {
    for (int a = 0; a < 64; ++a) {
        const double u1 = 2.0 * r.uniform() - 1.0;
        const double u2 = 2.0 * r.uniform() - 1.0;
        const double s = u1 * u1 + u2 * u2;
        if (s > 0.0 && s < 1.0) {
            const double f = std::sqrt(-2.0 * det_log(s) / s);
            n1 = u1 * f;
            n2 = u2 * f;
            return;
        }
    }
    n1 = n2 = 0.0;
}

// sampleNormal<vector>
V3 normal3(ocoll::Philox& r) {
    double a, b, c, d;
    polar_pair(r, a, b);
    polar_pair(r, c, d);
    return v3(a, b, c);
}

// tetPointRef::randomPoint as barycentric coordinates 1..3 of the tet
void tet_point(ocoll::Philox& r, double* y) {
    double s = r.uniform(), t = r.uniform(), u = r.uniform();
    if (s + t > 1.0) {
        s = 1.0 - s;
        t = 1.0 - t;
    }
    if (t + u > 1.0) {
        const double tmp = u;
        u = 1.0 - s - t;
        t = 1.0 - tmp;
    } else if (s + t + u > 1.0) {
        const double tmp = u;
        u = s + t + u - 1.0;
        s = 1.0 - t - tmp;
    }
    y[0] = s;
    y[1] = t;
    y[2] = u;
}

// The tet of cell c holding x (largest smallest coordinate), clamped and
// renormalised coordinates; false when x is outside by more than 1e-9.
bool locate_in_cell(const HexMesh& m, int c, const double* x, int& tet, double* y) {
    double best_min = -1e300, by[3] = {0, 0, 0};
    int best = -1;
    for (int t = 0; t < 12; ++t) {
        double q[3];
        om::tet_coords(m, c, t, x, q);
        const double q0 = 1.0 - q[0] - q[1] - q[2];
        const double mn = std::fmin(std::fmin(q0, q[0]), std::fmin(q[1], q[2]));
        if (mn > best_min) {
            best_min = mn;
            best = t;
            by[0] = q[0];
            by[1] = q[1];
            by[2] = q[2];
        }
    }
    if (best_min < -1e-9) return false;
    const double y0 = 1.0 - by[0] - by[1] - by[2];
    const double yy[4] = {std::fmax(y0, 0.0), std::fmax(by[0], 0.0), std::fmax(by[1], 0.0), std::fmax(by[2], 0.0)};
    const double s = yy[0] + yy[1] + yy[2] + yy[3];
    for (int a = 0; a < 3; ++a) y[a] = yy[a + 1] / s;
    tet = best;
    return true;
}

// meshTools::constrainDirection(mesh, solutionD, p): the point's components
// along empty axes become zero; the point is then located in its cell again.
bool constrain(const HexMesh& m, int c, int& t, double* y) {
    const double* off = &m.cls_offset[size_t(m.cell_class[c]) * 24];
    double x[3];
    for (int a = 0; a < 3; ++a)
        x[a] = m.cc[3 * size_t(c) + a] + y[0] * off[3 * m.tt.tri[t][0] + a] + y[1] * off[3 * m.tt.tri[t][1] + a] +
               y[2] * off[3 * m.tt.tri[t][2] + a];
    for (int a = 0; a < 3; ++a)
        if (m.empty[a]) x[a] = 0.0;
    return locate_in_cell(m, c, x, t, y);
}

struct Sampling {
    double n = 0, w = 1, scale[3] = {0, 0, 0}, drift[3] = {0, 0, 0}, speed = 0, displacement = 0;
    long long cell_count = 0;
    bool place = false;
};

Parcel make_parcel(int c, int t, const double* y, V3 U) {
    Parcel p;
    p.cell = c;
    p.tet = t;
    p.y[1] = y[0];
    p.y[2] = y[1];
    p.y[3] = y[2];
    p.y[0] = 1.0 - p.y[1] - p.y[2] - p.y[3];
    p.U = U;
    return p;
}

V3 velocity(const Sampling& q, ocoll::Philox& r) {
    const V3 n = normal3(r);
    return v3(q.scale[0] * n.x + q.drift[0], q.scale[1] * n.y + q.drift[1], q.scale[2] * n.z + q.drift[2]);
}

}  // namespace oinit

int oracle_initialise_impl(Oracle& o, const picgpu_init* in, picgpu_init_stats* out) {
    using namespace oinit;
    const HexMesh& m = o.m;
    const int ns = o.cfg.n_species, nc = m.n_cells;
    if (in->model < PICGPU_INIT_NONE || in->model > PICGPU_INIT_UNIFORM_DISPLACEMENT) {
        o.err = "initialise: unknown InitializationModel";
        return PICGPU_INVALID_ARG;
    }
    picgpu_init_stats S{};
    if (in->clear_particles)
        for (auto& cl : o.cloud) cl.clear();
    Sampling smp[PICGPU_MAX_SPECIES];
    bool calc_T = false, calc_n = false;
    for (int sp = 0; sp < ns; ++sp) {
        const picgpu_species& P = o.cfg.species[sp];
        Sampling& q = smp[sp];
        q.n = in->number_density[sp];
        q.w = P.weight;
        // equipartitionLinearVelocity (PICCloud.C:1506-1515): sqrt(kT/m) N(0,1)^3
        const double th = std::sqrt(kBoltzmann * in->temperature[sp] / P.mass);
        switch (in->model) {
            case PICGPU_INIT_EQUIPARTITION:  // EquipartitionInitialization.C:128-135: + velocity
                for (int a = 0; a < 3; ++a) { q.scale[a] = th; q.drift[a] = in->velocity[a]; }
                q.place = q.n > 0;
                break;
            case PICGPU_INIT_MAXWELLIAN:  // MaxwellianInitialization.C:112-119
                for (int a = 0; a < 3; ++a) {
                    q.scale[a] = in->thermal_velocity[sp][a];
                    q.drift[a] = in->drift_velocity[sp][a];
                }
                q.place = q.n > 0;
                calc_T = true;
                break;
            case PICGPU_INIT_ISOTROPIZATION: {  // IsotropizationInitialization.C:95-110
                const double f = in->tperp_over_tpara;
                if (!(f > 0)) { o.err = "initialise: Tperp_over_Tpara must be > 0"; return PICGPU_INVALID_ARG; }
                const double T = in->temperature[sp];
                q.scale[0] = std::sqrt(kBoltzmann * T / (((2.0 / 3.0) * f + (1.0 / 3.0)) * P.mass));
                q.scale[1] = std::sqrt(kBoltzmann * T / (((2.0 / 3.0) + (1.0 / (3.0 * f))) * P.mass));
                q.scale[2] = q.scale[1];
                q.place = q.n > 0;
                break;
            }
            case PICGPU_INIT_QUASINEUTRAL_PLASMA:
                for (int a = 0; a < 3; ++a) q.scale[a] = th;
                q.speed = std::sqrt(in->temperature[sp] * kBoltzmann * 3.0 / P.mass);
                calc_n = true;
                break;
            case PICGPU_INIT_UNIFORM_DISPLACEMENT:
                for (int a = 0; a < 3; ++a) q.scale[a] = th;
                q.displacement = in->displacement[sp];
                q.place = (in->species_mask >> sp) & 1;
                calc_n = true;
                break;
            default:
                calc_T = calc_n = true;
                break;
        }
    }
    if (in->model == PICGPU_INIT_QUASINEUTRAL_PLASMA) {
        // QuasineutralPlasmaInitialization.C:38-80
        const int ion = in->ion_species, el = o.cfg.electron_species;
        if (ion < 0 || ion >= ns || el < 0 || el >= ns) { o.err = "initialise: species"; return PICGPU_INVALID_ARG; }
        if (o.cfg.species[ion].charge + o.cfg.species[el].charge != 0.0) {
            o.err = "initialise: ion and electron charge must be of same magnitude and opposite signs";
            return PICGPU_INVALID_ARG;
        }
        for (int sp : {ion, el}) {
            smp[sp].cell_count = (long long)(in->cell_count / o.cfg.species[sp].weight);
            smp[sp].place = smp[sp].cell_count > 0;
        }
    }
    const bool cons = m.empty[0] || m.empty[1] || m.empty[2];
    for (int sp = 0; sp < ns && in->model != PICGPU_INIT_NONE; ++sp) {
        const Sampling& q = smp[sp];
        if (!q.place) continue;
        auto& cl = o.cloud[sp];
        const size_t before = cl.size();
        if (in->model == PICGPU_INIT_QUASINEUTRAL_PLASMA) {
            // QuasineutralPlasmaInitialization.C:102-175
            for (int c = 0; c < nc; ++c)
                for (long long k = 0; k < q.cell_count; ++k) {
                    ocoll::Philox r(in->seed, ocoll::kStreamInitParticle | uint32_t(sp), uint32_t(c), uint32_t(k));
                    int t = int((12.0 - 1.0) * r.uniform());  // label((cellTets.size()-1.0)*scalar01())
                    double y[3];
                    tet_point(r, y);
                    if (cons && !constrain(m, c, t, y)) { o.err = "initialise: point left its cell"; return PICGPU_INVALID_ARG; }
                    V3 U;
                    if (in->use_maxwellian) {
                        U = velocity(q, r);
                    } else {
                        const double d0 = r.uniform(), d1 = r.uniform(), d2 = r.uniform();
                        const double inv = 1.0 / std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                        U = v3((d0 * inv) * q.speed, (d1 * inv) * q.speed, (d2 * inv) * q.speed);
                    }
                    cl.push_back(make_parcel(c, t, y, U));
                }
        } else if (in->model == PICGPU_INIT_UNIFORM_DISPLACEMENT) {
            // UniformInitialization.C:60-125
            double lo[3], hi[3], dir[3], span[3], delta[3];
            const int gtop = om::grid_point_id(m, m.n[0], m.n[1], m.n[2]);
            for (int a = 0; a < 3; ++a) {
                lo[a] = in->use_bounds ? in->min[a] : m.grid_pts[a];
                hi[a] = in->use_bounds ? in->max[a] : m.grid_pts[3 * size_t(gtop) + a];
            }
            const double dm = std::sqrt(in->displacement_dir[0] * in->displacement_dir[0] +
                                        in->displacement_dir[1] * in->displacement_dir[1] +
                                        in->displacement_dir[2] * in->displacement_dir[2]);
            for (int a = 0; a < 3; ++a) dir[a] = in->displacement_dir[a] / dm;
            for (int a = 0; a < 3; ++a) span[a] = hi[a] - lo[a];
            const double span_len = span[0] * dir[0] + span[1] * dir[1] + span[2] * dir[2];
            for (int a = 0; a < 3; ++a)
                delta[a] = span[a] / double(std::max<long long>(in->particle_numbers[a] - 1, 2));
            const long long nx = in->particle_numbers[0], ny = in->particle_numbers[1], nz = in->particle_numbers[2];
            for (long long i = 0; i < nx; ++i)
                for (long long j = 0; j < ny; ++j)
                    for (long long k = 0; k < nz; ++k) {
                        const long long idx = (i * ny + j) * nz + k;
                        const double p[3] = {lo[0] + delta[0] * double(i), lo[1] + delta[1] * double(j),
                                             lo[2] + delta[2] * double(k)};
                        const double dist = (p[0] - lo[0]) * dir[0] + (p[1] - lo[1]) * dir[1] + (p[2] - lo[2]) * dir[2];
                        const double cur = q.displacement * det_sin(dist / span_len * in->cycles * 3.141592653589793116);
                        double x[3];
                        for (int a = 0; a < 3; ++a) x[a] = p[a] + dir[a] * cur;
                        double by[3];
                        const long long tg = om::locate(m, x, by);  // mesh.findCell
                        if (tg < 0) { o.err = "initialise: tried to create a particle outside of the mesh"; return PICGPU_INVALID_ARG; }
                        int t = 0;
                        double y[3];
                        if (!locate_in_cell(m, int(tg / 12), x, t, y)) { o.err = "initialise: locate"; return PICGPU_INVALID_ARG; }
                        ocoll::Philox r(in->seed, ocoll::kStreamInitLattice | uint32_t(sp), uint32_t(idx >> 32), uint32_t(idx));
                        cl.push_back(make_parcel(int(tg / 12), t, y, velocity(q, r)));
                    }
        } else {
            // per-tet models: particlesRequired = n V / w, floor plus one with
            // probability of the remainder
            for (int c = 0; c < nc; ++c)
                for (int t = 0; t < 12; ++t) {
                    const double V = om::tet_volume(m, m.cell_class[c], t);
                    const double req = (q.n * V) / q.w;
                    long long cnt = (long long)req;
                    ocoll::Philox rc(in->seed, ocoll::kStreamInitCount | uint32_t(sp), uint32_t(c), uint32_t(t));
                    if (req - double(cnt) > rc.uniform()) ++cnt;
                    if (cnt >= (1LL << 24)) { o.err = "initialise: more than 2^24 particles in one tet"; return PICGPU_CAPACITY; }
                    for (long long k = 0; k < cnt; ++k) {
                        ocoll::Philox r(in->seed, ocoll::kStreamInitParticle | uint32_t(sp), uint32_t(c),
                                        (uint32_t(t) << 24) | uint32_t(k));
                        double y[3];
                        tet_point(r, y);
                        int tt = t;
                        if (cons && !constrain(m, c, tt, y)) { o.err = "initialise: point left its cell"; return PICGPU_INVALID_ARG; }
                        cl.push_back(make_parcel(c, tt, y, velocity(q, r)));
                    }
                }
        }
        S.added[sp] = (long long)(cl.size() - before);
    }

    // statistics (picInitialise.C:86-188)
    double vol = 0, lsum = 0;
    for (int c = 0; c < nc; ++c) {
        vol += m.vol[c];
        lsum += std::cbrt(m.vol[c]);
    }
    S.mesh_volume = vol;
    S.average_cell_size = nc > 0 ? lsum / nc : 0.0;
    for (int sp = 0; sp < ns; ++sp) {
        const picgpu_species& P = o.cfg.species[sp];
        std::vector<long long> occ(nc, 0);
        double N = 0, vs = 0, d[3] = {0, 0, 0};
        for (const Parcel& p : o.cloud[sp]) {
            if (!p.alive) continue;
            occ[p.cell]++;
            N += P.weight;
            d[0] += p.U.x * P.weight;
            d[1] += p.U.y * P.weight;
            d[2] += p.U.z * P.weight;
            vs += dotv(p.U, p.U) * P.weight;
        }
        long long mn = nc > 0 ? (1LL << 62) : 0, mx = 0, sum = 0;
        for (long long v : occ) { mn = std::min(mn, v); mx = std::max(mx, v); sum += v; }
        S.occupancy_min[sp] = mn;
        S.occupancy_max[sp] = mx;
        S.occupancy_avg[sp] = nc > 0 ? double(sum) / nc : 0.0;
        if (N > 0) {
            double dd = 0;
            for (int a = 0; a < 3; ++a) { S.drift[sp][a] = d[a] / N; dd += S.drift[sp][a] * S.drift[sp][a]; }
            S.temperature[sp] = P.mass / (3.0 * kBoltzmann) * (vs / N - dd);
        }
        S.number_density[sp] = vol > 0 ? N / vol : 0.0;
        S.model_temperature[sp] = calc_T ? S.temperature[sp] : in->temperature[sp];
        S.model_number_density[sp] = calc_n ? S.number_density[sp] : in->number_density[sp];
    }
    const double eps0 = 1.0 / (kMu0 * kC * kC);
    double inv_l2 = 0;
    for (int sp = 0; sp < ns; ++sp) {
        const double qq = o.cfg.species[sp].charge, T = S.model_temperature[sp], n = S.model_number_density[sp];
        if (qq == 0.0 || n <= 0.0 || T <= 0.0) continue;
        inv_l2 += n * qq * qq / eps0 / (T * kBoltzmann);
    }
    S.debye_length = inv_l2 > 0 ? std::sqrt(1.0 / inv_l2) : 0.0;
    const int el = o.cfg.electron_species;
    if (el >= 0 && el < ns && S.model_number_density[el] > 0) {
        const double qq = o.cfg.species[el].charge;
        S.plasma_frequency_dt = std::sqrt(S.model_number_density[el] * qq * qq / eps0 / o.cfg.species[el].mass) * o.cfg.dt;
    }
    // calculateFields, solveMaxwellEquations, initalizeLeapFrog (picInitialise.C:209-227)
    calculate_fields(o);
    if (in->solve_fields) {
        const int r = solve_fields(o, nullptr);
        if (r) return r;
    }
    if (in->leapfrog)
        for (int sp = 0; sp < ns; ++sp)
            for (Parcel& p : o.cloud[sp])
                if (p.alive) push(o, p, sp, -0.5 * o.cfg.dt);
    if (out) *out = S;
    return 0;
}

// SimpleInjection::injection (SimpleInjection.C:197-240) before the move:
// frequency / weight * dt parcels per listed species plus the carried
// remainder, each emitted by ParticleEmitter::emitParticle
// (ParticleEmitter.C:265-418) -- area-weighted face triangle, uniform point
// on it, moved U(0.1, 0.5) of the normal distance towards the cell centre,
// velocity model about the inward normal (:420-535), constrainDirection,
// syncVelocityAtBoundary(-0.5) (:401) -- and, on a floating patch, its
// charge taken off the patch (particleEjection, SimpleInjection.C:295-302).
// FreeStream::injection (SM/BoundaryModel/FreeStream/FreeStream.C:126-396):
// per face and species the accumulator gains Bird's eq. 4.22 flux; the
// integer part, plus one when the remainder exceeds a uniform draw, is
// emitted on the face -- a triangle by area share, a uniform point on it, the
// normal speed ratio by acceptance-rejection (eq. 12.5), thermal tangential
// components plus the drift's tangential part -- then
// syncVelocityAtBoundary(-0.5).  Faces in order, each face's parcels in turn.
void freestream_inject(Oracle& o) {
    using namespace oinit;
    for (size_t i = 0; i < o.freestreams.size(); ++i) {
        Oracle::FreeStream& Z = o.freestreams[i];
        const ob::FreeStreamFaces& F = Z.F;
        for (int j = 0; j < Z.cfg.n_species; ++j) {
            const int sp = Z.cfg.species[j];
            const picgpu_species& S = o.cfg.species[sp];
            const uint32_t key = (uint32_t(i) << 4) | uint32_t(sp);
            std::vector<int> counts(F.n_faces);
            for (int f = 0; f < F.n_faces; ++f) {
                const size_t q = size_t(f) * F.n_species + j;
                double a = Z.acc[q] + F.add[q];
                long long n = a < 2.0e9 ? (long long)a : (1LL << 31);
                if (n < 0) n = 0;
                ocoll::Philox r(o.cfg.seed, ocoll::kStreamFreeStreamCount | key, uint32_t(o.step_index), uint32_t(f));
                if (a - double(n) > r.uniform()) ++n;
                if (n > (1LL << 30)) n = 0;
                Z.acc[q] = a - double(n);
                counts[f] = int(n);
            }
            for (int f = 0; f < F.n_faces; ++f) {
                if (counts[f] == 0) continue;
                ocoll::Philox r(o.cfg.seed, ocoll::kStreamFreeStream | key, uint32_t(o.step_index), uint32_t(f));
                const double s = F.s[size_t(f) * F.n_species + j];
                const double root = std::sqrt(s * s + 2.0);
                const double qa = s + root;
                const double qb = 0.5 * (1.0 + s * (s - root));
                const double scaling = s < -3.0 ? std::fabs(s) + 1.0 : 3.0;
                const double* n = &F.n_in[3 * size_t(f)];
                const double* t1 = &F.t1[3 * size_t(f)];
                const double* t2 = &F.t2[3 * size_t(f)];
                const double* Ud = Z.cfg.velocity;
                const double d1 = t1[0] * Ud[0] + t1[1] * Ud[1] + t1[2] * Ud[2];
                const double d2 = t2[0] * Ud[0] + t2[1] * Ud[1] + t2[2] * Ud[2];
                for (int k = 0; k < counts[f]; ++k) {
                    const double sel = r.uniform();
                    const int t = F.tet0[f] + (F.frac0[f] >= sel ? 0 : 1);
                    const double r1 = r.uniform(), r2 = r.uniform();
                    const double sr = std::sqrt(r1);
                    const double y[3] = {1.0 - sr, sr * (1.0 - r2), sr * r2};
                    double u = 0.0;
                    for (int it = 0; it < 10000; ++it) {  // do { ... } while (P < U01)
                        const double ut = scaling * (2.0 * r.uniform() - 1.0);
                        u = ut + s;
                        const double pr = u < 0.0 ? -1.0 : 2.0 * u / qa * det_exp(qb - ut * ut);
                        if (!(pr < r.uniform())) break;
                    }
                    double n1, n2;
                    polar_pair(r, n1, n2);
                    double U[3];
                    for (int a = 0; a < 3; ++a)
                        U[a] = ((F.v_t[j] * (n1 * t1[a] + n2 * t2[a]) + d1 * t1[a]) + d2 * t2[a]) +
                               F.c_mp[j] * u * n[a];
                    Parcel p = make_parcel(F.cell[f], t, y, v3(U[0], U[1], U[2]));
                    if (o.cfg.sync_velocity_at_boundary && S.charge != 0.0 && o.cfg.pusher != PICGPU_PUSHER_NONE)
                        push(o, p, sp, -0.5 * o.cfg.dt);
                    o.cloud[sp].push_back(p);
                }
            }
        }
    }
}

// ParticleEmitter::emitParticle for n parcels of species sp from the
// patch's face triangles T (the RNG stream of emitter `index`), with the
// floating / circuit patch charge taken off first.
void emit_parcels(Oracle& o, const PatchTriangles& T, int index, int patch, int sp, long long n, int model,
                  double temperature) {
    using namespace oinit;
    const HexMesh& m = o.m;
    const double dt = o.cfg.dt;
    const bool cons = m.empty[0] || m.empty[1] || m.empty[2];
    const picgpu_species& S = o.cfg.species[sp];
    const int ntri = int(T.cell.size());
    const int pk = m.patches[patch].p.kind;
    if (pk == PICGPU_PATCH_FLOATING || pk == PICGPU_PATCH_CIRCUIT)
        o.Qconv[patch] = o.Qconv[patch] - double(n) * S.charge * S.weight;
    for (long long k = 0; k < n; ++k) {
        ocoll::Philox r(o.cfg.seed, ocoll::kStreamInject | (uint32_t(index) << 4) | uint32_t(sp),
                        uint32_t(o.step_index), uint32_t(k));
        const double af = r.uniform() * T.area;
        int tri = 0;
        for (int q = ntri - 1; q >= 0; --q)
            if (af > T.cum[q]) { tri = q; break; }
        const int c = T.cell[tri], tt = T.tet[tri];
        const double* off = &m.cls_offset[size_t(m.cell_class[c]) * 24];
        const double* cc = &m.cc[3 * size_t(c)];
        double A[3], B[3], Cc[3];
        for (int a = 0; a < 3; ++a) {
            A[a] = cc[a] + off[3 * m.tt.tri[tt][0] + a];
            B[a] = cc[a] + off[3 * m.tt.tri[tt][1] + a];
            Cc[a] = cc[a] + off[3 * m.tt.tri[tt][2] + a];
        }
        // triPointRef::randomPoint: (1 - sqrt r1) A + sqrt r1 (1 - r2) B + sqrt r1 r2 C
        const double r1 = r.uniform(), r2 = r.uniform();
        const double sr = std::sqrt(r1);
        double pf[3];
        for (int a = 0; a < 3; ++a) pf[a] = (1.0 - sr) * A[a] + sr * (1.0 - r2) * B[a] + sr * r2 * Cc[a];
        const double fa = 0.1 + 0.4 * r.uniform();  // scalarAB(0.1, 0.5)
        const double* nrm = &T.normal[3 * size_t(tri)];
        const double dn =
            std::fabs((pf[0] - cc[0]) * nrm[0] + (pf[1] - cc[1]) * nrm[1] + (pf[2] - cc[2]) * nrm[2]);
        double x[3];
        for (int a = 0; a < 3; ++a) x[a] = pf[a] - fa * (dn * nrm[a]);
        const double* fc = &T.centre[3 * size_t(tri)];
        double nn[3], t1[3], t2[3];
        for (int a = 0; a < 3; ++a) {
            nn[a] = -nrm[a];
            t1[a] = fc[a] - A[a];
        }
        const double m1 = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
        for (int a = 0; a < 3; ++a) t1[a] = t1[a] / m1;
        t2[0] = nn[1] * t1[2] - nn[2] * t1[1];
        t2[1] = nn[2] * t1[0] - nn[0] * t1[2];
        t2[2] = nn[0] * t1[1] - nn[1] * t1[0];
        const double m2 = std::sqrt(t2[0] * t2[0] + t2[1] * t2[1] + t2[2] * t2[2]);
        for (int a = 0; a < 3; ++a) t2[a] = t2[a] / m2;
        double U[3];
        const double vt = std::sqrt(kBoltzmann * temperature / S.mass);
        if (model == PICGPU_EMIT_MOST_PROBABLE_SPEED) {
            const double vmp = std::sqrt(2.0 * kBoltzmann * temperature / S.mass);
            for (int a = 0; a < 3; ++a) U[a] = vmp * nn[a];
        } else {
            double n1, n2;
            polar_pair(r, n1, n2);
            double tg[3];
            for (int a = 0; a < 3; ++a) tg[a] = vt * (n1 * t1[a] + n2 * t2[a]);
            double un;
            if (model == PICGPU_EMIT_BIRD_MAXWELLIAN_FLUX) {
                const double vmp = std::sqrt(2.0 * kBoltzmann * temperature / S.mass);
                double u = 0.0;
                for (int it = 0; it < 1000; ++it) {  // do { ... } while (P < U01)
                    u = 3.0 * (2.0 * r.uniform() - 1.0);
                    const double pr = u < 0.0 ? -1.0 : 2.0 * u / 1.4142135623730951 * det_exp(0.5 - u * u);
                    if (!(pr < r.uniform())) break;
                }
                un = vmp * u;
            } else if (model == PICGPU_EMIT_HALF_MAXWELLIAN_FLUX) {
                double n3, n4;
                polar_pair(r, n3, n4);
                un = std::fabs(n3) * vt;
            } else {
                const double R = r.uniform();
                un = vt * std::sqrt(-2.0 * det_log(1.0 - R));
            }
            for (int a = 0; a < 3; ++a) U[a] = tg[a] + un * nn[a];
        }
        for (int a = 0; a < 3; ++a)
            if (cons && m.empty[a]) x[a] = 0.0;
        int tet = 0;
        double y[3] = {0, 0, 0};
        locate_in_cell(m, c, x, tet, y);
        Parcel p = make_parcel(c, tet, y, v3(U[0], U[1], U[2]));
        if (o.cfg.sync_velocity_at_boundary && S.charge != 0.0 && o.cfg.pusher != PICGPU_PUSHER_NONE)
            push(o, p, sp, -0.5 * dt);
        o.cloud[sp].push_back(p);
    }
}

void inject(Oracle& o) {
    using namespace oinit;
    const double dt = o.cfg.dt;
    const double t = double(o.step_index + 1) * dt;
    for (size_t i = 0; i < o.injectors.size(); ++i) {
        Oracle::Injector& I = o.injectors[i];
        if (t > I.cfg.end_time) continue;
        const PatchTriangles& T = I.tri;
        for (int j = 0; j < I.cfg.n_species; ++j) {
            const int sp = I.cfg.species[j];
            const picgpu_species& S = o.cfg.species[sp];
            const double np = I.cfg.frequency[j] / S.weight * dt + I.remainder[j];
            const long long n = (long long)np;
            I.remainder[j] = np - double(n);
            if (n <= 0) continue;
            emit_parcels(o, T, int(i), I.cfg.patch, sp, n, I.cfg.velocity_model,
                         I.cfg.eV[j] * 1.602176634e-19 / kBoltzmann);
        }
    }
    freestream_inject(o);
    // EmissionModels (SM/Helper/Emission): n = J A dt / (w e) + remainder
    for (size_t i = 0; i < o.emitters.size(); ++i) {
        Oracle::Emitter& Z = o.emitters[i];
        const int sp = o.cfg.electron_species;
        const picgpu_species& S = o.cfg.species[sp];
        const double qe = std::fabs(S.charge);
        double j = Z.j;
        double temperature = Z.cfg.temperature;
        if (Z.cfg.model == PICGPU_EMISSION_FOWLER_NORDHEIM) {
            j = ob::lane_sum(int(Z.faces.size()), [&](int k) {
                const int b = Z.faces[k];
                return ob::fowler_nordheim_face(&o.Eb[3 * size_t(b)], o.m.bfaces[b].normal, Z.cfg.work_function);
            });
            temperature = Z.cfg.work_function * qe / kBoltzmann;
        }
        const double ne = j * Z.tri.area * dt / (S.weight * qe) + Z.remainder;
        const long long n = (long long)ne;
        Z.remainder = ne - double(n);
        if (n > 0)
            emit_parcels(o, Z.tri, PICGPU_MAX_INJECTORS + int(i), Z.cfg.patch, sp, n, PICGPU_EMIT_MAXWELLIAN_FLUX,
                         temperature);
    }
}

struct oracle_ctx {
    Oracle o;
};

extern "C" {

// Known-answer checks of the oracle's mesh from first principles; out[k] is
// the worst deviation of check k (all should be at round-off):
//  0 tet volumes summed per cell against the cell volume dx dy dz (relative)
//  1 position(locate(x)) - x over pseudo-random points (per cell size)
//  2 barycentric coordinates of each tet's own vertices against unit vectors
//  3 the Gauss Laplacian of a linear potential in cells without boundary faces
//    (relative to the sum of the coefficients' magnitudes)
//  4 the distance weights of VolumeWeighting summed over the cells at a point, minus 1
//  5 the point-interpolation weights summed per point, minus 1
//  6 the outward face area vectors summed over a cell (closed surface), per face area
//  7 tet moves: crossing a face and crossing back returns the start tet (0 or 1)
// Returns the number of checks, or -1 when the mesh cannot be built.
int oracle_mesh_selfcheck(const picgpu_mesh_desc* desc, double* out, int n_out) {
    om::Mesh m;
    try {
        m = om::build(*desc);
    } catch (const std::exception&) {
        return -1;
    }
    double r[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double h[3], vcell = 1.0;
    for (int a = 0; a < 3; ++a) {
        h[a] = desc->length[a] / desc->n[a];
        vcell *= h[a];
    }
    double vt = 0.0;
    for (int t = 0; t < 12; ++t) vt += om::tet_volume(m, 0, t);
    r[0] = std::fabs(vt - vcell) / vcell;
    uint64_t lcg = 0x9E3779B97F4A7C15ull;
    auto uni = [&lcg]() {
        lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
        return double(lcg >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int k = 0; k < 4000; ++k) {
        double x[3], y[3], back[3];
        for (int a = 0; a < 3; ++a) x[a] = desc->origin[a] + desc->length[a] * (0.001 + 0.998 * uni());
        const long long tet = om::locate(m, x, y);
        if (tet < 0) continue;  // inside a removed box
        om::position(m, tet, y, back);
        for (int a = 0; a < 3; ++a) r[1] = std::fmax(r[1], std::fabs(back[a] - x[a]) / h[a]);
    }
    const double* off = m.cls_offset.data();
    for (int t = 0; t < 12; ++t)
        for (int v = 0; v < 3; ++v) {
            double x[3], y[3];
            for (int a = 0; a < 3; ++a) x[a] = m.cc[a] + off[3 * m.tt.tri[t][v] + a];
            om::tet_coords(m, 0, t, x, y);
            for (int k = 0; k < 3; ++k) r[2] = std::fmax(r[2], std::fabs(y[k] - (k == v ? 1.0 : 0.0)));
        }
    const double g[3] = {0.3, -1.7, 2.9};
    for (int c = 0; c < m.n_cells; ++c) {
        bool inner = true;
        for (int f = 0; f < 6; ++f) {
            const int nb = m.nbr[6 * size_t(c) + f];
            // a coupled face that wraps (cyclic) does not see a linear field
            if (nb < 0 || std::abs(m.cell_ijk[3 * size_t(nb) + f / 2] - m.cell_ijk[3 * size_t(c) + f / 2]) != 1)
                inner = false;
        }
        if (!inner) continue;
        double lap = 0.0, scale = 0.0;
        for (int f = 0; f < 6; ++f) {
            const int nb = m.nbr[6 * size_t(c) + f];
            double dphi = 0.0;
            for (int a = 0; a < 3; ++a) dphi += g[a] * (m.cc[3 * size_t(nb) + a] - m.cc[3 * size_t(c) + a]);
            lap += m.lap_off[6 * size_t(c) + f] * dphi;
            scale += std::fabs(m.lap_off[6 * size_t(c) + f] * dphi);
        }
        if (scale > 0) r[3] = std::fmax(r[3], std::fabs(lap) / scale);
    }
    // points inside removed boxes touch no cell and carry no weights
    std::vector<double> wsum(m.n_points, 0.0);
    std::vector<char> used(m.n_points, 0);
    for (int c = 0; c < m.n_cells; ++c)
        for (int q = 0; q < 8; ++q) {
            wsum[m.cell_pt[8 * size_t(c) + q]] += m.vw_weight[8 * size_t(c) + q];
            used[m.cell_pt[8 * size_t(c) + q]] = 1;
        }
    for (int p = 0; p < m.n_points; ++p)
        if (used[p]) r[4] = std::fmax(r[4], std::fabs(wsum[p] - 1.0));
    for (int p = 0; p < m.n_points; ++p) {
        if (!used[p]) continue;
        double w = 0.0;
        for (int k = m.pi_start[p]; k < m.pi_start[p + 1]; ++k) w += m.pi_w[k];
        r[5] = std::fmax(r[5], std::fabs(w - 1.0));
    }
    double S[3] = {0, 0, 0};
    for (int f = 0; f < 6; ++f)
        for (int a = 0; a < 3; ++a) S[a] += m.cls_farea[f] * m.cls_fnormal[3 * f + a];
    r[6] = std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]) / m.cls_farea[0];
    for (int t = 0; t < 12; ++t) {
        for (int i = 1; i <= 3; ++i) {
            const int u = m.tt.inner_next[t][i];
            bool back = false;
            for (int j = 1; j <= 3; ++j) back |= m.tt.inner_next[u][j] == t;
            if (!back) r[7] = 1.0;
        }
        if (m.tt.cross_next[m.tt.cross_next[t]] != t) r[7] = 1.0;
    }
    for (int k = 0; k < n_out && k < 8; ++k) out[k] = r[k];
    return 8;
}

int oracle_create(const picgpu_mesh_desc* mesh, const picgpu_config* cfg, int nthreads,
                  oracle_ctx** out) {
    if (!mesh || !cfg || !out) return PICGPU_INVALID_ARG;
    *out = nullptr;
    auto* c = new oracle_ctx();
    Oracle& o = c->o;
    try {
        o.m = om::build(*mesh);
    } catch (const std::exception& e) {
        o.err = e.what();
        *out = c;
        return PICGPU_INVALID_ARG;
    }
    o.cfg = *cfg;
    if (cfg->n_species < 1 || cfg->n_species > PICGPU_MAX_SPECIES || !(cfg->dt > 0)) {
        o.err = "config: bad species count or dt";
        *out = c;
        return PICGPU_INVALID_ARG;
    }
    o.nthreads = nthreads > 0 ? nthreads : 1;
    const HexMesh& m = o.m;
    o.cloud.resize(cfg->n_species);
    o.phi.assign(m.n_cells, 0.0);
    o.rho.assign(m.n_cells, 0.0);
    o.E.assign(3 * size_t(m.n_cells), 0.0);
    o.Ept.assign(3 * size_t(m.n_points), 0.0);
    o.Eb.assign(3 * m.bfaces.size(), 0.0);
    o.ccData.assign(m.n_cells, 0.0);
    o.vtxData.assign(m.n_points, 0.0);
    o.ccFix.assign(m.n_cells, 0);
    o.vtxFix.assign(m.n_points, 0);
    o.sigma.assign(m.patches.size(), 0.0);
    o.gradBC.assign(m.patches.size(), 0.0);
    o.Qconv.assign(m.patches.size(), 0.0);
    {
        const std::string ce = ob::check_circuit(m, cfg->circuit, cfg->dt);
        if (!ce.empty()) { o.err = ce; *out = c; return PICGPU_INVALID_ARG; }
    }
    o.rlcK.assign(m.patches.size(), 0.0);
    if (cfg->circuit.model != PICGPU_CIRCUIT_NONE) {
        const picgpu_circuit& cc = cfg->circuit;
        const double area = m.patches[cc.cathode_patch].area;
        o.rlc = ob::rlc_coefficients(cc, cfg->dt, area);
        if (cc.model == PICGPU_CIRCUIT_RLC) o.rlcK[cc.cathode_patch] = o.rlc.k;
        o.circuitI = ob::circuit_current_source(cc, area);
        o.cathodeFaces = ob::circuit_cathode_faces(m, cc);
        o.circuit = ob::circuit_start(cc);
        if (cc.model == PICGPU_CIRCUIT_IDEAL_CURRENT) o.gradBC[cc.cathode_patch] = o.circuit.sigma / kEps0;
    }
    o.Mdiag.resize(m.n_cells);
    o.dinv.resize(m.n_cells);
    o.Moff.resize(6 * size_t(m.n_cells));
    for (int i = 0; i < m.n_cells; ++i) o.Mdiag[i] = -m.lap_diag[i];
    ob::circuit_add_diagonal(m, cfg->circuit, cfg->dt, o.Mdiag);
    for (int i = 0; i < m.n_cells; ++i) o.dinv[i] = 1.0 / o.Mdiag[i];
    for (size_t i = 0; i < o.Moff.size(); ++i) o.Moff[i] = -m.lap_off[i];
    double qmax = 0;
    for (int s = 0; s < cfg->n_species; ++s)
        qmax = std::fmax(qmax, std::fabs(cfg->species[s].charge * cfg->species[s].weight));
    o.fixScale = qmax > 0 ? std::ldexp(1.0, 39 - std::ilogb(qmax)) : 1.0;
    o.rotation = cfg->B[0] != 0.0 || cfg->B[1] != 0.0 || cfg->B[2] != 0.0;
    if (cfg->maxwell_solver != PICGPU_MAXWELL_ELECTROSTATIC) set_applied_field(o);
    o.svmax.assign(m.n_cells, 0.0);
    o.remainder.assign(m.n_cells, 0.0);
    if (cfg->mcc.enabled) {
        std::string e = ocoll::init_mcc(o.cfg, o.xs, m.n_cells, o.svmax, o.remainder);
        if (!e.empty()) { o.err = e; *out = c; return PICGPU_INVALID_ARG; }
        if (cfg->mcc.neutral_parcels) {
            const int ns = cfg->mcc.neutral_species;
            if (ns < 0 || ns >= cfg->n_species || cfg->species[ns].charge != 0.0 ||
                cfg->species[ns].weight != cfg->species[cfg->electron_species].weight ||
                (cfg->mcc.create_ion && cfg->species[ns].weight != cfg->species[cfg->mcc.ion_species].weight) ||
                cfg->binary.enabled) {
                o.err = "mcc: unsupported neutral-parcel set-up";
                *out = c;
                return PICGPU_INVALID_ARG;
            }
            o.psvmax = o.svmax;
            o.premainder.resize(m.n_cells);
            for (int k = 0; k < m.n_cells; ++k) {
                ocoll::Philox r(cfg->seed, ocoll::kStreamRemainder | 1u, uint32_t(k), 0u);
                o.premainder[k] = r.uniform();
            }
        }
    }
    o.isvmax.assign(m.n_cells, 0.0);
    o.iremainder.assign(m.n_cells, 0.0);
    if (cfg->ion_mcc.enabled) {
        std::string e = ocoll::init_ion_mcc(o.cfg, o.ixs, m.n_cells, o.isvmax, o.iremainder);
        if (!e.empty()) { o.err = e; *out = c; return PICGPU_INVALID_ARG; }
        if (cfg->ion_mcc.neutral_parcels) {
            const int ns = cfg->ion_mcc.neutral_species;
            if (ns < 0 || ns >= cfg->n_species || cfg->species[ns].charge != 0.0 || cfg->binary.enabled) {
                o.err = "ion mcc: unsupported neutral-parcel set-up";
                *out = c;
                return PICGPU_INVALID_ARG;
            }
            o.ipsvmax = o.isvmax;
            o.ipremainder.resize(m.n_cells);
            for (int k = 0; k < m.n_cells; ++k) {
                ocoll::Philox r(cfg->seed, ocoll::kStreamIonRemainder | 1u, uint32_t(k), 0u);
                o.ipremainder[k] = r.uniform();
            }
        }
    }
    o.perez.assign(size_t(cfg->n_species), Oracle::PerezTab{});
    if (cfg->perez.enabled) {
        // PerezIonizationModel.C:30-118: one entry per ion species; a limit
        // below 1 switches the species off
        const picgpu_perez& pz = cfg->perez;
        const int es = cfg->electron_species;
        bool okp = cfg->coulomb.enabled && es >= 0 && es < cfg->n_species && cfg->species[es].charge != 0.0 &&
                   pz.n_ions >= 0 && pz.n_ions <= PICGPU_PEREZ_MAX_IONS;
        for (int k = 0; okp && k < pz.n_ions; ++k) {
            const picgpu_perez_ion& in = pz.ion[k];
            okp = in.species >= 0 && in.species < cfg->n_species && in.species != es && in.atomic_number >= 1 &&
                  in.atomic_number <= PICGPU_PEREZ_MAX_Z;
            if (okp && in.ionization_limit != 0) o.perez[size_t(in.species)] = perez_tables(in);
        }
        if (!okp) {
            o.err = "Perez ionisation: bad settings";
            *out = c;
            return PICGPU_INVALID_ARG;
        }
    }
    if (cfg->merging.enabled) {
        // PairMerging.C:35-68: the settings and the species list
        const picgpu_merging& mg = cfg->merging;
        bool okm = mg.n_species >= 1 && mg.n_species <= PICGPU_MAX_SPECIES && mg.n_check_neighbors >= 1 &&
                   mg.reduction_factor > 0.0 && mg.reduction_factor <= 1.0 && mg.cell_parcels_max >= 1 &&
                   mg.max_checks >= 0 && mg.merge_maximum_per_cell >= 0 && mg.velocity_ratio >= 0.0 &&
                   double(mg.cell_parcels_max) * mg.reduction_factor >= double(mg.n_check_neighbors);
        for (int k = 0; okm && k < mg.n_species; ++k) okm = mg.species[k] >= 0 && mg.species[k] < cfg->n_species;
        if (!okm) {
            o.err = "PairMerging: bad settings";
            *out = c;
            return PICGPU_INVALID_ARG;
        }
    }
    if (cfg->coulomb.enabled && cfg->coulomb.pairing == 1) {
        double w = -1.0;
        for (int s = 0; s < cfg->n_species; ++s) {
            if (cfg->species[s].charge == 0.0 || !cfg->species[s].solve_movement) continue;
            if (w < 0) w = cfg->species[s].weight;
            else if (cfg->species[s].weight != w) {
                o.err = "coulomb: TakizukaAbe pairing needs equal species weights";
                *out = c;
                return PICGPU_INVALID_ARG;
            }
        }
    }
    *out = c;
    return 0;
}

void oracle_destroy(oracle_ctx* ctx) { delete ctx; }

const char* oracle_last_error(const oracle_ctx* ctx) { return ctx ? ctx->o.err.c_str() : "null"; }

int oracle_set_precond(oracle_ctx* ctx, int precond) {
    ctx->o.precond = precond;
    return 0;
}

int oracle_mesh_query(const oracle_ctx* ctx, picgpu_mesh_info* info) {
    info->n_cells = ctx->o.m.n_cells;
    info->n_points = ctx->o.m.n_points;
    info->n_tets = 12LL * ctx->o.m.n_cells;
    info->n_patches = (long long)ctx->o.m.patches.size();
    return 0;
}

int oracle_set_particles(oracle_ctx* ctx, int species, size_t n, const int32_t* tet,
                         const double* bary, const double* U) {
    Oracle& o = ctx->o;
    if (species < 0 || species >= o.cfg.n_species) return PICGPU_INVALID_ARG;
    auto& cl = o.cloud[species];
    cl.assign(n, Parcel{});
    const long long ntet = 12LL * o.m.n_cells;
    for (size_t i = 0; i < n; ++i) {
        if (tet[i] < 0 || tet[i] >= ntet) { o.err = "particles: tet index out of range"; cl.clear(); return PICGPU_INVALID_ARG; }
        Parcel& p = cl[i];
        p.cell = tet[i] / 12;
        p.tet = tet[i] % 12;
        p.y[1] = bary[3 * i];
        p.y[2] = bary[3 * i + 1];
        p.y[3] = bary[3 * i + 2];
        p.y[0] = 1.0 - p.y[1] - p.y[2] - p.y[3];
        p.U = v3(U[3 * i], U[3 * i + 1], U[3 * i + 2]);
    }
    return 0;
}

int oracle_set_parcel_attributes(oracle_ctx* ctx, int species, size_t n, const double* nParticle,
                                 const int32_t* chargeModifier) {
    Oracle& o = ctx->o;
    if (species < 0 || species >= o.cfg.n_species) return PICGPU_INVALID_ARG;
    auto& cl = o.cloud[species];
    if (n != cl.size() || (n && (!nParticle || !chargeModifier))) return PICGPU_INVALID_ARG;
    const double w = o.cfg.species[species].weight;
    for (size_t i = 0; i < n; ++i)
        if (!(nParticle[i] > 0.0) || !(nParticle[i] <= 4096.0 * w) || chargeModifier[i] < 0 || chargeModifier[i] > 1024)
            return PICGPU_INVALID_ARG;
    for (size_t i = 0; i < n; ++i) {
        cl[i].nw = nParticle[i];
        cl[i].zq = chargeModifier[i];
    }
    return 0;
}

int oracle_get_parcel_attributes(oracle_ctx* ctx, int species, size_t cap, double* nParticle,
                                 int32_t* chargeModifier, size_t* n) {
    Oracle& o = ctx->o;
    if (species < 0 || species >= o.cfg.n_species) return PICGPU_INVALID_ARG;
    const auto& cl = o.cloud[species];
    *n = cl.size();
    if (!nParticle) return 0;
    if (cap < cl.size() || !chargeModifier) return PICGPU_INVALID_ARG;
    for (size_t i = 0; i < cl.size(); ++i) {
        nParticle[i] = pweight(o, cl[i], species);
        chargeModifier[i] = cl[i].zq;
    }
    return 0;
}

int oracle_count_particles(oracle_ctx* ctx, int species, size_t* n) {
    if (species < 0 || species >= ctx->o.cfg.n_species) return PICGPU_INVALID_ARG;
    *n = ctx->o.cloud[species].size();
    return 0;
}

int oracle_get_particles(oracle_ctx* ctx, int species, size_t cap, int32_t* tet, double* bary,
                         double* U, size_t* n) {
    Oracle& o = ctx->o;
    if (species < 0 || species >= o.cfg.n_species) return PICGPU_INVALID_ARG;
    const auto& cl = o.cloud[species];
    *n = cl.size();
    if (cap < cl.size()) return PICGPU_INVALID_ARG;
    for (size_t i = 0; i < cl.size(); ++i) {
        tet[i] = cl[i].cell * 12 + cl[i].tet;
        for (int a = 0; a < 3; ++a) bary[3 * i + a] = cl[i].y[a + 1];
        U[3 * i] = cl[i].U.x;
        U[3 * i + 1] = cl[i].U.y;
        U[3 * i + 2] = cl[i].U.z;
    }
    return 0;
}

// The fixed-operation logarithm and sine of the initial-condition sampler
// (accuracy checks against the C library in the tests).
double oracle_det_log(double x) { return oinit::det_log(x); }
double oracle_det_sin(double x) { return oinit::det_sin(x); }

int oracle_set_injection(oracle_ctx* ctx, int n, const picgpu_injection* inj) {
    Oracle& o = ctx->o;
    if (n < 0 || n > PICGPU_MAX_INJECTORS || (n > 0 && !inj)) return PICGPU_INVALID_ARG;
    o.injectors.clear();
    for (int i = 0; i < n; ++i) {
        const picgpu_injection& q = inj[i];
        if (q.patch < 0 || q.patch >= int(o.m.patches.size())) return PICGPU_INVALID_ARG;
        const int kind = o.m.patches[q.patch].p.kind;
        if (kind == PICGPU_PATCH_CYCLIC || kind == PICGPU_PATCH_EMPTY) return PICGPU_INVALID_ARG;
        for (int j = 0; j < q.n_species; ++j)
            if (q.species[j] < 0 || q.species[j] >= o.cfg.n_species) return PICGPU_INVALID_ARG;
        Oracle::Injector I;
        I.cfg = q;
        I.tri = patch_triangles(o.m, q.patch);
        if (I.tri.cell.empty()) return PICGPU_INVALID_ARG;
        o.injectors.push_back(I);
    }
    return 0;
}

int oracle_set_emission(oracle_ctx* ctx, int n, const picgpu_emission* em) {
    Oracle& o = ctx->o;
    if (n < 0 || n > PICGPU_MAX_EMISSIONS || (n > 0 && !em)) return PICGPU_INVALID_ARG;
    const int es = o.cfg.electron_species;
    for (int i = 0; i < n; ++i) {
        const picgpu_emission& q = em[i];
        if (es < 0 || es >= o.cfg.n_species || o.cfg.species[es].charge == 0.0) return PICGPU_INVALID_ARG;
        if (q.patch < 0 || q.patch >= int(o.m.patches.size())) return PICGPU_INVALID_ARG;
        const int kind = o.m.patches[q.patch].p.kind;
        if (kind == PICGPU_PATCH_CYCLIC || kind == PICGPU_PATCH_EMPTY) return PICGPU_INVALID_ARG;
        if (q.model != PICGPU_EMISSION_THERMIONIC && q.model != PICGPU_EMISSION_FOWLER_NORDHEIM)
            return PICGPU_INVALID_ARG;
        if (!(q.work_function > 0.0)) return PICGPU_INVALID_ARG;
        if (q.model == PICGPU_EMISSION_THERMIONIC && !(q.temperature > 0.0 && q.lambda_r >= 0.0))
            return PICGPU_INVALID_ARG;
        if (q.weight > 0.0 && q.weight != o.cfg.species[es].weight) return PICGPU_INVALID_ARG;
    }
    o.emitters.clear();
    for (int i = 0; i < n; ++i) {
        Oracle::Emitter Z;
        Z.cfg = em[i];
        Z.tri = patch_triangles(o.m, em[i].patch);
        if (Z.tri.cell.empty()) return PICGPU_INVALID_ARG;
        if (em[i].model == PICGPU_EMISSION_THERMIONIC)
            Z.j = ob::thermionic_current(em[i].lambda_r, em[i].temperature, em[i].work_function,
                                         std::fabs(o.cfg.species[es].charge));
        for (size_t b = 0; b < o.m.bfaces.size(); ++b)
            if (o.m.bfaces[b].patch == em[i].patch) Z.faces.push_back(int(b));
        o.emitters.push_back(Z);
    }
    return 0;
}

int oracle_set_freestream(oracle_ctx* ctx, int n, const picgpu_freestream* fs) {
    Oracle& o = ctx->o;
    if (n < 0 || n > PICGPU_MAX_FREESTREAMS || (n > 0 && !fs)) return PICGPU_INVALID_ARG;
    for (int i = 0; i < n; ++i) {
        const std::string e = ob::check_freestream(o.m, o.cfg, fs[i]);
        if (!e.empty()) {
            o.err = e;
            return PICGPU_INVALID_ARG;
        }
    }
    o.freestreams.clear();
    for (int i = 0; i < n; ++i) {
        Oracle::FreeStream Z;
        Z.cfg = fs[i];
        Z.F = ob::freestream_faces(o.m, o.cfg, fs[i]);
        Z.acc.assign(size_t(Z.F.n_faces) * Z.F.n_species, 0.0);
        o.freestreams.push_back(Z);
    }
    return 0;
}

int oracle_initialise(oracle_ctx* ctx, const picgpu_init* init, picgpu_init_stats* stats) {
    if (!ctx || !init) return PICGPU_INVALID_ARG;
    return oracle_initialise_impl(ctx->o, init, stats);
}

int oracle_initialise_fields(oracle_ctx* ctx) {
    Oracle& o = ctx->o;
    calculate_fields(o);
    return solve_fields(o, nullptr);
}

int oracle_move(oracle_ctx* ctx, picgpu_step_stats* st) {
    Oracle& o = ctx->o;
    if (st) std::memset(st, 0, sizeof *st);
    int s = move_all(o, st);
    calculate_fields(o);
    fill_counts(o, st);
    return s;
}

// PICCloud::evolve (PICCloud.C:1426-1471)
int oracle_step(oracle_ctx* ctx, int nsteps, picgpu_step_stats* st) {
    Oracle& o = ctx->o;
    if (st) std::memset(st, 0, sizeof *st);
    int status = 0;
    for (int k = 0; k < nsteps; ++k) {
        inject(o);
        int s = move_all(o, st);
        if (s) return s;
        o.occ_n.assign(o.cloud.size(), 0);
        for (size_t q = 0; q < o.cloud.size(); ++q) o.occ_n[q] = long(o.cloud[q].size());
        collisions(o, st);
        calculate_fields(o);
        floating_pre_update(o);
        circuit_pre_update(o);
        s = solve_fields(o, st);
        if (s) status = s;
        circuit_post_update(o);
        // ParticleMerging::checkAndMerge, the last call of the step (PICCloud.C:1470)
        if (o.cfg.merging.enabled) merge_parcels(o, st);
        o.step_index++;
    }
    fill_counts(o, st);
    return status;
}

int oracle_solve_poisson(oracle_ctx* ctx, const double* rho, double* phi_inout,
                         picgpu_step_stats* st) {
    Oracle& o = ctx->o;
    if (st) std::memset(st, 0, sizeof *st);
    std::copy(rho, rho + o.m.n_cells, o.rho.begin());
    std::copy(phi_inout, phi_inout + o.m.n_cells, o.phi.begin());
    const int saved = o.cfg.maxwell_solver;
    o.cfg.maxwell_solver = PICGPU_MAXWELL_ELECTROSTATIC;
    int s = solve_fields(o, st);
    o.cfg.maxwell_solver = saved;
    std::copy(o.phi.begin(), o.phi.end(), phi_inout);
    return s;
}

int oracle_compute_field(oracle_ctx* ctx) {
    if (!ctx) return PICGPU_INVALID_ARG;
    if (ctx->o.cfg.maxwell_solver == PICGPU_MAXWELL_ELECTROSTATIC) compute_E(ctx->o);
    return 0;
}

int oracle_set_step_index(oracle_ctx* ctx, int64_t steps_done) {
    if (!ctx || steps_done < 0) return PICGPU_INVALID_ARG;
    ctx->o.step_index = steps_done;
    return 0;
}

int oracle_get_field(oracle_ctx* ctx, int which, double* out, size_t n) {
    Oracle& o = ctx->o;
    const std::vector<double>* v = nullptr;
    switch (which) {
        case PICGPU_FIELD_PHI: v = &o.phi; break;
        case PICGPU_FIELD_E_CELL: v = &o.E; break;
        case PICGPU_FIELD_RHO: v = &o.rho; break;
        case PICGPU_FIELD_E_POINT: v = &o.Ept; break;
        case PICGPU_FIELD_SIGMA_V_MAX: v = &o.svmax; break;
        case PICGPU_FIELD_PATCH_SIGMA:
            if (n < o.m.patches.size()) return PICGPU_INVALID_ARG;
            for (size_t p = 0; p < o.m.patches.size(); ++p)
                out[p] = o.m.patches[p].p.kind == PICGPU_PATCH_FLOATING ? o.sigma[p] : 0.0;
            return 0;
        case PICGPU_FIELD_B_CELL:
            if (o.Bcell.empty()) {
                if (n < 3 * size_t(o.m.n_cells)) return PICGPU_INVALID_ARG;
                for (size_t k = 0; k < 3 * size_t(o.m.n_cells); ++k) out[k] = o.cfg.B[k % 3];
                return 0;
            }
            v = &o.Bcell;
            break;
        default: return PICGPU_INVALID_ARG;
    }
    if (n < v->size()) return PICGPU_INVALID_ARG;
    std::copy(v->begin(), v->end(), out);
    return 0;
}

int oracle_set_field(oracle_ctx* ctx, int which, const double* in, size_t n) {
    Oracle& o = ctx->o;
    std::vector<double>* v = nullptr;
    switch (which) {
        case PICGPU_FIELD_PHI: v = &o.phi; break;
        case PICGPU_FIELD_E_CELL: v = &o.E; break;
        case PICGPU_FIELD_RHO: v = &o.rho; break;
        case PICGPU_FIELD_E_POINT: v = &o.Ept; break;
        case PICGPU_FIELD_PATCH_SIGMA:
            if (n < o.m.patches.size()) return PICGPU_INVALID_ARG;
            for (size_t p = 0; p < o.m.patches.size(); ++p) {
                if (o.m.patches[p].p.kind != PICGPU_PATCH_FLOATING) continue;
                o.sigma[p] = in[p];
                o.Qconv[p] = 0.0;
            }
            floating_pre_update(o);
            return 0;
        case PICGPU_FIELD_B_CELL: {
            if (n < 3 * size_t(o.m.n_cells)) return PICGPU_INVALID_ARG;
            o.Bcell.assign(in, in + 3 * size_t(o.m.n_cells));
            o.rotation = false;
            for (double b : o.Bcell) o.rotation = o.rotation || b != 0.0;
            return 0;
        }
        default: return PICGPU_INVALID_ARG;
    }
    if (n < v->size()) return PICGPU_INVALID_ARG;
    std::copy(in, in + v->size(), v->begin());
    return 0;
}

// KineticEnergyInfo.C:72-81, TemperatureInfo.C:71-76, FieldEnergyInfo.C:107-115
int oracle_diagnostics(oracle_ctx* ctx, picgpu_diagnostics* out) {
    Oracle& o = ctx->o;
    std::memset(out, 0, sizeof *out);
    for (size_t s = 0; s < o.cloud.size(); ++s) {
        const double m = o.cfg.species[s].mass;
        for (const Parcel& p : o.cloud[s]) {
            const double w = pweight(o, p, int(s));
            const double u2 = dotv(p.U, p.U);
            out->kinetic_energy[s] += 0.5 * m * u2 * w;
            const double b = magv(p.U) / kC;
            out->kinetic_energy_rel[s] += (1.0 / std::sqrt(1.0 - b * b) - 1.0) * m * kC * kC;
            out->momentum[s][0] += w * m * p.U.x;
            out->momentum[s][1] += w * m * p.U.y;
            out->momentum[s][2] += w * m * p.U.z;
            out->velocity_sq[s][0] += w * p.U.x * p.U.x;
            out->velocity_sq[s][1] += w * p.U.y * p.U.y;
            out->velocity_sq[s][2] += w * p.U.z * p.U.z;
            out->weight_sum[s] += w;
        }
    }
    double fe = 0;
    for (int c = 0; c < o.m.n_cells; ++c) {
        const double* e = &o.E[3 * size_t(c)];
        fe += (e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) * o.m.vol[c];
    }
    out->field_energy = 0.5 * kEps0 * fe;
    return 0;
}

double oracle_move_seconds(const oracle_ctx* ctx) { return ctx->o.move_seconds; }

void oracle_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    ocoll::Philox r(uint64_t(key[0]) | (uint64_t(key[1]) << 32), ctr[1], ctr[2], ctr[3]);
    r.ctr[0] = ctr[0];
    r.block();
    for (int k = 0; k < 4; ++k) out[k] = r.buf[k];
}

double oracle_debye_length(oracle_ctx* ctx, int cell) {
    Oracle& o = ctx->o;
    if (cell < 0 || cell >= o.m.n_cells) return 0.0;
    std::vector<int> charged;
    for (int s = 0; s < o.cfg.n_species; ++s)
        if (o.cfg.species[s].charge != 0.0 && o.cfg.species[s].solve_movement) charged.push_back(s);
    std::vector<std::vector<std::vector<int>>> occ(o.cfg.n_species, std::vector<std::vector<int>>(o.m.n_cells));
    for (int s = 0; s < o.cfg.n_species; ++s)
        for (size_t i = 0; i < o.cloud[s].size(); ++i)
            if (o.cloud[s][i].cell == cell) occ[s][cell].push_back(int(i));
    return debye_length(o, charged, occ, cell);
}

}  // extern "C"
