// oboundary.hpp -- the oracle's boundary models: the potential rule of each
// patch, the circuit models, FreeStream's face set-up and the emission
// currents.
//
// TEST INFRASTRUCTURE ONLY, written for the checker from the picFoam sources
// (paths relative to the picFoam tree, PICMCCFVM/submodels abbreviated SM/):
//   fixedValue / circuitBoundary / RLCBoundary potential conditions
//       SM/BoundaryModel/BoundaryConditions/circuitBoundary/circuitBoundaryFvPatchField.C:129-175,
//       SM/BoundaryModel/BoundaryConditions/RLCBoundary/RLCBoundaryFvPatchField.C
//   circuitRLC          SM/BoundaryModel/circuitRLC/circuitRLC.C:75-80,183-243
//   IdealVoltageSource  SM/BoundaryModel/IdealVoltageSource/IdealVoltageSource.C:126-151
//   IdealCurrentSource  SM/BoundaryModel/IdealCurrentSource/IdealCurrentSource.C:100-184
//   FreeStream          SM/BoundaryModel/FreeStream/FreeStream.C:126-396
//   ThermionicEmission  SM/Helper/Emission/ThermionicEmission/ThermionicEmission.C:36-52
//   FowlerNordheim      SM/Helper/Emission/FowlerNordheim/FowlerNordheim.C:49-104
// Where a sum runs over faces, the oracle adds in the order the library's
// reduction uses (256 strided lanes, then a halving tree), and the
// exponential of the Fowler-Nordheim current is the library's fixed-operation
// one (Taylor series after reduction by ln 2), so the two can be compared
// bit for bit; both are conventions of the library that the oracle states
// on its own.
#pragma once

#include <cmath>
#include <string>
#include <vector>

#include "omesh.hpp"
#include "picgpu.h"

namespace ob {

using om::BFace;
using om::Mesh;

// ----------------------------------------------------- potential rules ---
// How a boundary face enters -laplacian(phi) = rho / eps0.
enum { kRuleNone = 0, kRuleFixed = 1, kRuleGradient = 2, kRuleRlc = 3 };

inline int face_rule(int kind, int phi_bc) {
    const bool circuit = kind == PICGPU_PATCH_CIRCUIT;
    if (kind == PICGPU_PATCH_FLOATING || (circuit && phi_bc == PICGPU_PHI_CIRCUIT_GRADIENT)) return kRuleGradient;
    if (circuit && phi_bc == PICGPU_PHI_RLC) return kRuleRlc;
    return phi_bc == PICGPU_PHI_FIXED_VALUE ? kRuleFixed : kRuleNone;
}

// Right-hand side: fixedValue |S|/d phi_b; circuitBoundary |S| g (g = sigma/eps0);
// RLCBoundary |S| coeff1 coeff2 with coeff1 = 1/(k + d), k = a0 eps A, g = coeff2.
inline double face_rhs(int rule, double phi_b, double g, double k, double area, double d) {
    switch (rule) {
        case kRuleFixed: return (area / d) * phi_b;
        case kRuleGradient: return area * g;
        case kRuleRlc: return area * (g / (k + d));
        default: return 0.0;
    }
}

// The face value for the Gauss gradient; RLCBoundary evaluates to
// (1 - coeff1 / deltaCoeffs) phi_P.
inline double face_value(int rule, double phi_b, double g, double k, double d, double phi_c) {
    switch (rule) {
        case kRuleFixed: return phi_b;
        case kRuleGradient: return phi_c + g * d;
        case kRuleRlc: return (1.0 - d / (k + d)) * phi_c;
        default: return phi_c;
    }
}

// snGrad = (face value - phi_P) deltaCoeffs.
inline double face_sn_grad(int rule, double phi_b, double g, double k, double d, double phi_c) {
    switch (rule) {
        case kRuleFixed: return (phi_b - phi_c) / d;
        case kRuleGradient: return g;
        case kRuleRlc: return -(phi_c / (k + d));
        default: return 0.0;
    }
}

// ------------------------------------------------------------ circuits ---
struct RlcCoeffs {
    double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    double k = 0.0;      // a0 epsilon A (RLCBoundary)
};

inline double circuit_epsilon(const picgpu_circuit& cc) {
    if (cc.epsilon > 0.0) return cc.epsilon;
    const double c = 299792458.0, mu0 = 4.0 * 3.14159265358979323846 * 1e-7;
    return 1.0 / (mu0 * c * c);
}

// circuitRLC.C:75-80: second-order backward differences of
// L Q'' + R Q' + Q / C over Q^n .. Q^(n-4).
inline RlcCoeffs rlc_coefficients(const picgpu_circuit& cc, double dt, double cathode_area) {
    RlcCoeffs r;
    if (cc.model != PICGPU_CIRCUIT_RLC) return r;
    const double L = cc.L, R = cc.R, C = cc.C;
    r.a[0] = 2.25 * L / dt / dt + 1.5 * R / dt + 1.0 / C;
    r.a[1] = -6.0 * L / dt / dt - 2.0 * R / dt;
    r.a[2] = 5.5 * L / dt / dt + 0.5 * R / dt;
    r.a[3] = -2.0 * L / dt / dt;
    r.a[4] = 0.25 * L / dt / dt;
    r.k = r.a[0] * circuit_epsilon(cc) * cathode_area;
    return r;
}

// IdealCurrentSource.C:124-139: I scaled by A / refArea, or J A.
inline double circuit_current_source(const picgpu_circuit& cc, double cathode_area) {
    if (cc.J > 0.0) return cc.J * cathode_area;
    if (cc.ref_area > 0.0) return cc.I * (cathode_area / cc.ref_area);
    return cc.I;
}

// circuitRLC's source(): V sin(omega t + phase), the phase added in one
// fused operation (the library's rounding convention for both hosts).
inline double circuit_source(const picgpu_circuit& cc, double t) {
    return cc.V * std::sin(std::fma(cc.omega, t, cc.phase));
}

// The constructors' FatalErrors; empty when the circuit is usable.
inline std::string check_circuit(const Mesh& m, const picgpu_circuit& cc, double dt) {
    const int np = int(m.patches.size());
    int electrodes = 0;
    for (int p = 0; p < np; ++p) {
        const picgpu_patch& P = m.patches[p].p;
        if (P.kind == PICGPU_PATCH_CIRCUIT) {
            ++electrodes;
        } else if (P.phi_bc == PICGPU_PHI_RLC || P.phi_bc == PICGPU_PHI_CIRCUIT_GRADIENT) {
            return "circuit: circuit potential condition on a patch that is no electrode";
        }
    }
    if (cc.model == PICGPU_CIRCUIT_NONE) return electrodes ? "circuit: electrodes without a circuit model" : "";
    if (cc.model < PICGPU_CIRCUIT_NONE || cc.model > PICGPU_CIRCUIT_IDEAL_CURRENT) return "circuit: unknown model";
    if (cc.cathode_patch < 0 || cc.cathode_patch >= np) return "circuit: cathode out of range";
    if (cc.anode_patch < -1 || cc.anode_patch >= np || cc.anode_patch == cc.cathode_patch)
        return "circuit: anode out of range";
    for (int p = 0; p < np; ++p)
        if (m.patches[p].p.kind == PICGPU_PATCH_CIRCUIT && p != cc.cathode_patch && p != cc.anode_patch)
            return "circuit: an electrode that is neither anode nor cathode";
    const picgpu_patch& K = m.patches[cc.cathode_patch].p;
    if (K.kind != PICGPU_PATCH_CIRCUIT || m.patches[cc.cathode_patch].n_faces == 0)
        return "circuit: the cathode is no electrode with faces";
    if (cc.anode_patch >= 0) {
        const picgpu_patch& A = m.patches[cc.anode_patch].p;
        if (A.kind != PICGPU_PATCH_CIRCUIT || A.phi_bc != PICGPU_PHI_FIXED_VALUE)
            return "circuit: the anode needs a fixedValue potential";
    }
    if (!m.has_dirichlet) return "circuit: no fixedValue potential anywhere";
    switch (cc.model) {
        case PICGPU_CIRCUIT_RLC:
            if (K.phi_bc != PICGPU_PHI_RLC) return "circuit: circuitRLC needs RLCBoundary on the cathode";
            if (!(cc.C > 0.0) || !(cc.L >= 0.0) || !(cc.R >= 0.0) || !(dt > 0.0)) return "circuit: bad R, L or C";
            break;
        case PICGPU_CIRCUIT_IDEAL_VOLTAGE:
            if (K.phi_bc != PICGPU_PHI_FIXED_VALUE) return "circuit: the cathode needs a fixedValue potential";
            break;
        default:
            if (K.phi_bc != PICGPU_PHI_CIRCUIT_GRADIENT) return "circuit: the cathode needs circuitBoundary";
            if (cc.I < 0.0 && cc.J < 0.0) return "circuit: neither I nor J given";
    }
    return "";
}

inline std::vector<int> circuit_cathode_faces(const Mesh& m, const picgpu_circuit& cc) {
    std::vector<int> faces;
    if (cc.model == PICGPU_CIRCUIT_NONE) return faces;
    for (int b = 0; b < int(m.bfaces.size()); ++b)
        if (m.bfaces[b].patch == cc.cathode_patch) faces.push_back(b);
    return faces;
}

// RLCBoundary adds |S| coeff1 per cathode face to the SPD operator's diagonal.
inline void circuit_add_diagonal(const Mesh& m, const picgpu_circuit& cc, double dt, std::vector<double>& diag) {
    if (cc.model != PICGPU_CIRCUIT_RLC) return;
    const double k = rlc_coefficients(cc, dt, m.patches[cc.cathode_patch].area).k;
    for (const BFace& b : m.bfaces)
        if (b.patch == cc.cathode_patch) diag[b.cell] = diag[b.cell] + b.area / (k + b.delta);
}

// A sum over n faces in the library's reduction order: lane t of 256 adds
// faces t, t + 256, ...; the lanes then add pairwise, halving.
template <class Value>
inline double lane_sum(int n, Value&& value) {
    std::vector<double> acc(256, 0.0);
    for (int i = 0; i < n; ++i) acc[i % 256] = acc[i % 256] + value(i);
    for (int half = 128; half >= 1; half /= 2)
        for (int t = 0; t < half; ++t) acc[t] = acc[t] + acc[t + half];
    return acc[0];
}

struct CircuitState {
    double Q[4];            // circuitRLC Qex_, Qex1_, Qex2_, Qex3_
    double sigma;           // cathode surface charge density
    double voltage, current, cathode_current, charge;
    double qa[3], qc[3];    // IdealVoltageSource: anode and cathode charge histories
};

inline CircuitState circuit_start(const picgpu_circuit& cc) {
    CircuitState S{};
    for (int i = 0; i < 4; ++i) S.Q[i] = cc.Q[i];
    S.sigma = cc.sigma;
    if (cc.model == PICGPU_CIRCUIT_RLC) S.charge = cc.Q[0];
    return S;
}

// preUpdate_Boundary: circuitRLC sets coeff2 = a0 A sigma + a0 (q_acc - Q) + (source - k)
// (circuitRLC.C:183-191); IdealCurrentSource advances sigma by (q_acc - I dt) / A
// and sets the gradient sigma / eps0 (IdealCurrentSource.C:157-170).
inline void circuit_pre_update(int model, int cathode, const double* a, double area, double I, double dt,
                               double eps0, double src, double* qconv, double* g, CircuitState& S) {
    if (model == PICGPU_CIRCUIT_RLC) {
        const double k = a[1] * S.Q[0] + a[2] * S.Q[1] + a[3] * S.Q[2] + a[4] * S.Q[3];
        g[cathode] = a[0] * area * S.sigma + a[0] * (qconv[cathode] - S.Q[0]) + (src - k);
        return;
    }
    if (model == PICGPU_CIRCUIT_IDEAL_CURRENT) {
        S.sigma = S.sigma + (qconv[cathode] - I * dt) / area;
        g[cathode] = S.sigma / eps0;
        qconv[cathode] = 0.0;
        S.charge = S.sigma * area;
    }
}

// postUpdate_Boundary.  face_sum: the cathode faces' RLCBoundary face values
// (circuitRLC) or |S| phi_P (IdealCurrentSource); beta = dt / (t - averageStart).
inline void circuit_post_update(int model, int anode, int cathode, int n_faces, const double* a, double area,
                                double dt, double src, double beta, double face_sum, double* qconv,
                                CircuitState& S) {
    auto history = [](double* h, double dq) {
        h[2] = h[1];
        h[1] = h[0];
        h[0] = h[0] - dq;
    };
    auto average = [dt, beta](double old, const double* h) {
        return (1.0 - beta) * old + beta * ((2.0 * (h[0] - h[1]) + 0.5 * (h[2] - h[0])) / dt);
    };
    switch (model) {
        case PICGPU_CIRCUIT_RLC: {
            // circuitRLC.C:194-243
            const double k = (a[1] * S.Q[0] + a[2] * S.Q[1] + a[3] * S.Q[2] + a[4] * S.Q[3]) / a[0];
            const double phi_bound = face_sum / double(n_faces);
            for (int i = 3; i > 0; --i) S.Q[i] = S.Q[i - 1];
            S.Q[0] = (src - phi_bound) / a[0] - k;
            const double Iex = (S.Q[0] - S.Q[1]) / dt;
            S.sigma = S.sigma + (qconv[cathode] + Iex * dt) / area;
            S.voltage = phi_bound;
            S.current = Iex;
            S.charge = S.Q[0];
            qconv[cathode] = 0.0;
            if (anode >= 0) qconv[anode] = 0.0;
            break;
        }
        case PICGPU_CIRCUIT_IDEAL_VOLTAGE: {
            // IdealVoltageSource.C:126-151: running averages of the electrode currents
            history(S.qa, anode >= 0 ? qconv[anode] : 0.0);
            history(S.qc, qconv[cathode]);
            if (anode >= 0) qconv[anode] = 0.0;
            qconv[cathode] = 0.0;
            S.current = average(S.current, S.qa);
            S.cathode_current = average(S.cathode_current, S.qc);
            break;
        }
        case PICGPU_CIRCUIT_IDEAL_CURRENT:
            // IdealCurrentSource.C:173-184: the area-weighted cathode potential
            S.voltage = face_sum / area;
            if (anode >= 0) qconv[anode] = 0.0;
            break;
        default: break;
    }
}

// ---------------------------------------------------------- FreeStream ---
constexpr double kBoltzmann = 1.380649e-23;

struct FreeStreamFaces {
    int n_faces = 0, n_species = 0;
    std::vector<int> cell, tet0;
    std::vector<double> frac0, n_in, t1, t2, add, s, c_mp, v_t;
};

inline std::string check_freestream(const Mesh& m, const picgpu_config& cfg, const picgpu_freestream& fs) {
    if (fs.patch < 0 || fs.patch >= int(m.patches.size())) return "freestream: patch out of range";
    if (m.patches[fs.patch].p.kind != PICGPU_PATCH_ABSORB) return "freestream: the patch must absorb";
    if (m.patches[fs.patch].n_faces == 0) return "freestream: patch without faces";
    if (fs.n_species < 1 || fs.n_species > PICGPU_MAX_SPECIES) return "freestream: bad species count";
    for (int j = 0; j < fs.n_species; ++j)
        if (fs.species[j] < 0 || fs.species[j] >= cfg.n_species || !(fs.number_density[j] >= 0.0))
            return "freestream: bad species or number density";
    if (!(fs.temperature > 1e-300)) return "freestream: zero boundary temperature";  // FreeStream.C:176-183
    return "";
}

// Per face of the patch: the accumulator increment of Bird's eq. 4.22,
// |S| n/w dt c_mp (exp(-s^2) + sqrt(pi) s (1 + erf s)) / (2 sqrt(pi)) with
// s = U . n_in / c_mp (FreeStream.C:186-205), and the frame the parcels are
// emitted in: inward normal, t1 from the face's first point to its centre
// and t2 = n x t1 (FreeStream.C:255-263).
inline FreeStreamFaces freestream_faces(const Mesh& m, const picgpu_config& cfg, const picgpu_freestream& fs) {
    FreeStreamFaces F;
    F.n_species = fs.n_species;
    const double rpi = std::sqrt(3.14159265358979323846);
    for (int j = 0; j < fs.n_species; ++j) {
        const double kTm = kBoltzmann * fs.temperature / cfg.species[fs.species[j]].mass;
        F.c_mp.push_back(std::sqrt(2.0 * kTm));
        F.v_t.push_back(std::sqrt(kTm));
    }
    for (const BFace& b : m.bfaces) {
        if (b.patch != fs.patch) continue;
        const double* off = &m.cls_offset[size_t(m.cell_class[b.cell]) * 24];
        const int t0 = 2 * b.local_face;
        double part[2];
        for (int k = 0; k < 2; ++k) {
            const double* A = off + 3 * m.tt.tri[t0 + k][0];
            const double* B = off + 3 * m.tt.tri[t0 + k][1];
            const double* C = off + 3 * m.tt.tri[t0 + k][2];
            const double u[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
            const double v[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
            double w[3];
            om::vcross(u, v, w);
            part[k] = 0.5 * std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        }
        F.cell.push_back(b.cell);
        F.tet0.push_back(t0);
        F.frac0.push_back(part[0] / b.area);
        const double n[3] = {-b.normal[0], -b.normal[1], -b.normal[2]};
        const double* first = off + 3 * m.tt.tri[t0][0];
        double t1[3], t2[3];
        for (int a = 0; a < 3; ++a) t1[a] = b.centre[a] - (m.cc[3 * size_t(b.cell) + a] + first[a]);
        const double m1 = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
        for (double& x : t1) x = x / m1;
        om::vcross(n, t1, t2);
        const double m2 = std::sqrt(t2[0] * t2[0] + t2[1] * t2[1] + t2[2] * t2[2]);
        for (int a = 0; a < 3; ++a) {
            t2[a] = t2[a] / m2;
            F.n_in.push_back(n[a]);
            F.t1.push_back(t1[a]);
            F.t2.push_back(t2[a]);
        }
        const double un = fs.velocity[0] * n[0] + fs.velocity[1] * n[1] + fs.velocity[2] * n[2];
        for (int j = 0; j < fs.n_species; ++j) {
            const double s = un / F.c_mp[j];
            // exp(-s^2) + sqrt(pi) s (1 + erf s), the product added in one fused operation
            const double shape = std::fma(rpi * s, 1.0 + std::erf(s), std::exp(-(s * s)));
            const double w = cfg.species[fs.species[j]].weight;
            F.add.push_back(b.area * (fs.number_density[j] / w) * cfg.dt * F.c_mp[j] * shape / (2.0 * rpi));
            F.s.push_back(s);
        }
        ++F.n_faces;
    }
    return F;
}

// ----------------------------------------------------------- emission ---
// exp(x) in fixed FP64 operations (the library's convention, so GPU and
// oracle count the same emitted parcels): x = k ln 2 + r with ln 2 in two
// parts, e^r = sum of r^i / i! for i <= 17 by Horner's rule, then 2^k.
inline double fixed_exp(double x) {
    if (x < -745.0) return 0.0;
    const double ln2a = 0.6931471805599452862, ln2b = 2.3190468138462996e-17;
    const double k = std::rint(x / ln2a);
    const double r = (x - k * ln2a) - k * ln2b;
    double factorial[18];
    factorial[0] = 1.0;
    for (int i = 1; i < 18; ++i) factorial[i] = factorial[i - 1] * double(i);
    double p = 1.0 / factorial[17];
    for (int i = 16; i >= 1; --i) p = p * r + 1.0 / factorial[i];
    p = p * r + 1.0;
    return std::ldexp(p, int(k));
}

// FowlerNordheim.C:76-89 (t = 1): faces with an outward field only.
inline double fowler_nordheim_face(const double* E, const double* n, double W) {
    const double A = 1.541434e-6, B = 6.830889776e9;
    if (!(E[0] * n[0] + E[1] * n[1] + E[2] * n[2] > 0.0)) return 0.0;
    const double magE = std::sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
    const double y = 3.7947e-5 * std::sqrt(magE) / W;
    const double v = 0.956 - 1.062 * y * y;
    const double rw = std::sqrt(W);
    return A * magE * magE / W * fixed_exp(-(B * v * rw * rw * rw / magE));
}

// ThermionicEmission.C:49: Richardson-Dushman with A0 = 4 pi m k^2 e / h^3.
inline double thermionic_current(double lambda_r, double T, double W, double qe) {
    return lambda_r * 1201732.101 * T * T * std::exp(-(W * qe / (T * kBoltzmann)));
}

}  // namespace ob
