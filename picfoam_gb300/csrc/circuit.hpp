// circuit.hpp -- circuit boundary models, shared by the device code and the
// oracle so both evaluate the same expressions:
//   circuitRLC          PICMCCFVM/submodels/BoundaryModel/circuitRLC/circuitRLC.C
//   RLCBoundary         .../BoundaryConditions/RLCBoundary/RLCBoundaryFvPatchField.C
//   IdealVoltageSource  .../BoundaryModel/IdealVoltageSource/IdealVoltageSource.C
//   IdealCurrentSource  .../BoundaryModel/IdealCurrentSource/IdealCurrentSource.C
//
// The potential boundary rules of every patch kind are here too: the matrix
// diagonal, the right-hand side, the face value used by the Gauss gradient
// and the normal gradient used for the boundary value of E.
#pragma once

#include <cmath>
#include <string>
#include <vector>

#include "hexmesh.hpp"
#include "picgpu.h"

#ifdef __CUDACC__
#define PG_HD __host__ __device__
#else
#define PG_HD
#endif

namespace pg {

// How the potential sees a boundary face of a patch.
enum FaceRule { kRuleNone = 0, kRuleFixed = 1, kRuleGradient = 2, kRuleRlc = 3 };

PG_HD inline int face_rule(int kind, int phi_bc) {
    if (kind == PICGPU_PATCH_FLOATING) return kRuleGradient;
    if (kind == PICGPU_PATCH_CIRCUIT && phi_bc == PICGPU_PHI_CIRCUIT_GRADIENT) return kRuleGradient;
    if (kind == PICGPU_PATCH_CIRCUIT && phi_bc == PICGPU_PHI_RLC) return kRuleRlc;
    if (phi_bc == PICGPU_PHI_FIXED_VALUE) return kRuleFixed;
    return kRuleNone;
}

// Right-hand side term of a boundary face in -laplacian(phi) = rho/eps0:
// fixedValue |S|/d phi_b, circuitBoundary |S| g, RLCBoundary
// |S| coeff1 coeff2 with coeff1 = 1/(k + d), k = a0 epsilon A
// (RLCBoundaryFvPatchField.C gradientBoundaryCoeffs, circuitRLC.C:147).
// g: the patch's gradient (circuitBoundary) or coeff2 (RLC).
PG_HD inline double face_rhs(int rule, double phi_b, double g, double k, double area, double d) {
    if (rule == kRuleFixed) return (area / d) * phi_b;
    if (rule == kRuleGradient) return area * g;
    if (rule == kRuleRlc) return area * (g / (k + d));
    return 0.0;
}

// Face value of the potential for the Gauss gradient.  RLCBoundary evaluates
// to (1 - coeff1/deltaCoeffs) phi_P (RLCBoundaryFvPatchField.C evaluate).
PG_HD inline double face_value(int rule, double phi_b, double g, double k, double d, double phi_c) {
    if (rule == kRuleFixed) return phi_b;
    if (rule == kRuleGradient) return phi_c + g * d;
    if (rule == kRuleRlc) return (1.0 - d / (k + d)) * phi_c;
    return phi_c;
}

// Normal gradient (face value - phi_P) * deltaCoeffs.
PG_HD inline double face_sn_grad(int rule, double phi_b, double g, double k, double d, double phi_c) {
    if (rule == kRuleFixed) return (phi_b - phi_c) / d;
    if (rule == kRuleGradient) return g;
    if (rule == kRuleRlc) return -(phi_c / (k + d));
    return 0.0;
}

// circuitRLC.C:75-80: backward-difference coefficients of
// L Q'' + R Q' + Q/C = source - phi_cathode over the charges Q^n .. Q^(n-4).
struct RlcCoeffs {
    double a[5] = {0, 0, 0, 0, 0};
    double k = 0.0;   // a0 * epsilon * cathode area
};

inline double circuit_eps(const picgpu_circuit& cc) {
    return cc.epsilon > 0.0 ? cc.epsilon : 1.0 / (4.0 * 3.14159265358979323846 * 1e-7 * 299792458.0 * 299792458.0);
}

inline RlcCoeffs rlc_coefficients(const picgpu_circuit& cc, double dt, double cathode_area) {
    RlcCoeffs r;
    if (cc.model != PICGPU_CIRCUIT_RLC) return r;
    r.a[0] = 2.25 * cc.L / dt / dt + 1.5 * cc.R / dt + 1.0 / cc.C;
    r.a[1] = -6.0 * cc.L / dt / dt - 2.0 * cc.R / dt;
    r.a[2] = 5.5 * cc.L / dt / dt + 0.5 * cc.R / dt;
    r.a[3] = -2.0 * cc.L / dt / dt;
    r.a[4] = 0.25 * cc.L / dt / dt;
    r.k = r.a[0] * circuit_eps(cc) * cathode_area;
    return r;
}

// IdealCurrentSource.C:124-139: the supplied current, scaled by
// cathode area / refArea, or J * cathode area when J is given.
inline double circuit_current_source(const picgpu_circuit& cc, double cathode_area) {
    double I = cc.I;
    if (cc.ref_area > 0.0) I = I * (cathode_area / cc.ref_area);
    if (cc.J > 0.0) I = cc.J * cathode_area;
    return I;
}

// source() of circuitRLC (circuitRLCI.H): V sin(omega t + phase).
inline double circuit_source(const picgpu_circuit& cc, double t) {
    return cc.V * std::sin(std::fma(cc.omega, t, cc.phase));
}

// Checks a circuit against the mesh (the FatalErrors of the three
// constructors); returns an empty string when it is usable.
inline std::string check_circuit(const HexMesh& m, const picgpu_circuit& cc, double dt) {
    const int np = int(m.patches.size());
    int n_circuit = 0;
    for (int p = 0; p < np; ++p) {
        const picgpu_patch& P = m.patches[p].p;
        if (P.kind != PICGPU_PATCH_CIRCUIT &&
            (P.phi_bc == PICGPU_PHI_RLC || P.phi_bc == PICGPU_PHI_CIRCUIT_GRADIENT))
            return "circuit: RLCBoundary / circuitBoundary potential on a patch that is not a circuit electrode";
        if (P.kind == PICGPU_PATCH_CIRCUIT) ++n_circuit;
    }
    if (cc.model == PICGPU_CIRCUIT_NONE) {
        if (n_circuit) return "circuit: circuit patches without a circuit model";
        return "";
    }
    if (cc.model < PICGPU_CIRCUIT_NONE || cc.model > PICGPU_CIRCUIT_IDEAL_CURRENT) return "circuit: unknown model";
    if (cc.cathode_patch < 0 || cc.cathode_patch >= np) return "circuit: cathode patch out of range";
    if (cc.anode_patch < -1 || cc.anode_patch >= np || cc.anode_patch == cc.cathode_patch)
        return "circuit: anode patch out of range";
    for (int p = 0; p < np; ++p)
        if (m.patches[p].p.kind == PICGPU_PATCH_CIRCUIT && p != cc.cathode_patch && p != cc.anode_patch)
            return "circuit: a circuit patch that is neither the anode nor the cathode";
    const picgpu_patch& K = m.patches[cc.cathode_patch].p;
    if (K.kind != PICGPU_PATCH_CIRCUIT) return "circuit: the cathode patch is not of kind CIRCUIT";
    if (m.patches[cc.cathode_patch].n_faces == 0) return "circuit: the cathode patch has no faces";
    if (cc.anode_patch >= 0) {
        const picgpu_patch& A = m.patches[cc.anode_patch].p;
        if (A.kind != PICGPU_PATCH_CIRCUIT) return "circuit: the anode patch is not of kind CIRCUIT";
        if (A.phi_bc != PICGPU_PHI_FIXED_VALUE) return "circuit: expected fixedValue potential on the anode";
    }
    if (!m.has_dirichlet) return "circuit: the case needs a fixedValue potential patch (the anode)";
    if (cc.model == PICGPU_CIRCUIT_RLC) {
        if (K.phi_bc != PICGPU_PHI_RLC) return "circuit: circuitRLC expects the RLCBoundary potential on the cathode";
        if (!(cc.C > 0.0) || !(cc.L >= 0.0) || !(cc.R >= 0.0) || !(dt > 0.0))
            return "circuit: circuitRLC needs C > 0, L >= 0, R >= 0";
    } else if (cc.model == PICGPU_CIRCUIT_IDEAL_VOLTAGE) {
        if (K.phi_bc != PICGPU_PHI_FIXED_VALUE) return "circuit: expected fixedValue potential on the cathode";
    } else {
        if (K.phi_bc != PICGPU_PHI_CIRCUIT_GRADIENT)
            return "circuit: IdealCurrentSource expects the circuitBoundary potential on the cathode";
        if (cc.I < 0.0 && cc.J < 0.0) return "circuit: no current I or current density J was given";
    }
    return "";
}

// Boundary faces of the cathode in face order (the order of the fixed
// reduction over them).
inline std::vector<int> circuit_cathode_faces(const HexMesh& m, const picgpu_circuit& cc) {
    std::vector<int> f;
    if (cc.model == PICGPU_CIRCUIT_NONE) return f;
    for (size_t b = 0; b < m.bfaces.size(); ++b)
        if (m.bfaces[b].patch == cc.cathode_patch) f.push_back(int(b));
    return f;
}

// RLCBoundary's matrix diagonal: |S| coeff1 per cathode face
// (gradientInternalCoeffs = -coeff1 of the negative-definite laplacian).
inline void circuit_add_diagonal(const HexMesh& m, const picgpu_circuit& cc, double dt, std::vector<double>& Mdiag) {
    if (cc.model != PICGPU_CIRCUIT_RLC) return;
    const RlcCoeffs r = rlc_coefficients(cc, dt, m.patches[cc.cathode_patch].area);
    for (const BFace& B : m.bfaces)
        if (B.patch == cc.cathode_patch) Mdiag[B.cell] = Mdiag[B.cell] + B.area / (r.k + B.delta);
}

// Sum over the cathode faces in the device's fixed order: 256 lanes, lane t
// adds faces t, t + 256, ... in turn, then a halving tree over the lanes.
constexpr int kCircuitLanes = 256;

template <class F>
inline double circuit_face_sum(int n, F&& value) {
    double lane[kCircuitLanes];
    for (int t = 0; t < kCircuitLanes; ++t) {
        double a = 0.0;
        for (int i = t; i < n; i += kCircuitLanes) a = a + value(i);
        lane[t] = a;
    }
    for (int s = kCircuitLanes / 2; s > 0; s >>= 1)
        for (int t = 0; t < s; ++t) lane[t] = lane[t] + lane[t + s];
    return lane[0];
}

// Per-patch circuit state advanced once per step (FP64).
struct CircuitState {
    double Q[4];        // circuitRLC Qex_, Qex1_, Qex2_, Qex3_
    double sigma;       // cathode surface charge density (sigma1_ / sigma_)
    double voltage;     // last reported voltage
    double current;     // circuitRLC Iex_ / IdealVoltageSource anode average
    double cathode_current;
    double charge;      // reported charge
    double qa[3];       // IdealVoltageSource Qconv_, Qconv1_, Qconv2_
    double qc[3];       // ... Cathode
};

// preUpdate_Boundary (circuitRLC.C:183-191, IdealCurrentSource.C:157-170).
// qconv: charge gathered on each patch this step; g: per-patch gradient /
// coeff2 of the potential condition.
PG_HD inline void circuit_pre_update(int model, int cathode, const double* a, double area, double I, double dt,
                                     double eps0, double src, double* qconv, double* g, CircuitState& S) {
    if (model == PICGPU_CIRCUIT_RLC) {
        const double k = a[1] * S.Q[0] + a[2] * S.Q[1] + a[3] * S.Q[2] + a[4] * S.Q[3];
        g[cathode] = a[0] * area * S.sigma + a[0] * (qconv[cathode] - S.Q[0]) + (src - k);
    } else if (model == PICGPU_CIRCUIT_IDEAL_CURRENT) {
        S.sigma = S.sigma + (qconv[cathode] - I * dt) / area;
        g[cathode] = S.sigma / eps0;
        qconv[cathode] = 0.0;
        S.charge = S.sigma * area;
    }
}

// postUpdate_Boundary (circuitRLC.C:194-243, IdealVoltageSource.C:126-151,
// IdealCurrentSource.C:173-184).  face_sum: the fixed-order sum over the
// cathode faces of the RLCBoundary face value (RLC) or |S| phi_P (ideal
// current); beta = dt / (t - averageStart).
PG_HD inline void circuit_post_update(int model, int anode, int cathode, int n_faces, const double* a, double area,
                                      double dt, double src, double beta, double face_sum, double* qconv,
                                      CircuitState& S) {
    if (model == PICGPU_CIRCUIT_RLC) {
        const double k = (a[1] * S.Q[0] + a[2] * S.Q[1] + a[3] * S.Q[2] + a[4] * S.Q[3]) / a[0];
        const double phi_b = face_sum / double(n_faces);
        S.Q[3] = S.Q[2];
        S.Q[2] = S.Q[1];
        S.Q[1] = S.Q[0];
        S.Q[0] = (src - phi_b) / a[0] - k;
        const double Iex = (S.Q[0] - S.Q[1]) / dt;
        S.sigma = S.sigma + (qconv[cathode] + Iex * dt) / area;
        S.voltage = phi_b;
        S.current = Iex;
        S.charge = S.Q[0];
        qconv[cathode] = 0.0;
        if (anode >= 0) qconv[anode] = 0.0;
    } else if (model == PICGPU_CIRCUIT_IDEAL_VOLTAGE) {
        const double qa = anode >= 0 ? qconv[anode] : 0.0;
        S.qa[2] = S.qa[1];
        S.qa[1] = S.qa[0];
        S.qa[0] = S.qa[0] - qa;
        S.qc[2] = S.qc[1];
        S.qc[1] = S.qc[0];
        S.qc[0] = S.qc[0] - qconv[cathode];
        if (anode >= 0) qconv[anode] = 0.0;
        qconv[cathode] = 0.0;
        S.current = (1.0 - beta) * S.current +
                    beta * ((2.0 * (S.qa[0] - S.qa[1]) + 0.5 * (S.qa[2] - S.qa[0])) / dt);
        S.cathode_current = (1.0 - beta) * S.cathode_current +
                            beta * ((2.0 * (S.qc[0] - S.qc[1]) + 0.5 * (S.qc[2] - S.qc[0])) / dt);
    } else if (model == PICGPU_CIRCUIT_IDEAL_CURRENT) {
        S.voltage = face_sum / area;
        if (anode >= 0) qconv[anode] = 0.0;
    }
}

inline CircuitState circuit_start(const picgpu_circuit& cc) {
    CircuitState S{};
    for (int i = 0; i < 4; ++i) S.Q[i] = cc.Q[i];
    S.sigma = cc.sigma;
    S.charge = cc.model == PICGPU_CIRCUIT_RLC ? cc.Q[0] : 0.0;
    return S;
}

}  // namespace pg
