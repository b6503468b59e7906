// emission.hpp -- the EmissionModels of the circuit boundary models
// (PICMCCFVM/submodels/Helper/Emission): the current density each one
// draws from the cathode, shared by the device code and the oracle.
//   ThermionicEmission  ThermionicEmission.C:36-52: Richardson-Dushman,
//                       J = lambdaR A0 T^2 exp(-W e / (k T)), constant;
//   FowlerNordheim      FowlerNordheim.C:49-98: per face with an outward
//                       field, J = A |E|^2 / (W t^2) exp(-B v(y) W^1.5 / |E|)
//                       with y = 3.7947e-5 sqrt(|E|) / W and
//                       v = 0.956 - 1.062 y^2 (Wang and Loew); the face
//                       values are summed, as the reference does.
#pragma once

#include <cmath>

#include "picgpu.h"

#ifdef __CUDACC__
#define PG_EM_HD __host__ __device__
#else
#define PG_EM_HD
#endif

namespace pg {

constexpr double kRichardsonA0 = 1201732.101;       // 4 pi m k^2 e / h^3 [A m^-2 K^-2]
constexpr double kFowlerA = 1.541434e-6;            // [A eV V^-2]
constexpr double kFowlerB = 6.830889776e9;          // [eV^-3/2 V m^-1]
constexpr double kEmitKb = 1.380649e-23;

// e^x in fixed FP64 operations: x = k ln2 + r (ln 2 in two parts,
// |r| <= ln2/2), e^r by its Taylor series to r^17, then 2^k; 0 below -745.
PG_EM_HD inline double emission_exp(double x) {
    if (x < -745.0) return 0.0;
    const double ln2_hi = 0.6931471805599452862, ln2_lo = 2.3190468138462996e-17;
    const double k = rint(x / ln2_hi);
    const double r = (x - k * ln2_hi) - k * ln2_lo;
    double p = 1.0 / 355687428096000.0;
    const double inv[16] = {20922789888000.0, 1307674368000.0, 87178291200.0, 6227020800.0, 479001600.0,
                            39916800.0, 3628800.0, 362880.0, 40320.0, 5040.0, 720.0, 120.0, 24.0, 6.0, 2.0, 1.0};
    for (int i = 0; i < 16; ++i) p = p * r + 1.0 / inv[i];
    p = p * r + 1.0;
    return ldexp(p, int(k));
}

// Fowler-Nordheim current density of one face: E the boundary field, n the
// outward unit normal, W the work function [eV] (t = 1).
PG_EM_HD inline double fowler_nordheim_face(const double* E, const double* n, double W) {
    if (!(E[0] * n[0] + E[1] * n[1] + E[2] * n[2] > 0.0)) return 0.0;
    const double magE = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
    const double y = 3.7947e-5 * sqrt(magE) / W;
    const double v = 0.956 - 1.062 * y * y;
    const double sw = sqrt(W);
    return kFowlerA * magE * magE / W * emission_exp(-(kFowlerB * v * sw * sw * sw / magE));
}

// qe: the electron species' |charge| (the reference takes the cloud's).
inline double thermionic_current(double lambda_r, double T, double W, double qe) {
    return lambda_r * kRichardsonA0 * T * T * std::exp(-(W * qe / (T * kEmitKb)));
}

// Sum over the patch faces in the device's fixed order: 256 lanes, lane t
// adds faces t, t + 256, ... in turn, then a halving tree over the lanes.
constexpr int kEmissionLanes = 256;

template <class F>
inline double emission_face_sum(int n, F&& value) {
    double lane[kEmissionLanes];
    for (int t = 0; t < kEmissionLanes; ++t) {
        double a = 0.0;
        for (int i = t; i < n; i += kEmissionLanes) a = a + value(i);
        lane[t] = a;
    }
    for (int s = kEmissionLanes / 2; s > 0; s >>= 1)
        for (int t = 0; t < s; ++t) lane[t] = lane[t] + lane[t + s];
    return lane[0];
}

}  // namespace pg
