// collisions.hpp -- oracle-side random numbers and cross-section tables.
//
// TEST INFRASTRUCTURE ONLY.  Counter-based Philox4x32-10 (Salmon, Moraes,
// Dror & Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11) gives
// one independent stream per (purpose, cell, time step) so that a cell's
// collision sequence does not depend on the processing order; picFoam draws
// from one sequential Foam::Random (PICCloud.C:931), which only the
// statistics, not the individual draws, can be compared against.
#pragma once

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "picgpu.h"

namespace ocoll {

struct Philox {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    int used = 4;

    Philox(uint64_t seed, uint32_t a, uint32_t b, uint32_t c) {
        key[0] = uint32_t(seed);
        key[1] = uint32_t(seed >> 32);
        ctr[0] = 0;
        ctr[1] = a;
        ctr[2] = b;
        ctr[3] = c;
    }
    static inline void mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
        const uint64_t p = uint64_t(a) * uint64_t(b);
        hi = uint32_t(p >> 32);
        lo = uint32_t(p);
    }
    void block() {
        uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
        uint32_t k0 = key[0], k1 = key[1];
        for (int r = 0; r < 10; ++r) {
            uint32_t hi0, lo0, hi1, lo1;
            mulhilo(0xD2511F53u, c0, hi0, lo0);
            mulhilo(0xCD9E8D57u, c2, hi1, lo1);
            const uint32_t n0 = hi1 ^ c1 ^ k0;
            const uint32_t n1 = lo1;
            const uint32_t n2 = hi0 ^ c3 ^ k1;
            const uint32_t n3 = lo0;
            c0 = n0; c1 = n1; c2 = n2; c3 = n3;
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        buf[0] = c0; buf[1] = c1; buf[2] = c2; buf[3] = c3;
        ctr[0] += 1;
        used = 0;
    }
    uint32_t u32() {
        if (used >= 4) block();
        return buf[used++];
    }
    // uniform in [0, 1) with 53 random bits
    double uniform() {
        const uint32_t a = u32() >> 5, b = u32() >> 6;
        return (double(a) * 67108864.0 + double(b)) * (1.0 / 9007199254740992.0);
    }
    // uniform in (0, 1]
    double uniform_pos() { return 1.0 - uniform(); }
    // standard normal, Box-Muller (cosine branch)
    double normal() {
        const double u1 = uniform_pos(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

enum : uint32_t {
    kStreamMerge = 0u,                   // PairMerging per (merge-list entry, cell, step)
    kStreamIonize = 1u << 27,            // Perez ionisation per (Coulomb collision ordinal, cell, step)
    kStreamMcc = 1u << 28,
    kStreamCoulomb = 2u << 28,
    kStreamRemainder = 3u << 28,
    kStreamIonMcc = 4u << 28,
    kStreamIonRemainder = 5u << 28,
    kStreamInitCount = 6u << 28,      // initial conditions: remainder draw per (species, cell, tet)
    kStreamInitParticle = 7u << 28,   // per (species, cell, tet << 24 | k) or (species, cell, k)
    kStreamInitLattice = 8u << 28,    // per (species, lattice index)
    kStreamInject = 9u << 28,         // per (injector << 4 | species, step, parcel)
    kStreamBinary = 10u << 28,        // neutral pair collisions per (cell, step)
    kStreamBinaryBg = 11u << 28,      // neutral - background collisions per (cell, step)
    kStreamBinaryRemainder = 12u << 28,
    kStreamBinaryBgRemainder = 13u << 28,
    kStreamFreeStreamCount = 14u << 28,  // FreeStream remainder draw per (injector << 4 | species, step, face)
    kStreamFreeStream = 15u << 28,       // FreeStream parcels per (injector << 4 | species, step, face)
};

// The Coulomb stream of a cell and step: the pairing shuffles draw from
// counter block 0 on; the collision of ordinal k (its position in the
// sequential pairing order of the cell) draws from blocks 2^31 + 8k on (a
// collision takes at most three uniforms, two blocks), so that collisions
// with disjoint parcels can run in any order.
inline Philox coulomb_pair_stream(uint64_t seed, uint32_t cell, uint32_t step, long k) {
    Philox p(seed, kStreamCoulomb, cell, step);
    p.ctr[0] = 0x80000000u + uint32_t(k) * 8u;
    return p;
}

// The Perez ionisation draws of the Coulomb collision of ordinal k in a cell
// and step.
inline Philox ionize_stream(uint64_t seed, uint32_t cell, uint32_t step, long k) {
    return Philox(seed, kStreamIonize | uint32_t(k), cell, step);
}

// The sum of f(t), t in [0, n), in the order of a 32-lane warp reduction:
// lane l adds t = l, l + 32, ... from zero, then lanes l < off add lane
// l + off for off = 16, 8, 4, 2, 1; lane 0 holds the sum.
template <class F>
inline double warp_sum(long n, F f) {
    double p[32];
    for (int l = 0; l < 32; ++l) {
        p[l] = 0.0;
        for (long t = l; t < n; t += 32) p[l] += f(t);
    }
    for (int off = 16; off > 0; off >>= 1)
        for (int l = 0; l < off; ++l) p[l] += p[l + off];
    return p[0];
}

// List cross section: interpolateXY (ListCrossSection.C:33-88): linear in
// energy between the bracketing nodes, end values held outside the table.
inline double interp_xs(double x, const std::vector<double>& xs, const std::vector<double>& ys) {
    const int n = int(xs.size());
    if (n == 0) return 0.0;
    if (x <= xs[0]) return ys[0];
    if (x >= xs[n - 1]) return ys[n - 1];
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (xs[mid] <= x) lo = mid; else hi = mid;
    }
    if (xs[lo] == x) return ys[lo];
    return ys[lo] + ((x - xs[lo]) / (xs[hi] - xs[lo])) * (ys[hi] - ys[lo]);
}

struct Tables {
    std::vector<double> e, el, ex, iz;
};

constexpr double kEcharge = 1.602176634e-19;

// Cross-section tables and the (sigma v)_max initialisation
// (ElectronNeutralCollisionModel.C:383-424 FindMaximum), collision remainders
// seeded U(0,1) (ElectronNeutralCollisionModel.C:286-296).
inline std::string init_mcc(const picgpu_config& cfg, Tables& t, int n_cells,
                            std::vector<double>& svmax, std::vector<double>& rem) {
    const picgpu_mcc& m = cfg.mcc;
    if (m.n_xs < 2 || m.n_xs > PICGPU_MAX_XS_POINTS || !m.xs_energy || !m.xs_elastic ||
        !m.xs_excitation || !m.xs_ionization)
        return "mcc: cross-section tables missing";
    if (cfg.electron_species < 0 || cfg.electron_species >= cfg.n_species)
        return "mcc: electron species not set";
    t.e.assign(m.xs_energy, m.xs_energy + m.n_xs);
    t.el.assign(m.xs_elastic, m.xs_elastic + m.n_xs);
    t.ex.assign(m.xs_excitation, m.xs_excitation + m.n_xs);
    t.iz.assign(m.xs_ionization, m.xs_ionization + m.n_xs);
    for (int i = 1; i < m.n_xs; ++i)
        if (!(t.e[i] > t.e[i - 1])) return "mcc: energies must ascend";
    double sv = m.sigma_v_max_init;
    if (!(sv > 0)) {
        const double me = cfg.species[cfg.electron_species].mass;
        const double emax = m.find_max_energy > 0 ? m.find_max_energy : t.e.back();
        const double step = m.find_energy_step > 0 ? m.find_energy_step : emax / 100000.0;
        sv = 0.0;
        for (double eV = 0.0; eV < emax; eV += step) {
            const double q = interp_xs(eV, t.e, t.el) + interp_xs(eV, t.e, t.ex) + interp_xs(eV, t.e, t.iz);
            sv = std::fmax(sv, std::sqrt(2.0 * kEcharge * eV / me) * q);
        }
    }
    svmax.assign(n_cells, sv);
    rem.resize(n_cells);
    for (int c = 0; c < n_cells; ++c) {
        Philox r(cfg.seed, kStreamRemainder, uint32_t(c), 0u);
        rem[c] = r.uniform();
    }
    return "";
}

// Ion-neutral tables (elastic in el, charge exchange in ex) and the
// FindMaximum search with the ion mass (IonNeutralCollisionModel.C:284-333);
// remainders seeded U(0,1) (IonNeutralCollisionModel.C:199).
inline std::string init_ion_mcc(const picgpu_config& cfg, Tables& t, int n_cells,
                                std::vector<double>& svmax, std::vector<double>& rem) {
    const picgpu_ion_mcc& m = cfg.ion_mcc;
    if (m.n_xs < 2 || m.n_xs > PICGPU_MAX_XS_POINTS || !m.xs_energy || !m.xs_elastic || !m.xs_charge_exchange)
        return "ion_mcc: cross-section tables missing";
    if (m.ion_species < 0 || m.ion_species >= cfg.n_species) return "ion_mcc: ion species not set";
    if ((!(cfg.mcc.gas_density > 0) && !m.neutral_parcels) || !(cfg.mcc.gas_mass > 0))
        return "ion_mcc: background gas (mcc.gas_*) not set";
    t.e.assign(m.xs_energy, m.xs_energy + m.n_xs);
    t.el.assign(m.xs_elastic, m.xs_elastic + m.n_xs);
    t.ex.assign(m.xs_charge_exchange, m.xs_charge_exchange + m.n_xs);
    t.iz.clear();
    for (int i = 1; i < m.n_xs; ++i)
        if (!(t.e[i] > t.e[i - 1])) return "ion_mcc: energies must ascend";
    double sv = m.sigma_v_max_init;
    if (!(sv > 0)) {
        const double mi = cfg.species[m.ion_species].mass;
        const double emax = m.find_max_energy > 0 ? m.find_max_energy : t.e.back();
        const double step = m.find_energy_step > 0 ? m.find_energy_step : emax / 100000.0;
        sv = 0.0;
        for (double eV = 0.0; eV < emax; eV += step) {
            const double q = interp_xs(eV, t.e, t.el) + interp_xs(eV, t.e, t.ex);
            sv = std::fmax(sv, std::sqrt(2.0 * kEcharge * eV / mi) * q);
        }
    }
    svmax.assign(n_cells, sv);
    rem.resize(n_cells);
    for (int c = 0; c < n_cells; ++c) {
        Philox r(cfg.seed, kStreamIonRemainder, uint32_t(c), 0u);
        rem[c] = r.uniform();
    }
    return "";
}

}  // namespace ocoll
