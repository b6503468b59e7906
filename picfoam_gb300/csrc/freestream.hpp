// freestream.hpp -- the per-face set-up of the FreeStream boundary model
// (PICMCCFVM/submodels/BoundaryModel/FreeStream/FreeStream.C:126-396),
// shared by the device path and the oracle so both start from the same
// numbers.  Host code only.
#pragma once

#include <cmath>
#include <string>
#include <vector>

#include "hexmesh.hpp"
#include "picgpu.h"

namespace pg {

// One FreeStream model: its patch's boundary faces in face order and, per
// face and species (index f * n_species + j), the parcels added to the face
// accumulator each step and the speed ratio s = U . n_in / c_mp.
struct FreeStreamFaces {
    int n_faces = 0, n_species = 0;
    std::vector<int> cell;          // owner cell
    std::vector<int> tet0;          // local tet of the face's first triangle (2 * local face)
    std::vector<double> frac0;      // first triangle's share of the face area
    std::vector<double> n_in;       // 3 per face: inward unit normal
    std::vector<double> t1, t2;     // 3 per face: tangents
    std::vector<double> add;        // n_faces * n_species: parcels per step (Bird eq. 4.22)
    std::vector<double> s;          // n_faces * n_species: speed ratio of the drift along n_in
    std::vector<double> c_mp;       // per species: most probable speed sqrt(2kT/m)
    std::vector<double> v_t;        // per species: sqrt(kT/m)
};

constexpr double kFreeStreamKb = 1.380649e-23;

inline std::string check_freestream(const HexMesh& m, const picgpu_config& cfg, const picgpu_freestream& fs) {
    if (fs.patch < 0 || fs.patch >= int(m.patches.size())) return "freestream: patch out of range";
    if (m.patches[fs.patch].p.kind != PICGPU_PATCH_ABSORB)
        return "freestream: the patch must be of kind ABSORB (FreeStream deletes the parcels reaching it)";
    if (m.patches[fs.patch].n_faces == 0) return "freestream: the patch has no faces";
    if (fs.n_species < 1 || fs.n_species > PICGPU_MAX_SPECIES) return "freestream: n_species must be 1..4";
    for (int j = 0; j < fs.n_species; ++j) {
        if (fs.species[j] < 0 || fs.species[j] >= cfg.n_species) return "freestream: species out of range";
        if (!(fs.number_density[j] >= 0.0)) return "freestream: negative number density";
    }
    if (!(fs.temperature > 1e-300)) return "freestream: zero boundary temperature";  // FreeStream.C:176-183
    return "";
}

inline FreeStreamFaces freestream_faces(const HexMesh& m, const picgpu_config& cfg, const picgpu_freestream& fs) {
    FreeStreamFaces F;
    F.n_species = fs.n_species;
    const double sqrt_pi = std::sqrt(3.14159265358979323846);
    for (int j = 0; j < fs.n_species; ++j) {
        const double mass = cfg.species[fs.species[j]].mass;
        F.c_mp.push_back(std::sqrt(2.0 * kFreeStreamKb * fs.temperature / mass));
        F.v_t.push_back(std::sqrt(kFreeStreamKb * fs.temperature / mass));
    }
    for (const BFace& b : m.bfaces) {
        if (b.patch != fs.patch) continue;
        const double* off = &m.cls_offset[size_t(m.cell_class[b.cell]) * 24];
        const int t0 = 2 * b.local_face;
        double tri_area[2];
        for (int k = 0; k < 2; ++k) {
            const double* A = off + 3 * m.tt.tri[t0 + k][0];
            const double* B = off + 3 * m.tt.tri[t0 + k][1];
            const double* C = off + 3 * m.tt.tri[t0 + k][2];
            const double u[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
            const double v[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
            const double w[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
            tri_area[k] = 0.5 * std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        }
        F.cell.push_back(b.cell);
        F.tet0.push_back(t0);
        F.frac0.push_back(tri_area[0] / b.area);
        double n[3], t1[3], t2[3];
        for (int a = 0; a < 3; ++a) n[a] = -b.normal[a];
        // tangent from the face centre's offset to the face's first point
        // (the first point of its first triangle), then n x t1
        const double* P0 = off + 3 * m.tt.tri[t0][0];
        for (int a = 0; a < 3; ++a) t1[a] = b.centre[a] - (m.cc[3 * size_t(b.cell) + a] + P0[a]);
        const double m1 = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
        for (int a = 0; a < 3; ++a) t1[a] = t1[a] / m1;
        t2[0] = n[1] * t1[2] - n[2] * t1[1];
        t2[1] = n[2] * t1[0] - n[0] * t1[2];
        t2[2] = n[0] * t1[1] - n[1] * t1[0];
        const double m2 = std::sqrt(t2[0] * t2[0] + t2[1] * t2[1] + t2[2] * t2[2]);
        for (int a = 0; a < 3; ++a) {
            t2[a] = t2[a] / m2;
            F.n_in.push_back(n[a]);
            F.t1.push_back(t1[a]);
            F.t2.push_back(t2[a]);
        }
        const double un = fs.velocity[0] * n[0] + fs.velocity[1] * n[1] + fs.velocity[2] * n[2];
        for (int j = 0; j < fs.n_species; ++j) {
            const double w = cfg.species[fs.species[j]].weight;
            const double s = un / F.c_mp[j];
            const double shape = std::fma(sqrt_pi * s, 1.0 + std::erf(s), std::exp(-(s * s)));
            F.add.push_back(b.area * (fs.number_density[j] / w) * cfg.dt * F.c_mp[j] * shape / (2.0 * sqrt_pi));
            F.s.push_back(s);
        }
        ++F.n_faces;
    }
    return F;
}

}  // namespace pg
