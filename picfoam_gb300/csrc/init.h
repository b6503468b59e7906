// init.h -- particle initial conditions on the device (host declarations).
#pragma once

#include "common.cuh"

namespace pgd {

// Per-species sampling of one placement launch.
struct InitSpecies {
    double req_coef;      // per-tet models: particles per m^3 of tet = n / w (applied as (n V) / w)
    double n, w;          // number density, weight
    double scale[3];      // U = scale (x) N(0,1)^3 + drift
    double drift[3];
    double speed;         // QuasineutralPlasma without Maxwellian: |U|
    double displacement;  // UniformDisplacement
    int cell_count;       // QuasineutralPlasma: parcels per cell
    int pad;
};

struct InitParams {
    DMesh m;
    int model;            // PICGPU_INIT_*
    int species;
    int constrain;        // any empty axis: zero those coordinates of the point and relocate it in its cell
    int use_maxwellian;
    uint64_t seed;
    InitSpecies sp;
    const double* tet_vol;    // 12 per geometry class
    // UniformDisplacement lattice
    long long nl[3];
    double lo[3], delta[3], dir[3], span_len, cycles;
    double grid_lo[3], grid_hi[3];
    int grid_n[3];
    const int* grid_cell;     // block cell -> cell id or -1
    // output (FP64 or FP32 store of this species, from slot `first`)
    long long first;
    int32_t* tet;
    double* y64[3];
    double* u64[3];
    float* y32[3];
    float* u32[3];
    int* error;               // set to 1 when a point falls outside the mesh
};

cudaError_t init_set_tables(const TetConst& t);
// Per-tet models (Equipartition, Maxwellian, Isotropization): counts per
// cell, their exclusive scan (64-bit offsets; offsets[n_cells] = total).
void launch_init_count(const InitParams& P, int* counts, cudaStream_t s);
cudaError_t init_scan(const int* counts, long long* offsets, long long* block_sums, int n, cudaStream_t s);
long long init_scan_scratch(int n);
void launch_init_fill_tets(const InitParams& P, const long long* offsets, cudaStream_t s);
// QuasineutralPlasma: sp.cell_count parcels in every cell.
void launch_init_fill_cells(const InitParams& P, cudaStream_t s);
// UniformDisplacement: nl[0] x nl[1] x nl[2] lattice points.
void launch_init_fill_lattice(const InitParams& P, cudaStream_t s);
// Particles per cell of a store (tet >= 0 slots of [0, n)) -> counts (zeroed first).
void launch_init_occupancy(const int32_t* tet, long long n, int n_cells, int* counts, cudaStream_t s);
// min, max and sum of counts[0..n) -> out[0..2].
void launch_init_minmax(const int* counts, int n, long long* out, cudaStream_t s);

// SimpleInjection through the ParticleEmitter: n parcels of one species on
// one patch's face triangles.
struct InjectParams {
    DMesh m;
    uint64_t seed;
    uint32_t step;
    int injector, species, model, constrain;
    double mass, temperature;     // [kg], [K]
    long long n;
    int n_tri;
    const double* tri_cum;        // n_tri + 1 cumulative triangle areas, tri_cum[0] = 0
    const int* tri_cell;          // owner cell of triangle i
    const int* tri_tet;           // local tet (2 face + k) whose face triangle it is
    const double* tri_normal;     // 3 per triangle: outward unit face normal
    const double* tri_fc;         // 3 per triangle: face centre
    double area;                  // patch area (sum of the face areas)
    double* qconv;                // floating patch charge (nullptr otherwise)
    int patch;
    double ejected_charge;        // n q w, taken off qconv[patch]
    long long first;
    int32_t* tet;
    double* y64[3];
    double* u64[3];
    float* y32[3];
    float* u32[3];
    int* error;
};
void launch_inject(const InjectParams& P, cudaStream_t s);

// FreeStream (FreeStream.C:126-396) for one model and one of its species:
// the per-face accumulators and counts, then the parcels of every face at
// first + offsets[f] (the exclusive scan of the counts).
struct FreeStreamParams {
    DMesh m;
    uint64_t seed;
    uint32_t step;
    int injector, species, j, n_species, n_faces;
    const int* cell;          // per face: owner cell
    const int* tet0;          // per face: local tet of its first triangle
    const double* frac0;      // per face: first triangle's area share
    const double* n_in;       // 3 per face
    const double* t1;
    const double* t2;
    const double* add;        // n_faces * n_species
    const double* s;          // n_faces * n_species
    double c_mp, v_t, U[3];
    double* acc;              // n_faces * n_species accumulators
    int* counts;              // n_faces
    const long long* offsets; // n_faces + 1
    long long first;
    int32_t* tet;
    double* y64[3];
    double* u64[3];
    float* y32[3];
    float* u32[3];
    int* error;               // set to 2 when one face would emit more than 2^30 parcels
};
void launch_freestream_count(const FreeStreamParams& P, cudaStream_t s);
void launch_freestream_emit(const FreeStreamParams& P, cudaStream_t s);

}  // namespace pgd
