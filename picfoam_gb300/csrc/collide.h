// collide.h -- collision step (cell sort, null-collision MCC, Coulomb).
#pragma once

#include <string>

#include "common.cuh"

namespace pgd {

// Device state owned by the collision step.
struct CollideState {
    int enabled = 0;
    double* svmax = nullptr;      // (sigma v)_max per cell
    double* remainder = nullptr;  // collision remainder per cell
    double* xs = nullptr;         // 4 x n_xs: energy, elastic, excitation, ionisation
    int n_xs = 0;
    int* cell_start = nullptr;    // per species: n_cells + 1 offsets of the sorted store
    int* cell_count = nullptr;
    int* cell_cursor = nullptr;
    int* perm = nullptr;          // sorted slot -> old slot
    long perm_cap = 0;
    unsigned long long* counts = nullptr;  // 8 counters
    int* new_count = nullptr;              // appended particles per species
};

struct CollideArgs {
    DMesh m;
    const picgpu_config* cfg;
    long long step;
    int n_species;
    bool mixed;
    DSpecies sp[PICGPU_MAX_SPECIES];
    DSpecies alt[PICGPU_MAX_SPECIES];
    long n[PICGPU_MAX_SPECIES];
    long cap[PICGPU_MAX_SPECIES];
    double* cc_data;
    double* vtx_data;
    long long* cc_fix;
    long long* vtx_fix;
    double fix_scale;
    cudaStream_t stream;
};

cudaError_t collide_set_tables(const TetConst& t);
// Returns a picgpu_status; msg describes a failure.
int collide_init(CollideState& st, const picgpu_config& cfg, const DMesh& m, cudaStream_t s, std::string* msg);
void collide_free(CollideState& st);
// counts: candidates, elastic, excitation, ionisation, coulomb pairs.
int run_collisions(CollideState& st, const CollideArgs& a, int64_t counts[8], long newn[],
                   int swapped[], std::string* msg, int64_t* launches, double* phase_ms);

}  // namespace pgd
