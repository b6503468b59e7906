// collide.h -- collision step (cell occupancy, electron- and ion-neutral
// null-collision MCC, binary Coulomb collisions).
#pragma once

#include <string>

#include "common.cuh"

namespace pgd {

// A secondary staged by the MCC kernels: the ionising electron's position
// (the new electron's), the new ion's position (the electron's with a
// background gas, the neutral parcel's otherwise) and their velocities.
struct Secondary {
    int32_t tet;
    int32_t flag;         // bit 0: electron, bit 1: ion
    double y[3];
    double ue[3];
    double ui[3];
    int32_t tet_i;
    int32_t pad;
    double y_i[3];
};

// Electron-neutral null-collision MCC against the background gas
// (ElectronNeutralCollisionModel.C:703-829) for one step: the per-cell
// candidate counts, remainders, (sigma v)_max, tables and the staging of
// secondaries.
struct MccParams {
    int n_cells;
    const int* e_start;   // n_cells + 1
    const int* e_idx;
    double* svmax;
    double* rem;
    const double* xs;     // 4 x n_xs
    const float* xs32;    // the same tables in FP32 (FP32 store), or null
    float me_c2_eV;       // electron rest energy m c^2 / e [eV] (FP32 kernel)
    int n_xs;
    double n_gas, vth_gas, mg, me, dt;
    double drift[3];
    double ex_th, iz_th;
    double wEwN, wNwE;
    int create_e, create_i;
    int relativistic;     // RelativisticElectronNeutral scattering
    uint64_t seed;
    uint32_t step;
    const int* cand_off;  // n_cells + 1
    unsigned long long* counts;
    long stage_cap;       // staging slots; a cell whose candidates do not fit drops its secondaries
    int* overflow;        // raised when that happens
    unsigned long long* iz_cell;  // optional ionisations per cell
    const unsigned* step_dev;     // optional: the step index read on the device (graph replays)
};

// A parcel made by PairMerging, staged per cell until it is appended.
struct MergedParcel {
    int32_t tet;
    int32_t pad;
    double y[3];
    double U[3];
    double nw;
};

// An electron parcel added by a Perez ionisation, staged with its sort key
// (cell << 32 | collision ordinal << 6 | ionisation level): appended in key
// order, the order picFoam's sequential loop adds them in.
struct PerezElectron {
    unsigned long long key;
    int32_t tet;
    int32_t pad;
    double y[3];
    double U[3];
    double nw;
};

// Counters of one collision step: background MCC candidates, elastic,
// excitation, ionisation (0-3); Coulomb pairs (4); ion background MCC
// candidates, elastic, charge exchange (5-7); binary (neutral) pairs tested,
// collisions; background tests, collisions (8-11); neutral parcels deleted
// by ionisation (12); electron - neutral parcel candidates, elastic,
// excitation, ionisation (13-16); ion - neutral parcel candidates, elastic,
// charge exchange (17-19).
// Perez ionisation: ionising collisions, electrons added (20-21).
constexpr int kCollideCounts = 22;
constexpr int kCountMccParcel = 13;
constexpr int kCountIonParcel = 17;

// Device state owned by the collision step.
struct CollideState {
    int enabled = 0;
    double* svmax = nullptr;      // (sigma v)_max per cell
    double* remainder = nullptr;  // collision remainder per cell
    double* xs = nullptr;         // 4 x n_xs: energy, elastic, excitation, ionisation
    float* xs32 = nullptr;        // the same in FP32 (FP32 store)
    int n_xs = 0;
    double* isvmax = nullptr;     // ion-neutral (sigma v)_max per cell
    double* iremainder = nullptr; // ion-neutral collision remainder per cell
    double* ixs = nullptr;        // 3 x n_ixs: energy, elastic, charge exchange
    int n_ixs = 0;
    int* cell_start = nullptr;    // per species: n_cells + 1 offsets into idx
    int* cell_count = nullptr;
    int* cell_cursor = nullptr;
    int* scan_tmp = nullptr;
    // candidates, elastic, excitation, ionisation, coulomb pairs,
    // ion candidates, ion elastic, ion charge exchange
    unsigned long long* counts = nullptr;
    int* idx[PICGPU_MAX_SPECIES] = {};     // particle indices grouped by cell
    int* sel[PICGPU_MAX_SPECIES] = {};     // pairing permutations (scratch)
    int* sel2[PICGPU_MAX_SPECIES] = {};
    long idx_cap[PICGPU_MAX_SPECIES] = {};
    int* ncand = nullptr;                  // MCC candidates per cell
    int* cand_off = nullptr;               // their staging offsets
    Secondary* stage = nullptr;
    int* flags = nullptr;
    int* pos = nullptr;
    int* stage_tmp = nullptr;
    long stage_cap = 0;
    int* overflow = nullptr;                // staging or store overflow (device-driven step)
    double svmax_init = 0.0;                // initial (sigma v)_max of the electron MCC
    double* psvmax = nullptr;               // electron - neutral parcel (sigma_T c_R)_max per cell
    double* premainder = nullptr;           // and its collision remainder per cell
    double* ipsvmax = nullptr;              // ion - neutral parcel (sigma_T c_R)_max per cell
    double* ipremainder = nullptr;
    int* n_live = nullptr;                  // neutral parcels per cell left after the electron - parcel step
    int mcc_block = 128;                    // threads per block of the MCC kernel (one cell each)
    unsigned long long* iz_cell = nullptr;  // MCC ionisations per cell (accumulated)
    // BinaryCollisionModel: (sigma_T c_r)_max, selection and background
    // remainders per cell; per-cell segments of the combined neutral list
    double* bsmax = nullptr;
    double* brem = nullptr;
    double* bbgrem = nullptr;
    int* blist = nullptr;
    int* boct = nullptr;
    long bcap = 0;
    // PairMerging: parcel speeds in list order, staged merged parcels and
    // their per-cell counts and offsets, counters (merged, checked) and the
    // kinetic-energy change
    double* mspeed = nullptr;
    long mspeed_cap = 0;
    MergedParcel* mstage = nullptr;
    long mstage_cap = 0;
    int* mcount = nullptr;
    int* moff = nullptr;
    unsigned long long* mcounts = nullptr;
    double* mkin = nullptr;
    // Perez ionisation: tables (cs, transferred, lost energy per charge
    // state and 100 energies) per species, staged electrons and their count
    double* ptab[PICGPU_MAX_SPECIES] = {};
    int patomic[PICGPU_MAX_SPECIES] = {};
    int plimit[PICGPU_MAX_SPECIES] = {};
    PerezElectron* pstage = nullptr;
    long pstage_cap = 0;
    unsigned long long* pcount = nullptr;
};

struct CollideArgs {
    DMesh m;
    const picgpu_config* cfg;
    long long step;
    int n_species;
    bool mixed;
    DSpecies sp[PICGPU_MAX_SPECIES];
    long n[PICGPU_MAX_SPECIES];
    long cap[PICGPU_MAX_SPECIES];
    cudaStream_t stream;
};

cudaError_t collide_set_tables(const TetConst& t);
// Returns a picgpu_status; msg describes a failure.
int collide_init(CollideState& st, const picgpu_config& cfg, const DMesh& m, cudaStream_t s, std::string* msg);
void collide_free(CollideState& st);
// Reorder species s into cell order (stable within a cell), dropping removed
// particles: src -> dst, *kept = particles written.
int sort_species(CollideState& st, const DMesh& m, int s, const DSpecies& src, const DSpecies& dst, long n,
                 bool mixed, long* kept, cudaStream_t stream, std::string* msg, int64_t* launches);
// counts: kCollideCounts counters (see above); newn
// receives the species counts after MCC secondaries were appended.
int run_collisions(CollideState& st, const CollideArgs& a, int64_t counts[kCollideCounts], long newn[], int swapped[],
                   std::string* msg, int64_t* launches, double* phase_ms);

// Device-driven form of run_collisions for a step captured in a CUDA graph:
// the species counts n_dev[s] stay on the device (MCC secondaries are
// appended there, first_dev[s] receiving the count before them), nothing is
// read back, and the counts in st.counts accumulate over steps.  Staging and
// lists are sized by collide_reserve_device from the species capacities a.cap;
// a step that would need more raises st.overflow and drops secondaries.
int collide_reserve_device(CollideState& st, const CollideArgs& a, std::string* msg);
int run_collisions_device(CollideState& st, const CollideArgs& a, int* n_dev, int* first_dev,
                          const unsigned* step_dev, std::string* msg, int64_t* launches);

// PairMerging (PairMerging::mergeParticles, PairMerging.C:71-259) of species
// s, entry li of the merge list, over the parcels in slots [0, a.n[s]) (the
// cell occupancy of the step; parcels created by this step's collisions do
// not take part): merged pairs are removed from the store (tet = -1) and the
// new parcels staged; *total receives their number.  merge_append then
// writes them to slots [first, first + total) of a.sp[s] (room reserved by
// the caller), with nParticle and charge modifier 1 (PICCloud::addNewParcel).
int merge_select(CollideState& st, const CollideArgs& a, int li, int s, long long* total, std::string* msg,
                 int64_t* launches);
int merge_append(CollideState& st, const CollideArgs& a, int s, long first, long long total, std::string* msg,
                 int64_t* launches);
// Merged parcels, candidates checked and the kinetic-energy change of the
// merges since the last call (and resets them).
int merge_counters(CollideState& st, cudaStream_t s, long long* merged, long long* checked, double* kin_err);

// The background MCC of the FP32 store in FP32 arithmetic with Nanbu
// scattering (mcc_fp32.cu): one thread per cell as mcc_kernel, the same
// candidate count, staging and counters; collisions and secondaries agree
// with the FP64 kernel statistically.
void launch_mcc_fp32(const MccParams& M, const DSpecies& el, Secondary* stage, int block, cudaStream_t s);

}  // namespace pgd
