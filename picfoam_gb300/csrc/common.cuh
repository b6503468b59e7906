// common.cuh -- device-side types shared by the picgpu kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "picgpu.h"

namespace pgd {

constexpr double kC = 299792458.0;
constexpr double kPi = 3.14159265358979323846;
constexpr int kMaxPatches = PICGPU_MAX_BOXES + 6;
// FP32 form: barycentric charge weights are accumulated as integers in units
// of 2^-kDepositBits (32 lanes x 2^25 still fits a 32-bit warp sum).
constexpr int kDepositBits = 25;

// Tet tables of the canonical hex (see hexmesh.hpp), in constant memory.
struct TetConst {
    int8_t tri[12][3];
    int8_t inner_next[12][4];
    int8_t inner_src[12][4][4];
    int8_t cross_next[12];
    int8_t cross_src[12][4];
};

// Patch data in constant memory.
struct PatchConst {
    int n;
    int kind[kMaxPatches];
    int phi_bc[kMaxPatches];
    double phi[kMaxPatches];
    double area[kMaxPatches];
    double rlc_k[kMaxPatches];   // RLCBoundary cathode: a0 * epsilon * area (0 elsewhere)
};

// Shared-memory tables of the FP32 move kernel: the geometry of a uniform
// block mesh and the tet-crossing tables packed as
//   bits 0-3 new local tet, bits 4+3j..6+3j source of coordinate j (7: zero).
struct Tables32 {
    float inv[108];
    float normal[18];
    float off[24];
    unsigned inner[48];
    unsigned cross[12];
    unsigned tri[12];            // corners of the face triangle, 4 bits each
    int kind[kMaxPatches];
};

// Read-only mesh arrays on the device.
struct DMesh {
    int n_cells, n_points, n_bfaces, n_classes;
    int empty[3];
    int any_empty;
    double mesh_centre[3];
    const int* cell_class;   // n_cells
    const int* nbr;          // 6 n_cells
    const int* cell_pt;      // 8 n_cells (cyclic-merged points)
    const double* cc;        // 3 n_cells
    const float* cc32;       // 3 n_cells
    const double* vol;       // n_cells
    const double* tetinv;    // 108 per class
    const float* tetinv32;   // 108 per class
    const double* offset;    // 24 per class
    const float* offset32;   // 24 per class
    const double* fnormal;   // 18 per class
    const float* fnormal32;  // 18 per class
    const double* farea;     // 6 per class
    const double* ip_weight; // 6 n_cells
    const int* cell_bface;   // 6 n_cells
    const int* bf_cell;
    const int* bf_patch;
    const double* bf_normal; // 3 per bface
    const double* bf_area;
    const double* bf_delta;
    const double* vw_weight; // 8 n_cells
    const int* pi_start;     // n_points + 1
    const int* pi_src;
    const double* pi_w;
    const double* Mdiag;     // SPD operator -laplacian
    const double* Moff;      // 6 n_cells
    const double* dinv;
    const int* pc_start;     // n_points + 1: point -> cell-corner slots
    const int* pc_slot;
    int uniform;             // one geometry class (block mesh of equal cells)
    int lap_uniform;         // every coupled face in direction f has M coefficient lap_coef[f]
    double lap_coef[6];
};

// Per-species particle storage (structure of arrays).
struct DSpecies {
    int32_t* tet;            // cell*12 + local tet; -1: removed
    double* y64[3];
    double* u64[3];
    float* y32[3];
    float* u32[3];
    // per-parcel weight and charge state (PICParcel nParticle_,
    // chargeModifier_), or null: every parcel has the species weight and
    // charge modifier 1
    double* nw;
    int32_t* zq;
};

// Counters written by the move kernels (one set per launch).
struct MoveCounters {
    unsigned long long tet_steps;
    unsigned long long faces;
    unsigned long long walls;
    unsigned long long absorbed;
    int error;               // PICGPU_TRACK_LOOP_CAP / PICGPU_SPEED_OF_LIGHT
    int pad;
};

// Particles that leave their cell in the FP32 in-cell mover wait for the
// crossing tracker in a per-block segment: block b of the mover wrote
// count[b] particle indices at queue[start[b] ...].
struct CrossQueue {
    int* queue;              // the species' idle double-buffer tet array (capacity >= n)
    int* count;              // per mover block
    int* start;
    int capacity;            // blocks the count / start arrays hold
};

struct MoveParams {
    DMesh m;
    int n;                   // particles in this species (including removed slots)
    int first;               // first slot to process
    const int* n_dev;        // FP32 form: when set, n (and first, from first_dev) are read on the
    const int* first_dev;    // device, so the launch can sit in a CUDA graph
    int species;
    int pusher;
    int field_weighting;
    int charge_distribution;
    int deposit_mode;
    int rotation;
    int solve_movement;
    int sync;
    int max_steps;
    double q, mass, value;   // charge, mass, charge * weight
    double weight;
    double dt;
    double B[3];
    double fix_scale;
    // FP32 form: the same constants pre-rounded on the host, so the kernel
    // never converts a double (GB300 issues FP64 at a small fraction of FP32)
    int charged;             // q != 0
    int has_value;           // q * weight != 0
    float qm_f;              // q / m
    float dt_f;
    float B_f[3];
    float centre_f[3];
    const double* Bc;             // per-cell magnetic field (3 n_cells), or null: the uniform B
    const float4* Bc4;            // FP32 form: the same per cell (xyz), or null
    const Tables32* t32;          // FP32 form: tables of this context's mesh (device memory)
    // FP32 in-cell mover (uniform block meshes): dt / cell size per axis and
    // 1 on solved axes, 0 on empty ones (tracking returns to the centre plane)
    int cell_mover;
    float dth[3], keep[3];
    CrossQueue xq;                // FP32 form: particles at reflecting patches (queue null: general kernel only)
    int reflecting;               // a patch reflects this species (wall, or a circuit electrode for neutrals)
    unsigned long long* acc9;     // this species' 2^-kDepositBits fixed-point deposit per cell: centre + 8 corners
    const float4* Ec4;            // E per cell: centre + 8 corners (FP32 form)
    const double* E;         // 3 n_cells
    const double* Ept;       // 3 n_points
    const float* E32;
    const float* Ept32;
    double* cc_data;         // FP64 accumulators
    double* vtx_data;
    long long* cc_fix;       // fixed-point accumulators
    long long* vtx_fix;
    double* qconv;           // per patch floating charge
    DSpecies p;
    MoveCounters* counters;
};

// Philox4x32-10 (Salmon et al., SC'11): counter-based random stream.
struct Philox {
    uint32_t key0, key1;
    uint32_t c0, c1, c2, c3;
    uint32_t buf[4];
    int used;
    __device__ __forceinline__ Philox(uint64_t seed, uint32_t a, uint32_t b, uint32_t c)
        : key0(uint32_t(seed)), key1(uint32_t(seed >> 32)), c0(0), c1(a), c2(b), c3(c), used(4) {}
    __device__ __forceinline__ void block() {
        uint32_t x0 = c0, x1 = c1, x2 = c2, x3 = c3, k0 = key0, k1 = key1;
#pragma unroll
        for (int r = 0; r < 10; ++r) {
            const uint32_t lo0 = 0xD2511F53u * x0, hi0 = __umulhi(0xD2511F53u, x0);
            const uint32_t lo1 = 0xCD9E8D57u * x2, hi1 = __umulhi(0xCD9E8D57u, x2);
            const uint32_t n0 = hi1 ^ x1 ^ k0, n2 = hi0 ^ x3 ^ k1;
            x0 = n0; x1 = lo1; x2 = n2; x3 = lo0;
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        buf[0] = x0; buf[1] = x1; buf[2] = x2; buf[3] = x3;
        c0 += 1;
        used = 0;
    }
    __device__ __forceinline__ uint32_t u32() {
        if (used >= 4) block();
        return buf[used++];
    }
    __device__ __forceinline__ double uniform() {
        const uint32_t a = u32() >> 5, b = u32() >> 6;
        return (double(a) * 67108864.0 + double(b)) * (1.0 / 9007199254740992.0);
    }
    __device__ __forceinline__ double uniform_pos() { return 1.0 - uniform(); }
    __device__ __forceinline__ double normal() {
        const double u1 = uniform_pos(), u2 = uniform();
        return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    }
};

enum : uint32_t {
    // PairMerging per (merge-list entry, cell, step); high nibble 0, bit 27 clear
    kStreamMerge = 0u,
    // Perez ionisation per (Coulomb collision ordinal, cell, step)
    kStreamIonize = 1u << 27,
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

}  // namespace pgd

#define PGD_CHECK(call)                                                   \
    do {                                                                  \
        cudaError_t e_ = (call);                                          \
        if (e_ != cudaSuccess) return pgd_fail(e_, #call, __FILE__, __LINE__); \
    } while (0)
