/*
 * oracle.h -- CPU oracle of the picFoam particle hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain C++ restatement of the
 * picFoam algorithms (push, barycentric tracking with patch interaction,
 * charge and field weighting, the electrostatic Poisson solve, null-collision
 * MCC, binary Coulomb collisions) used as the checker for the CUDA library
 * and as the timed CPU baseline.  Nothing in the product links or loads it.
 *
 * The API mirrors include/picgpu.h so one test can drive both sides with the
 * same inputs.  Parity status: the picFoam source cannot be built here (it
 * needs OpenFOAM-9, wmake and MPI) and ships no test vectors, so the oracle
 * is pinned by analytic known-answer tests (gyration radius, E x B drift,
 * plasma frequency, manufactured Poisson solutions, collision rates) rather
 * than by reference outputs: "parity unpinned" against picFoam binaries.
 */
#ifndef PICGPU_ORACLE_H
#define PICGPU_ORACLE_H

#include "picgpu.h"
#include "picgpu_init.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

/* Preconditioner of the oracle's PCG. */
enum {
    ORACLE_PRECOND_JACOBI = 0,  /* same arithmetic and reduction order as the GPU */
    ORACLE_PRECOND_DIC = 1      /* OpenFOAM PCG/DIC (tutorial fvSolution), sequential sums */
};

int  oracle_create(const picgpu_mesh_desc* mesh, const picgpu_config* cfg, int nthreads,
                   oracle_ctx** out);
void oracle_destroy(oracle_ctx* ctx);
const char* oracle_last_error(const oracle_ctx* ctx);
int  oracle_set_precond(oracle_ctx* ctx, int precond);
int  oracle_mesh_query(const oracle_ctx* ctx, picgpu_mesh_info* info);
int  oracle_mesh_selfcheck(const picgpu_mesh_desc* desc, double* out, int n_out);
int  oracle_set_step_index(oracle_ctx* ctx, int64_t steps_done);
int  oracle_compute_field(oracle_ctx* ctx);
int  oracle_set_particles(oracle_ctx* ctx, int species, size_t n, const int32_t* tet,
                          const double* bary, const double* U);
int  oracle_set_parcel_attributes(oracle_ctx* ctx, int species, size_t n, const double* nParticle,
                                  const int32_t* chargeModifier);
int  oracle_get_parcel_attributes(oracle_ctx* ctx, int species, size_t cap, double* nParticle,
                                  int32_t* chargeModifier, size_t* n);
int  oracle_count_particles(oracle_ctx* ctx, int species, size_t* n);
int  oracle_get_particles(oracle_ctx* ctx, int species, size_t cap, int32_t* tet,
                          double* bary, double* U, size_t* n);
int  oracle_initialise_fields(oracle_ctx* ctx);
/* picInitialise restated (picgpu_initialise's oracle): places the particles
 * of `init` in picFoam's order, reports the statistics, computes the fields,
 * optionally solves them and applies the leapfrog back-step. */
int  oracle_initialise(oracle_ctx* ctx, const picgpu_init* init, picgpu_init_stats* stats);
double oracle_det_log(double x);
/* SimpleInjection boundary models (picgpu_set_injection's oracle). */
int  oracle_set_injection(oracle_ctx* ctx, int n, const picgpu_injection* inj);
/* FreeStream boundary models (picgpu_set_freestream's oracle). */
int  oracle_set_freestream(oracle_ctx* ctx, int n, const picgpu_freestream* fs);
/* EmissionModels (picgpu_set_emission's oracle). */
int  oracle_set_emission(oracle_ctx* ctx, int n, const picgpu_emission* em);
double oracle_det_sin(double x);
int  oracle_step(oracle_ctx* ctx, int nsteps, picgpu_step_stats* stats);
int  oracle_move(oracle_ctx* ctx, picgpu_step_stats* stats);
int  oracle_solve_poisson(oracle_ctx* ctx, const double* rho, double* phi_inout,
                          picgpu_step_stats* stats);
int  oracle_get_field(oracle_ctx* ctx, int which, double* out, size_t n);
int  oracle_set_field(oracle_ctx* ctx, int which, const double* in, size_t n);
int  oracle_diagnostics(oracle_ctx* ctx, picgpu_diagnostics* out);
/* Wall-clock seconds spent in push + track + deposit since creation. */
double oracle_move_seconds(const oracle_ctx* ctx);
/* One Philox4x32-10 block of the collision generator (known-answer checks). */
void oracle_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Debye length of a cell over the Coulomb-colliding species for the current
 * particles (CoulombCollisionModel.C:249-309); 0 when undefined. */
double oracle_debye_length(oracle_ctx* ctx, int cell);

/* CPU reference of the learned warm-start U-Net (unet_ref.cpp), same weight
 * and tensor layouts as picgpu_unet_* (include/picgpu_learned.h); FP64, and
 * with emulate = 1 rounded to BF16 wherever the GPU stores BF16. */
size_t oracle_unet_param_count(void);
int oracle_unet_forward(int X, int Y, int Z, const float* w, const float* in, int emulate, double* out);
int oracle_unet_gradients(int X, int Y, int Z, const float* w, const float* in, const float* target,
                          const float* mask, int emulate, double* grad, double* loss);

#ifdef __cplusplus
}
#endif
#endif
