/* picgpu_init.h -- particle initial conditions generated on the device.
 *
 * Replaces the picInitialise application (preProcess/picInitialise/
 * picInitialise.C:30-319) for a picgpu context: the InitializationModel
 * selected in system/picInitialiseDict places the particles
 * (initialiseParticles), the statistics block reports occupancy, drift,
 * temperature and number density (picInitialise.C:86-188), the fields are
 * computed and optionally solved (:209-217), and initalizeLeapFrog pushes
 * every velocity back by half a time step (:219-227).  The particles go
 * straight into the context's device store; no host arrays are involved.
 *
 * Random numbers: picFoam draws from one sequential Foam::Random; here every
 * tet (or cell, or lattice point) of every species has its own counter-based
 * Philox4x32-10 stream keyed by `seed`, so the result does not depend on the
 * processing order and the CPU oracle reproduces it bit for bit (FP64 form).
 * Normal variates use Marsaglia's polar method with a logarithm evaluated in
 * fixed FP64 operations (no math library), points in a tet the folding
 * method of Rocchini & Cignoni (J. Graphics Tools 5(4), 2000).
 */
#ifndef PICGPU_INIT_H
#define PICGPU_INIT_H

#include "picgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* InitializationModel (TypeName in each model's .H) */
enum {
    PICGPU_INIT_NONE = 0,                 /* none: no particles (NoParticleInitialization) */
    PICGPU_INIT_EQUIPARTITION = 1,        /* Equipartition (EquipartitionInitialization.C:65-141) */
    PICGPU_INIT_MAXWELLIAN = 2,           /* Maxwellian (MaxwellianInitialization.C:73-126) */
    PICGPU_INIT_ISOTROPIZATION = 3,       /* Isotropization (IsotropizationInitialization.C:52-123) */
    PICGPU_INIT_QUASINEUTRAL_PLASMA = 4,  /* QuasineutralPlasma (QuasineutralPlasmaInitialization.C:38-175) */
    PICGPU_INIT_UNIFORM_DISPLACEMENT = 5  /* UniformDisplacement (UniformInitialization.C:51-127) */
};

typedef struct {
    int32_t model;               /* PICGPU_INIT_* */
    int32_t clear_particles;     /* clearParticles: 1 replaces the population, 0 appends to it */
    int32_t solve_fields;        /* solveMaxwellEquations: solve the potential after the charge deposit */
    int32_t leapfrog;            /* initalizeLeapFrog: every velocity pushed by -dt/2 once */
    /* readDefaultSettings (InitializationModel.C:61-110); temperatures in K
     * (electronVolt: multiply by e/k before) */
    double  number_density[PICGPU_MAX_SPECIES];   /* numberDensities [1/m^3] */
    double  temperature[PICGPU_MAX_SPECIES];      /* temperature [K] */
    /* Equipartition */
    double  velocity[3];                          /* drift added to every species [m/s] */
    /* Maxwellian: per species, U_i = thermalVelocity_i N(0,1) + driftVelocity_i */
    double  drift_velocity[PICGPU_MAX_SPECIES][3];
    double  thermal_velocity[PICGPU_MAX_SPECIES][3];
    /* Isotropization */
    double  tperp_over_tpara;                     /* Tperp_over_Tpara */
    /* QuasineutralPlasma */
    double  cell_count;                           /* cellCount: physical particles per cell and species */
    int32_t ion_species;                          /* ionSpecies (electrons: the config's electron_species) */
    int32_t use_maxwellian;                       /* useMaxwellian: 1 Maxwellian, 0 fixed speed sqrt(3kT/m) */
    /* UniformDisplacement */
    int32_t species_mask;                         /* bit s set: species s gets a lattice (species list) */
    int32_t use_bounds;                           /* 1: min / max below; 0: the mesh bounds */
    double  min[3], max[3];
    int64_t particle_numbers[3];                  /* particleNumbers */
    double  displacement_dir[3];                  /* displacementDir (normalised here) */
    double  displacement[PICGPU_MAX_SPECIES];     /* displacement per species [m] */
    double  cycles;
    uint64_t seed;
} picgpu_init;

typedef struct {
    int64_t added[PICGPU_MAX_SPECIES];            /* particles placed per species */
    double  occupancy_avg[PICGPU_MAX_SPECIES];    /* particles per cell after placement */
    int64_t occupancy_min[PICGPU_MAX_SPECIES];
    int64_t occupancy_max[PICGPU_MAX_SPECIES];
    double  drift[PICGPU_MAX_SPECIES][3];         /* weighted mean velocity [m/s] */
    double  temperature[PICGPU_MAX_SPECIES];      /* calculated m/(3k)(<|U|^2> - |drift|^2) [K] */
    double  number_density[PICGPU_MAX_SPECIES];   /* calculated sum(nParticle) / mesh volume [1/m^3] */
    double  model_temperature[PICGPU_MAX_SPECIES];    /* the model's: calculated or given (picInitialise.C:146-147) */
    double  model_number_density[PICGPU_MAX_SPECIES]; /* the model's: calculated or given (:170-171) */
    double  mesh_volume;                          /* [m^3] */
    double  debye_length;                         /* from the model's n and T of the charged species [m] */
    double  average_cell_size;                    /* mean cube root of the cell volumes [m] */
    double  plasma_frequency_dt;                  /* electron plasma frequency x dt */
    double  place_ms;                             /* device time of the placement kernels */
} picgpu_init_stats;

/* picInitialise for a context: place the particles of `init` on the device
 * (the context's particle store; clear_particles replaces it), report the
 * statistics, deposit the charge and compute the fields (solve_fields: with
 * the Poisson solve), then optionally the leapfrog back-step.  Errors:
 * PICGPU_INVALID_ARG (unknown model or species, a lattice point outside the
 * mesh, QuasineutralPlasma without opposite charges of equal magnitude),
 * PICGPU_CAPACITY (more than 2^31 particles of a species, or more than
 * 2^24 in one tet). */
picgpu_status picgpu_initialise(picgpu_ctx* ctx, const picgpu_init* init, picgpu_init_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* PICGPU_INIT_H */
