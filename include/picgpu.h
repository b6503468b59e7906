/*
 * picgpu.h -- C ABI of the GB300-native picFoam particle hot path.
 *
 * One context (picgpu_ctx) owns a device-resident PIC/MCC case: a hex mesh,
 * structure-of-arrays particle storage per species, the electric potential
 * and field, and the sub-model selection.  Every entry point takes plain
 * pointers and sizes, returns a picgpu_status and never aborts or traps.
 *
 * Each entry point replaces a run-time-selected picFoam sub-model call or a
 * whole-population loop of the PICCloud evolve step (paths are relative to
 * the picFoam source tree):
 *
 *   picgpu_create            PICCloud constructor + sub-model selection
 *                            (PICMCCFVM/clouds/Templates/PICCloud/PICCloud.C:378-518)
 *   picgpu_set_particles     picInitialise parcel creation / PICCloud::addNewParcel
 *                            (PICCloud.C:707-723)
 *   picgpu_step              PICCloud::evolve (PICCloud.C:1426-1471): move (push,
 *                            track, patch interaction), collisions, calculateFields,
 *                            boundary pre/post updates, Maxwell solve
 *   picgpu_solve_poisson     ElectroStaticSolver::solveFields
 *                            (submodels/MaxwellSolver/ElectroStatic/ElectroStaticSolver.C:52-71)
 *   picgpu_get_particles     parcel write-out (PICParcelIO.C:83-166)
 *   picgpu_get_field         field access (phiE, E, rhoCharge)
 *
 * Threading: one context per host thread; calls on one context are not
 * re-entrant.  The library owns all device memory; caller buffers are copied.
 */
#ifndef PICGPU_H
#define PICGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PICGPU_OK = 0,
    PICGPU_INVALID_ARG = 1,
    PICGPU_OOM = 2,
    PICGPU_TRACK_LOOP_CAP = 3,      /* a particle exceeded the tet-step cap   */
    PICGPU_PCG_NOT_CONVERGED = 4,   /* Poisson PCG hit its iteration cap      */
    PICGPU_NAN_DETECTED = 5,
    PICGPU_CUDA_ERROR = 6,
    PICGPU_SPEED_OF_LIGHT = 7,      /* |U| >= c after a push (PICParcel.C:61-66) */
    PICGPU_CAPACITY = 8,            /* particle storage capacity exceeded     */
    PICGPU_NOT_SUPPORTED = 9
} picgpu_status;

/* ParticlePusher TypeNames: "none", "Boris", "BorisNR", "Vay", "HigueraCary" */
enum {
    PICGPU_PUSHER_NONE = 0,
    PICGPU_PUSHER_BORIS = 1,
    PICGPU_PUSHER_BORIS_NR = 2,
    PICGPU_PUSHER_VAY = 3,
    PICGPU_PUSHER_HIGUERA_CARY = 4
};

/* FieldWeigthing / ChargeDistribution TypeNames: "CellAverage", "VolumeWeighting" */
enum {
    PICGPU_WEIGHTING_CELL_AVERAGE = 0,
    PICGPU_WEIGHTING_VOLUME = 1
};

/* MaxwellSolver TypeNames: "none", "ElectroStatic" */
enum {
    PICGPU_MAXWELL_NONE = 0,
    PICGPU_MAXWELL_ELECTROSTATIC = 1
};

/* Arithmetic form of push + track. */
enum {
    PICGPU_PREC_FP64 = 0,   /* FP64 barycentric + velocity (exact form)            */
    PICGPU_PREC_MIXED = 1   /* FP32 barycentric + velocity, FP64 charge and Poisson */
};

/* Charge accumulation. */
enum {
    PICGPU_DEPOSIT_ATOMIC_FP64 = 0,  /* FP64 atomics: order-dependent round-off     */
    PICGPU_DEPOSIT_FIXED_POINT = 1   /* 64-bit fixed point: order-independent sums  */
};

/* Particle-side behaviour of a boundary patch. */
enum {
    PICGPU_PATCH_CYCLIC = 0,    /* periodic pair (OpenFOAM cyclic)                    */
    PICGPU_PATCH_EMPTY = 1,     /* reduced-D direction (OpenFOAM empty)               */
    PICGPU_PATCH_ABSORB = 2,    /* patch + BoundaryModel "none" (NoInflow.C:56-61)    */
    PICGPU_PATCH_WALL = 3,      /* wall + WallReflectionModel SpecularReflection      */
    PICGPU_PATCH_FLOATING = 4,  /* BoundaryModel FloatingPotential + circuitBoundary  */
    PICGPU_PATCH_CIRCUIT = 5    /* electrode of a circuit BoundaryModel (circuitRLC,
                                   IdealVoltageSource, IdealCurrentSource): charged
                                   parcels absorbed and counted, neutral parcels
                                   reflected (circuitRLC.C:268-288)               */
};

/* Potential boundary condition of an ABSORB, WALL or CIRCUIT patch (RLC and
 * CIRCUIT_GRADIENT only on the cathode of a circuit). */
enum {
    PICGPU_PHI_FIXED_VALUE = 0,
    PICGPU_PHI_ZERO_GRADIENT = 1,
    PICGPU_PHI_RLC = 2,              /* RLCBoundary (RLCBoundaryFvPatchField.C) of circuitRLC */
    PICGPU_PHI_CIRCUIT_GRADIENT = 3  /* circuitBoundary driven by IdealCurrentSource */
};

typedef struct {
    int32_t kind;     /* PICGPU_PATCH_* */
    int32_t phi_bc;   /* PICGPU_PHI_* (ABSORB / WALL only) */
    double  phi;      /* fixedValue of the potential [V] */
} picgpu_patch;

/* A box of cells [lo, hi) removed from the block; its surface is one patch
 * (an embedded electrode). */
typedef struct {
    int32_t lo[3];
    int32_t hi[3];
    picgpu_patch patch;
} picgpu_box;

#define PICGPU_MAX_BOXES 8

/* blockMesh-style hexahedral block: n[0] x n[1] x n[2] uniform cells. */
typedef struct {
    int32_t n[3];
    double  origin[3];
    double  length[3];
    picgpu_patch side[6];          /* -x, +x, -y, +y, -z, +z */
    int32_t n_boxes;
    picgpu_box box[PICGPU_MAX_BOXES];
} picgpu_mesh_desc;

#define PICGPU_MAX_SPECIES 4

/* moleculeProperties entry (PICParcel.H:81-138). */
typedef struct {
    double  mass;           /* [kg] */
    double  charge;         /* [C] per real particle */
    double  weight;         /* nEquivalentParticles */
    int32_t solve_movement; /* solveMovement */
    int32_t capacity_hint;  /* optional storage capacity, allocated with the context with the staging of host arrays (0: automatic) */
} picgpu_species;

/* Background gas (uniformBackground.C:36-127) and null-collision MCC
 * (ElectronNeutralCollisionModel.C:703-829) with List cross sections.  The
 * gas_* fields describe the background gas of both the electron-neutral and
 * the ion-neutral model. */
#define PICGPU_MAX_XS_POINTS 1024
typedef struct {
    int32_t enabled;           /* ElectronNeutralCollisionModel != none */
    int32_t scatter;           /* 0: NanbuElectronNeutral, 1: RelativisticElectronNeutral */
    int32_t create_electron;   /* createElectron */
    int32_t create_ion;        /* createIon */
    int32_t ion_species;       /* species index of the created ion (-1: none) */
    int32_t n_xs;              /* cross-section table length */
    double  gas_density;       /* [m^-3] */
    double  gas_temperature;   /* [K] */
    double  gas_mass;          /* [kg] */
    double  gas_velocity[3];   /* drift [m/s] */
    double  gas_weight;        /* background nEquivalentParticles */
    double  ex_threshold;      /* [eV] */
    double  iz_threshold;      /* [eV] */
    double  sigma_v_max_init;  /* initial (sigma v)_max per cell [m^3/s]; 0: FindMaximum */
    double  find_max_energy;   /* FindMaximum search: maximumEnergy [eV] */
    double  find_energy_step;  /* FindMaximum search: energyStep [eV] */
    const double* xs_energy;   /* [n_xs] eV, ascending */
    const double* xs_elastic;  /* [n_xs] m^2 */
    const double* xs_excitation;
    const double* xs_ionization;
    /* Collisions with neutral parcels (performCollisions,
     * ElectronNeutralCollisionModel.C:833-1009): NTC candidates
     * eC nC w_max (sigma c_R)_max dt / V per cell with the neutral_species
     * parcels, before the background-gas collisions (which need
     * gas_density > 0).  The cross sections above are the neutral species'. */
    int32_t neutral_parcels;        /* 1: collide with the parcels of neutral_species */
    int32_t neutral_species;        /* species of the neutral parcels (charge 0) */
    int32_t keep_neutrals;          /* deleteNeutral false: an ionised neutral parcel stays */
    int32_t keep_neutral_velocity;  /* updateNeutralVelocity false: the neutral keeps its velocity */
} picgpu_mcc;

/* Null-collision MCC of ions against the background gas
 * (IonNeutralCollisionModel.C:453-577): IsotropicScattering elastic
 * (IonIsotropicScattering.C:103-143) and charge exchange (:419-426). */
typedef struct {
    int32_t enabled;           /* IonNeutralCollisionModel IsotropicScattering */
    int32_t ion_species;       /* the ion of the background gas */
    int32_t n_xs;
    int32_t pad;
    double  cx_threshold;      /* charge-exchange threshold [eV] */
    double  sigma_v_max_init;  /* 0: FindMaximum */
    double  find_max_energy;
    double  find_energy_step;
    const double* xs_energy;   /* [n_xs] eV, ascending */
    const double* xs_elastic;  /* [n_xs] m^2 */
    const double* xs_charge_exchange;
    /* Collisions with neutral parcels (performCollisions,
     * IonNeutralCollisionModel.C:579-707): NTC candidates nC iC w_max
     * (sigma_T c_R)_max dt / V per cell, isotropic elastic scattering of the
     * pair or the charge-exchange identity switch, before the background-gas
     * collisions (which need picgpu_mcc's gas_density > 0). */
    int32_t neutral_parcels;        /* 1: collide with the parcels of neutral_species */
    int32_t neutral_species;        /* species of the neutral parcels (charge 0) */
    int32_t keep_neutral_velocity;  /* updateNeutralVelocity false */
    /* WeightCorrection of an elastic ion-neutral parcel pair
     * (IonNeutralCollisionModel.C:443-444, applied after the isotropic
     * scatter and before the updateNeutralVelocity reset):
     * PICGPU_WEIGHT_CORRECTION_* (none, Nanbu, SentokuKempNR, SentokuKemp). */
    int32_t weight_correction;
} picgpu_ion_mcc;

/* Binary Coulomb collisions (CoulombCollisionModel.C:241-309). */
enum { PICGPU_PAIRING_NANBU_YONEMURA = 0, PICGPU_PAIRING_TAKIZUKA_ABE = 1 };
enum { PICGPU_COLLIDE_NANBU = 0, PICGPU_COLLIDE_PEREZ = 1 };
/* WeightCorrection TypeNames: none, Nanbu (NanbuCorrection.C:50-66), SentokuKempNR
 * (SentokuKempNonRelCorrection.C:50-125), SentokuKemp (SentokuKempCorrection.C:50-169) */
enum {
    PICGPU_WEIGHT_CORRECTION_NONE = 0,
    PICGPU_WEIGHT_CORRECTION_NANBU = 1,
    PICGPU_WEIGHT_CORRECTION_SENTOKU_KEMP_NR = 2,
    PICGPU_WEIGHT_CORRECTION_SENTOKU_KEMP = 3
};
typedef struct {
    int32_t enabled;
    int32_t pairing;           /* PICGPU_PAIRING_*; TakizukaAbe needs equal species weights */
    int32_t collide;           /* PICGPU_COLLIDE_*: Nanbu, Perez (relativistic, s_max cap) */
    int32_t allow_intra;       /* allowIntraCollision */
    double  coulomb_log;       /* fixed coulombLog (> 0); 0: from the cell Debye length */
    int32_t calculate_bmin;    /* calculateBmin: de Broglie floor of the impact parameter */
    int32_t debye_drift;       /* Debye length: subtract the drift velocity */
    int32_t weight_correction; /* PICGPU_WEIGHT_CORRECTION_*: none, Nanbu, SentokuKempNR, SentokuKemp */
    int32_t pad;
} picgpu_coulomb;

/* Preconditioner of the Poisson PCG (fvSolution phiE { preconditioner }).
 * Jacobi is the default and the form the oracle reproduces bit for bit.
 * MULTIGRID (the GAMG preconditioner's role) applies one FP32 V-cycle of
 * aggregation multigrid per iteration -- 2x2x2 cell aggregates on the block
 * grid, Galerkin coarse operators, weighted-Jacobi smoothing, a dense inverse
 * on the coarsest level -- inside a flexible FP64 PCG that still decides
 * convergence at pcg_tol.  It needs a block mesh (picgpu_mesh_desc). */
enum { PICGPU_PRECOND_JACOBI = 0, PICGPU_PRECOND_MULTIGRID = 1 };

/* Learned warm start of the Poisson PCG (a 3D U-Net on the cell grid, see
 * picgpu_learned.h; no picFoam counterpart).  The first train_steps solves
 * start from the previous potential and feed (start residual, potential
 * increment) pairs to the net, which trains train_iters Adam steps after
 * each; later solves start from the previous potential plus the net's
 * predicted increment, scaled by the A-norm line search, then the FP64 PCG
 * runs to the same tolerance.  After each window of 20 such solves the mean
 * PCG iterations are compared with the plain solves of the training phase;
 * if the net saved less than 2% the solver falls back to the previous
 * potential for good (learned_fallback).  Needs a block mesh whose cell
 * counts are multiples of 4 with n[0]*n[1]*n[2]/64 a multiple of 128. */
typedef struct {
    int32_t enabled;
    int32_t train_steps;      /* solves that feed the training set (0: 500) */
    int32_t train_iters;      /* Adam steps after each of those solves (0: 4) */
    int32_t replay;           /* training pairs kept, newest first (0: 16) */
    double  lr;               /* Adam learning rate (0: 1e-3) */
    int32_t refine;           /* further net passes on the remaining residual (0..3) */
    int32_t pad;
} picgpu_learned;

/* Settings of the multigrid preconditioner (GAMG's nPreSweeps, nPostSweeps,
 * nCellsInCoarsestLevel, scaleCorrection); 0 selects the default. */
typedef struct {
    int32_t pre_sweeps;       /* weighted-Jacobi sweeps before the coarse correction (0: 2) */
    int32_t post_sweeps;      /* and after it (0: 2) */
    int32_t coarsest_cells;   /* aggregate until a level has at most this many cells (0: 512, max 4096) */
    int32_t pad;
    double  omega;            /* Jacobi relaxation factor (0: 0.8) */
    double  scale_correction; /* factor on the prolonged coarse correction (0: 1.6) */
} picgpu_multigrid;

/* BinaryCollisionModel IsotropicScattering (SM/CollisionModels/
 * BinaryCollisionModel/BinaryCollisionModel.C:229-545,
 * IsotropicScattering/IsotropicScattering.C): no-time-counter collisions
 * among the parcels of the neutral (charge 0) species of each cell, partners
 * from the same octant sub-cell when it holds another parcel; optionally
 * collisions of those parcels with the background gas of picgpu_mcc
 * (gas_density, gas_temperature, gas_velocity) whose particles are of
 * background_species. */
enum { PICGPU_XS_HARD_SPHERE = 0, PICGPU_XS_VARIABLE_HARD_SPHERE = 1 };
typedef struct {
    int32_t enabled;
    int32_t cross_section;        /* TotalCrossSectionModel: HardSphere / VariableHardSphere */
    int32_t weight_correction;    /* WeightCorrection: PICGPU_WEIGHT_CORRECTION_* */
    int32_t background_species;   /* species of the background gas (-1: no background collisions) */
    double  diameter[PICGPU_MAX_SPECIES];  /* moleculeProperties diameter [m] */
    double  omega[PICGPU_MAX_SPECIES];     /* moleculeProperties omega (VHS viscosity index) */
    double  tref;                 /* VariableHardSphereCoeffs Tref [K] */
    double  sigma_tcr_max_init;   /* picSigmaTcRMax start value [m^3/s]; 0: BinaryCollisionModel::initialize */
    double  init_temperature;     /* its temperature [K] (0: 293.15) */
} picgpu_binary;

/* Circuit boundary models between an anode and a cathode patch (both of kind
 * PICGPU_PATCH_CIRCUIT):
 *   RLC            circuitRLC (SM/BoundaryModel/circuitRLC/circuitRLC.C): a
 *                  series R-L-C circuit with source V sin(omega t + phase)
 *                  drives the cathode through the RLCBoundary condition
 *                  (anode fixedValue, cathode PICGPU_PHI_RLC);
 *   IDEAL_VOLTAGE  IdealVoltageSource: both electrodes fixedValue; reports the
 *                  running-average anode and cathode currents;
 *   IDEAL_CURRENT  IdealCurrentSource: current I (or J * cathode area) into the
 *                  cathode's circuitBoundary (PICGPU_PHI_CIRCUIT_GRADIENT). */
enum {
    PICGPU_CIRCUIT_NONE = 0,
    PICGPU_CIRCUIT_RLC = 1,
    PICGPU_CIRCUIT_IDEAL_VOLTAGE = 2,
    PICGPU_CIRCUIT_IDEAL_CURRENT = 3
};
typedef struct {
    int32_t model;          /* PICGPU_CIRCUIT_* */
    int32_t anode_patch;    /* patch index (-1: none) */
    int32_t cathode_patch;  /* patch index */
    int32_t pad;
    double  R, L, C;        /* circuitRLC: resistance [Ohm], inductance [H], capacitance [F] */
    double  V, omega, phase;/* source V sin(omega t + phase) [V, rad/s, rad] (reference default phase pi/2) */
    double  epsilon;        /* permittivity of the RLC coupling (<= 0: epsilon0) */
    double  Q[4];           /* RLCBoundary start values Q, Q1, Q2, Q3 [C] */
    double  sigma;          /* cathode surface charge density at the start [C/m^2] */
    double  I;              /* IdealCurrentSource current [A] (< 0: unset) */
    double  J;              /* IdealCurrentSource current density [A/m^2] (< 0: unset) */
    double  ref_area;       /* IdealCurrentSource refArea (> 0: I scaled by cathode area / refArea) */
} picgpu_circuit;

/* ParticleMerging PairMerging (SM/ParticleMerging/PairMerging/PairMerging.C:35-259),
 * run at the end of every step (PICCloud::evolve, PICCloud.C:1470).  In a
 * cell whose parcels of a listed species outnumber cell_parcels_max, random
 * parcels are merged with a neighbour in speed order (the nCheckNeighbors
 * window) into one parcel at their weighted centre with their summed
 * nParticle and weighted mean velocity, until the count is down to
 * reduction_factor of it (at most merge_maximum_per_cell merges) or
 * max_checks attempts.  Listed species keep per-parcel attributes. */
typedef struct {
    int32_t enabled;
    int32_t n_species;                 /* entries of species[] (merge order) */
    int32_t species[PICGPU_MAX_SPECIES];
    double  n_deviation[PICGPU_MAX_SPECIES]; /* nDeviation: largest nParticle difference of a pair */
    double  reduction_factor;          /* reductionFactor */
    double  angle_difference;          /* angleDifference [degrees] */
    double  velocity_ratio;            /* velocityRatio */
    int32_t cell_parcels_max;          /* cellParcelsMax */
    int32_t max_checks;                /* maxChecks */
    int32_t n_check_neighbors;         /* nCheckNeighbors */
    int32_t merge_maximum_per_cell;    /* mergeMaximumPerCell */
} picgpu_merging;

/* CoulombCollisionModel IonizationModel Perez (PerezIonizationModel.C:30-118,
 * selected at CoulombCollisionModel.C:72-79): electron-impact ionisation of
 * ion parcels inside their Coulomb collisions with electrons (the
 * electron species is picgpu_config.electron_species).  Per ion species its
 * atomic number, the ionisation limit (< 0: the atomic number; 0: no
 * ionisation), the orbital binding energies and the ionisation energies of
 * the charge states [eV] (atomicNumber entries each).  An ionisation raises
 * the ion parcel's charge modifier and adds an electron parcel with the
 * ion's nParticle, so the ion and electron species keep per-parcel
 * attributes. */
#define PICGPU_PEREZ_MAX_Z 64
#define PICGPU_PEREZ_MAX_IONS 4
typedef struct {
    int32_t species;              /* ionSpecies */
    int32_t atomic_number;        /* atomicNumber (<= PICGPU_PEREZ_MAX_Z) */
    int32_t ionization_limit;     /* ionizationLimit */
    int32_t pad;
    double  binding_energy[PICGPU_PEREZ_MAX_Z];     /* bindingEnergy [eV] */
    double  ionization_energy[PICGPU_PEREZ_MAX_Z];  /* ionizationEnergy [eV] */
} picgpu_perez_ion;
typedef struct {
    int32_t enabled;
    int32_t n_ions;
    picgpu_perez_ion ion[PICGPU_PEREZ_MAX_IONS];
} picgpu_perez;

typedef struct {
    int32_t pusher;               /* PICGPU_PUSHER_* */
    int32_t field_weighting;      /* PICGPU_WEIGHTING_* */
    int32_t charge_distribution;  /* PICGPU_WEIGHTING_* */
    int32_t maxwell_solver;       /* PICGPU_MAXWELL_* */
    int32_t precision;            /* PICGPU_PREC_* */
    int32_t deposit_mode;         /* PICGPU_DEPOSIT_* */
    int32_t n_species;
    int32_t electron_species;     /* SpeciesRelations electronTypeId (-1: none) */
    picgpu_species species[PICGPU_MAX_SPECIES];
    double  dt;                   /* deltaT [s] */
    double  B[3];                 /* uniform magnetic field [T] */
    double  E_applied[3];         /* uniform field used when maxwell_solver is NONE [V/m] */
    double  space_charge;         /* SolverSettings spaceCharge [C/m^3] */
    int32_t sync_velocity_at_boundary;
    int32_t track_max_steps;      /* tet steps per particle per time step (0: 4096) */
    double  pcg_tol;              /* relative residual target */
    int32_t pcg_max_iter;
    int32_t pcg_norm;             /* 0: ||r||2/||b||2, 1: OpenFOAM-normalised L1 residual */
    int32_t sort_interval;        /* cell re-sort every N steps (0: never unless needed) */
    int32_t pcg_precond;          /* PICGPU_PRECOND_*: Jacobi (0) or multigrid (1) */
    uint64_t seed;
    picgpu_mcc mcc;
    picgpu_ion_mcc ion_mcc;
    picgpu_coulomb coulomb;
    picgpu_learned learned;
    picgpu_multigrid mg;
    picgpu_binary binary;
    picgpu_circuit circuit;
    picgpu_merging merging;
    picgpu_perez perez;
} picgpu_config;

typedef struct {
    int64_t n_particles[PICGPU_MAX_SPECIES];
    int64_t n_absorbed[PICGPU_MAX_SPECIES];    /* removed at patches this call */
    int64_t tet_steps;                          /* tet-to-tet moves this call */
    int64_t face_crossings;                     /* cell-face crossings this call */
    int64_t wall_hits;
    int32_t pcg_iterations;                     /* last solve */
    int32_t pcg_iterations_total;               /* summed over the call */
    double  pcg_residual_l2;                    /* last solve ||b-Ax||2/||b||2 */
    double  pcg_residual_of;                    /* last solve OpenFOAM-normalised */
    double  pcg_residual_initial;               /* last solve ||b-Ax0||2/||b||2 of the start guess */
    int64_t mcc_candidates;
    int64_t mcc_elastic;
    int64_t mcc_excitation;
    int64_t mcc_ionization;
    int64_t coulomb_pairs;
    int64_t ion_mcc_candidates;
    int64_t ion_mcc_elastic;
    int64_t ion_mcc_charge_exchange;
    double  floating_charge[PICGPU_MAX_BOXES + 6]; /* accumulated surface charge per patch [C] */
    double  learned_loss;                       /* last training loss of the warm-start net */
    double  learned_alpha;                      /* line-search factor of the last learned warm start */
    double  learned_residual;                   /* ||b-Ax||2/||b||2 before the net (the plain guess) */
    int32_t learned_active;                     /* 1 when the last solve started from the net's guess */
    int32_t learned_samples;                    /* training pairs collected so far */
    int32_t learned_fallback;                   /* 1 once the net was switched off: it did not cut iterations */
    int32_t pcg_refinements;                    /* last multigrid solve: FP64 refinement steps (0 with Jacobi) */
    int64_t binary_candidates;                  /* BinaryCollisionModel: neutral pairs tested */
    int64_t binary_collisions;                  /* accepted */
    int64_t binary_background_candidates;       /* neutral parcel - background gas tests */
    int64_t binary_background_collisions;
    double  circuit_voltage;                    /* circuitRLC: cathode potential; IdealCurrentSource: mean cathode-cell potential */
    double  circuit_current;                    /* circuitRLC: circuit current; IdealVoltageSource: mean anode current */
    double  circuit_cathode_current;            /* IdealVoltageSource: mean cathode current */
    double  circuit_charge;                     /* circuitRLC: capacitor charge Q; IdealCurrentSource: cathode surface charge */
    /* Collisions with neutral parcels, counted apart from the background-gas
     * collisions above (picFoam reports performCollisions and
     * performBackgroundCollisions separately). */
    int64_t mcc_parcel_candidates;              /* electron - neutral parcel pairs tested */
    int64_t mcc_parcel_elastic;
    int64_t mcc_parcel_excitation;
    int64_t mcc_parcel_ionization;
    int64_t ion_parcel_candidates;              /* ion - neutral parcel pairs tested */
    int64_t ion_parcel_elastic;
    int64_t ion_parcel_charge_exchange;
    int64_t merged_parcels;                     /* PairMerging: merges this step */
    int64_t merge_checks;                       /* candidate partners checked */
    double  merge_kinetic_energy_error;         /* kinetic energy after - before the merges [J] */
    int64_t coulomb_ionizations;                /* Perez ionisation: collisions that ionised */
    int64_t coulomb_ionization_electrons;       /* electron parcels they added */
} picgpu_step_stats;

typedef struct picgpu_ctx picgpu_ctx;

/* Field selectors for picgpu_get_field. */
enum {
    PICGPU_FIELD_PHI = 0,        /* n_cells          */
    PICGPU_FIELD_E_CELL = 1,     /* n_cells x 3      */
    PICGPU_FIELD_RHO = 2,        /* n_cells          */
    PICGPU_FIELD_E_POINT = 3,    /* n_points x 3 (cyclic-merged point numbering) */
    PICGPU_FIELD_SIGMA_V_MAX = 4, /* n_cells          */
    /* n_cells x 3: magnetic field per cell, the B[celli] every picFoam
     * pusher reads (BorisPusher.C:100, VayPusher.C:78, HigueraCary.C:99,
     * BorisNRPusher.C:92).  Setting it replaces the uniform picgpu_config.B
     * for the rest of the run; until then get_field returns the uniform B. */
    PICGPU_FIELD_B_CELL = 5,
    /* 6 + n_boxes (one per patch): surface charge density of the floating
     * patches (FloatingPotential's sigma, FloatingPotential.C:89-100); other
     * patches read 0 and ignore what is set.  Setting it (a restart) also
     * sets the patches' circuitBoundary gradient sigma / eps0. */
    PICGPU_FIELD_PATCH_SIGMA = 6
};

/* Size queries. */
typedef struct {
    int64_t n_cells;
    int64_t n_points;        /* cyclic-merged points */
    int64_t n_tets;          /* 12 per cell */
    int64_t n_patches;
} picgpu_mesh_info;

/* Build the context: mesh, sub-models, device buffers. */
picgpu_status picgpu_create(const picgpu_mesh_desc* mesh, const picgpu_config* cfg,
                            picgpu_ctx** out);
void          picgpu_destroy(picgpu_ctx* ctx);
const char*   picgpu_last_error(const picgpu_ctx* ctx);
picgpu_status picgpu_mesh_query(const picgpu_ctx* ctx, picgpu_mesh_info* info);

/* Host-only mesh handle (no GPU needed): the blockMesh + tet decomposition
 * the context builds, for placing particles (picInitialise,
 * preProcess/picInitialise/picInitialise.C:30-319) and reading positions. */
typedef struct picgpu_mesh picgpu_mesh;
picgpu_status picgpu_mesh_create(const picgpu_mesh_desc* desc, picgpu_mesh** out);
void          picgpu_mesh_destroy(picgpu_mesh* mesh);
picgpu_status picgpu_mesh_info_get(const picgpu_mesh* mesh, picgpu_mesh_info* info);
/* Locate Cartesian positions: tet index (cell*12 + local tet) and the three
 * barycentric coordinates on the tet's face triangle (row-major n x 3); the
 * cell-centre coordinate is 1 - sum.  Unlocated points get tet = -1. */
picgpu_status picgpu_mesh_locate(const picgpu_mesh* mesh, size_t n, const double* xyz,
                                 int32_t* tet, double* bary);
/* Cartesian position of (tet, bary). */
picgpu_status picgpu_mesh_position(const picgpu_mesh* mesh, size_t n, const int32_t* tet,
                                   const double* bary, double* xyz);
/* Cell centres (n_cells x 3) and volumes (n_cells). */
picgpu_status picgpu_mesh_cells(const picgpu_mesh* mesh, double* centres, double* volumes);

/* Page-locked host memory for particle and field transfers.  Arrays passed
 * to picgpu_set_particles / picgpu_get_particles (and the other host-buffer
 * calls) that lie in such memory go straight to the DMA engine; pageable
 * arrays are staged through the context's pinned ring by host threads.
 * picFoam has no counterpart (its parcels live in host memory only).
 * Free with picgpu_host_free. */
picgpu_status picgpu_host_alloc(size_t bytes, void** ptr);
picgpu_status picgpu_host_free(void* ptr);

/* Replace the particles of one species (host buffers, row-major n x 3). */
picgpu_status picgpu_set_particles(picgpu_ctx* ctx, int species, size_t n,
                                   const int32_t* tet, const double* bary,
                                   const double* U);
picgpu_status picgpu_count_particles(picgpu_ctx* ctx, int species, size_t* n);
/* Copy one species out, compacted (removed particles dropped), in storage order. */
picgpu_status picgpu_get_particles(picgpu_ctx* ctx, int species, size_t cap,
                                   int32_t* tet, double* bary, double* U, size_t* n);

/* Per-parcel weight and charge state of one species: PICParcel's
 * nParticle_ and chargeModifier_ (PICParcel.H:182-195; charge = species
 * charge x chargeModifier, PICCloud.C:368), in the order of
 * picgpu_get_particles.  Until set here, or until a model that changes them
 * (PairMerging, the Perez ionisation model) acts on the species, every
 * parcel has the species weight and charge modifier 1 and the store keeps
 * no per-parcel arrays.  Set: n must equal the species' parcel count,
 * nParticle in (0, 4096 x species weight], chargeModifier in [0, 1024];
 * the store is compacted first.  Parcels created later (injection,
 * collisions, picInitialise) get the defaults (PICCloud::addNewParcel,
 * PICCloud.C:707-723).  Get works with or without per-parcel arrays.
 * Species that a background or parcel MCC, ion-neutral or binary collision
 * model uses cannot have per-parcel arrays (those models take one weight per
 * species): PICGPU_NOT_SUPPORTED, also for PairMerging and Perez
 * ionisation on such species at context creation. */
picgpu_status picgpu_set_parcel_attributes(picgpu_ctx* ctx, int species, size_t n,
                                           const double* nParticle, const int32_t* chargeModifier);
picgpu_status picgpu_get_parcel_attributes(picgpu_ctx* ctx, int species, size_t cap,
                                           double* nParticle, int32_t* chargeModifier, size_t* n);

/* The whole population as one set of parcels (the cloud's IDLList of
 * PICParcel, PICParcel.H:182-195, with typeId per parcel): species[i],
 * tet[i] = 12 cell + local tet, bary[3 i..3 i+2] the coordinates of the
 * tet's three face points, U[3 i..3 i+2].  Upload replaces every species'
 * particles (parcels grouped by species in the given order); download
 * writes species 0 first, then 1, ..., each compacted in storage order. */
typedef struct {
    int32_t* species;
    int32_t* tet;
    double*  bary;
    double*  U;
} picgpu_particles_soa;
picgpu_status picgpu_upload_particles(picgpu_ctx* ctx, const picgpu_particles_soa* p, size_t n);
/* cap: room in p; *n: parcels written (on PICGPU_INVALID_ARG with cap too
 * small, *n is the number needed and nothing is written). */
picgpu_status picgpu_download_particles(picgpu_ctx* ctx, picgpu_particles_soa* p, size_t cap, size_t* n);

/* Deposit the current particles and solve the fields (what picInitialise does
 * before the first step: calculateFields + solveFields). */
picgpu_status picgpu_initialise_fields(picgpu_ctx* ctx);

/* SimpleInjection boundary model (SM/BoundaryModel/SimpleInjection/
 * SimpleInjection.C:197-240, emitter SM/Helper/ParticleEmitter/
 * ParticleEmitter.C:54-139 and :265-418): every step, before the move, each
 * listed species gets frequency / weight * dt parcels (the fraction carried
 * to the next step) at area-weighted random points of the patch's face
 * triangles, moved 10-50 % of the way towards the owner cell's centre plane,
 * with a velocity from the model below about the inward normal, then pushed
 * back by dt/2 (syncVelocityAtBoundary) when the species is charged and
 * sync_velocity_at_boundary is set.  The particles' later interaction with
 * the patch is the patch kind's (deletion: ABSORB, reflection: WALL,
 * floating: FLOATING, where each injected parcel also takes its charge off
 * the patch, SimpleInjection.C:295-302). */
enum {
    PICGPU_EMIT_BIRD_MAXWELLIAN_FLUX = 0,  /* birdMaxwellianFlux (ParticleEmitter.C:420-461) */
    PICGPU_EMIT_MOST_PROBABLE_SPEED = 1,   /* mostProbableSpeed (:464-481) */
    PICGPU_EMIT_MAXWELLIAN_FLUX = 2,       /* maxwellianFlux (:503-535) */
    PICGPU_EMIT_HALF_MAXWELLIAN_FLUX = 3   /* halfMaxwellianFlux (:484-496) */
};
#define PICGPU_MAX_INJECTORS 8
typedef struct {
    int32_t patch;                          /* side 0..5 or box 6 + b; not cyclic or empty */
    int32_t velocity_model;                 /* PICGPU_EMIT_* */
    int32_t n_species;                      /* entries of injectionTypeIds */
    int32_t pad;
    int32_t species[PICGPU_MAX_SPECIES];    /* injectionTypeIds */
    double  frequency[PICGPU_MAX_SPECIES];  /* frequencies: physical particles per second */
    double  eV[PICGPU_MAX_SPECIES];         /* temperature of the emitted flux [eV] */
    double  end_time;                       /* injectionEndTime [s]: no injection at t > end_time */
} picgpu_injection;

/* Replace the context's injectors (n = 0 removes them); remainders restart
 * at zero.  Not for ensemble contexts or picgpu_step_graph. */
picgpu_status picgpu_set_injection(picgpu_ctx* ctx, int n, const picgpu_injection* inj);

/* FreeStream boundary model (SM/BoundaryModel/FreeStream/FreeStream.C:126-396):
 * every step, before the move and after the SimpleInjection models, each
 * boundary face of an ABSORB patch gains |S| n/w dt c_mp (e^{-s^2} +
 * sqrt(pi) s (1 + erf s)) / (2 sqrt(pi)) parcels of each species (Bird eq.
 * 4.22, c_mp = sqrt(2kT/m), s = U.n_in / c_mp) in a per-face accumulator.
 * The integer part, plus one when the remainder exceeds a uniform draw, is
 * emitted on the face: one of its two triangles by area, a uniform point on
 * it, the normal speed by Bird's acceptance-rejection (eq. 12.5), thermal
 * tangential components plus the drift's tangential part, then
 * syncVelocityAtBoundary(-0.5).  Parcels reaching the patch are deleted.
 * n = 0 removes all; accumulators restart at zero.  Not for ensemble
 * contexts or picgpu_step_graph. */
#define PICGPU_MAX_FREESTREAMS 8
typedef struct {
    int32_t patch;                               /* an ABSORB side or box patch */
    int32_t n_species;                           /* entries of numberDensities */
    int32_t species[PICGPU_MAX_SPECIES];
    double  number_density[PICGPU_MAX_SPECIES];  /* numberDensities [1/m^3] (real particles) */
    double  temperature;                         /* boundaryT on the patch [K] */
    double  velocity[3];                         /* boundaryU on the patch [m/s] */
} picgpu_freestream;
picgpu_status picgpu_set_freestream(picgpu_ctx* ctx, int n, const picgpu_freestream* fs);

/* EmissionModels of the circuit models (SM/Helper/Emission): electrons of
 * the config's electron_species leave `patch` through the ParticleEmitter
 * with the maxwellianFlux velocity model, n = J A dt / (w e) + remainder per
 * step (A the patch area), after the SimpleInjection and FreeStream models.
 *   THERMIONIC       ThermionicEmission.C: J = lambdaR A0 T^2 exp(-W e/(k T)),
 *                    emitted at temperature T;
 *   FOWLER_NORDHEIM  FowlerNordheim.C: J summed over the patch faces with an
 *                    outward field E (Wang-Loew v(y), t = 1), emitted at
 *                    temperature W e / k.
 * The emitted charge is taken off a floating or circuit patch
 * (particleEjection).  n = 0 removes all.  Not for ensemble contexts or
 * picgpu_step_graph. */
enum { PICGPU_EMISSION_THERMIONIC = 0, PICGPU_EMISSION_FOWLER_NORDHEIM = 1 };
#define PICGPU_MAX_EMISSIONS 8
typedef struct {
    int32_t patch;          /* emitting patch (not cyclic / empty) */
    int32_t model;          /* PICGPU_EMISSION_* */
    double  work_function;  /* fnW [eV] */
    double  temperature;    /* T [K] (thermionic) */
    double  lambda_r;       /* lambdaR (thermionic) */
    double  weight;         /* nParticle (<= 0: the electron species' weight; otherwise it must equal it) */
} picgpu_emission;
picgpu_status picgpu_set_emission(picgpu_ctx* ctx, int n, const picgpu_emission* em);

/* Advance nsteps time steps. */
picgpu_status picgpu_step(picgpu_ctx* ctx, int nsteps, picgpu_step_stats* stats);

/* One pass of push + track + deposit over all particles (no collisions, no
 * field solve): the particle hot path alone. */
picgpu_status picgpu_move(picgpu_ctx* ctx, picgpu_step_stats* stats);

/* E (cells, points and the FP32 corner blocks) from the current potential
 * and boundary conditions, without a Poisson solve: the field part of
 * ElectroStaticSolver::solveFields (ElectroStaticSolver.C:52-71, E = -grad
 * phiE) for a run that continues from a written potential.  No-op when the
 * Maxwell solver is not ElectroStatic. */
picgpu_status picgpu_compute_field(picgpu_ctx* ctx);

/* Restart: the number of time steps already done, i.e. the time index the
 * picFoam run continues from (startFrom latestTime reads it from the time
 * directory, Time::setTime).  The random streams of the collision and
 * injection models, the cell re-sort schedule and the circuit sources are
 * keyed by it. */
picgpu_status picgpu_set_step_index(picgpu_ctx* ctx, int64_t steps_done);

/* ElectroStatic solve on a caller charge density (n_cells); writes the
 * potential (n_cells) and updates E. phi_inout is the initial guess. */
picgpu_status picgpu_solve_poisson(picgpu_ctx* ctx, const double* rho,
                                   double* phi_inout, picgpu_step_stats* stats);

picgpu_status picgpu_get_field(picgpu_ctx* ctx, int which, double* out, size_t n);
/* phi (n_cells), cell E (n_cells x 3) and rho (n_cells) at once; any may be NULL. */
picgpu_status picgpu_get_fields(picgpu_ctx* ctx, double* phi, double* E, double* rho);
picgpu_status picgpu_set_field(picgpu_ctx* ctx, int which, const double* in, size_t n);

/* Diagnostics (KineticEnergyInfo, FieldEnergyInfo, TemperatureInfo). */
typedef struct {
    double kinetic_energy[PICGPU_MAX_SPECIES];       /* sum 0.5 w m |U|^2 [J] */
    double kinetic_energy_rel[PICGPU_MAX_SPECIES];   /* sum (gamma-1) m c^2 (no weight, KineticEnergyInfo.C:75-77) */
    double momentum[PICGPU_MAX_SPECIES][3];          /* sum w m U */
    double velocity_sq[PICGPU_MAX_SPECIES][3];       /* sum w U_i^2 */
    double weight_sum[PICGPU_MAX_SPECIES];           /* sum w */
    double field_energy;                              /* 0.5 eps0 sum |E|^2 V [J] */
} picgpu_diagnostics;
picgpu_status picgpu_diagnostics_compute(picgpu_ctx* ctx, picgpu_diagnostics* out);

/* Phase timing with CUDA events on the context stream. */
enum {
    PICGPU_PHASE_MOVE = 0,       /* push + track + deposit kernel */
    PICGPU_PHASE_CHARGE = 1,     /* point -> cell charge           */
    PICGPU_PHASE_POISSON = 2,    /* PCG                            */
    PICGPU_PHASE_EFIELD = 3,     /* gradient + cell -> point       */
    PICGPU_PHASE_SORT = 4,
    PICGPU_PHASE_MCC = 5,
    PICGPU_PHASE_COULOMB = 6,
    PICGPU_PHASE_COUNT = 7
};
picgpu_status picgpu_set_profiling(picgpu_ctx* ctx, int enabled);
/* Per phase: summed milliseconds and launch counts since the last reset. */
picgpu_status picgpu_phase_times(picgpu_ctx* ctx, double* ms, int64_t* launches,
                                 int nphase, int reset);
/* Kernels launched by the library since creation (all phases). */
int64_t       picgpu_kernel_launches(const picgpu_ctx* ctx);
picgpu_status picgpu_synchronize(picgpu_ctx* ctx);
/* Device-time region on the context stream: start records an event, stop
 * records a second one, synchronises and returns the elapsed milliseconds. */
picgpu_status picgpu_timer_start(picgpu_ctx* ctx);
picgpu_status picgpu_timer_stop(picgpu_ctx* ctx, double* ms);

/* Allocation-free PCG solve.  This entry point has no counterpart in picFoam.
 *
 * For callers that cannot call cudaMalloc -- a solver plugin hosted by a
 * framework whose memory pool owns all device memory, or a time-critical
 * loop where cudaMalloc's implicit device-wide synchronisation is not
 * acceptable -- it solves M x = b with the same Jacobi-preconditioned PCG
 * kernels as picgpu_solve_poisson, without allocating anything.  All
 * pointers are DEVICE pointers owned by the caller:
 *   diag[n_cells]   M's diagonal (positive: M is -laplacian, SPD)
 *   off[6*n_cells]  M's off-diagonal coefficient per cell face (-|S|/|d|)
 *   nbr[6*n_cells]  neighbour cell per face, or -1 where there is none
 *   b[n_cells]      right-hand side
 *   x[n_cells]      initial guess in, solution out
 * Stops when ||b - M x||2 <= tol ||b||2 or after max_iter iterations;
 * iterations and residual (relative L2) are written to host memory.
 * Work runs on `stream` (a cudaStream_t; NULL = default stream) of the
 * current device and the call returns when it has finished.
 *
 * Limit: n_cells <= PICGPU_NOALLOC_MAX_CELLS; larger problems are rejected
 * with PICGPU_CAPACITY.  The working vectors live in a fixed __device__
 * array (about 3.2 MB) that every device using the library holds until the
 * process exits.  The first call on a device looks up that array's device
 * address; make that first call before any stream capture.  All calls on a
 * device share the array, so calls whose GPU work overlaps race: serialise
 * them.  Status: PICGPU_OK, PICGPU_INVALID_ARG, PICGPU_CAPACITY,
 * PICGPU_PCG_NOT_CONVERGED or PICGPU_CUDA_ERROR. */
#define PICGPU_NOALLOC_MAX_CELLS 65536
picgpu_status picgpu_solve_ldu_noalloc(int n_cells, const double* diag, const double* off,
                                       const int32_t* nbr, const double* b, double* x,
                                       double tol, int max_iter, int* iterations,
                                       double* residual, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PICGPU_H */
