"""ctypes mirror of include/picgpu.h (the C ABI of the particle hot path).

Every structure here has the exact field order and types of its C
counterpart; the library and the CPU oracle share the same structures.
"""
import ctypes as C

# status codes
OK = 0
INVALID_ARG = 1
OOM = 2
TRACK_LOOP_CAP = 3
PCG_NOT_CONVERGED = 4
NAN_DETECTED = 5
CUDA_ERROR = 6
SPEED_OF_LIGHT = 7
CAPACITY = 8
NOT_SUPPORTED = 9

STATUS_NAMES = {
    OK: "OK", INVALID_ARG: "INVALID_ARG", OOM: "OOM", TRACK_LOOP_CAP: "TRACK_LOOP_CAP",
    PCG_NOT_CONVERGED: "PCG_NOT_CONVERGED", NAN_DETECTED: "NAN_DETECTED",
    CUDA_ERROR: "CUDA_ERROR", SPEED_OF_LIGHT: "SPEED_OF_LIGHT", CAPACITY: "CAPACITY",
    NOT_SUPPORTED: "NOT_SUPPORTED",
}

PUSHER_NONE, PUSHER_BORIS, PUSHER_BORIS_NR, PUSHER_VAY, PUSHER_HIGUERA_CARY = range(5)
WEIGHTING_CELL_AVERAGE, WEIGHTING_VOLUME = range(2)
MAXWELL_NONE, MAXWELL_ELECTROSTATIC = range(2)
PREC_FP64, PREC_MIXED = range(2)
DEPOSIT_ATOMIC_FP64, DEPOSIT_FIXED_POINT = range(2)
PATCH_CYCLIC, PATCH_EMPTY, PATCH_ABSORB, PATCH_WALL, PATCH_FLOATING, PATCH_CIRCUIT = range(6)
PHI_FIXED_VALUE, PHI_ZERO_GRADIENT, PHI_RLC, PHI_CIRCUIT_GRADIENT = range(4)
CIRCUIT_NONE, CIRCUIT_RLC, CIRCUIT_IDEAL_VOLTAGE, CIRCUIT_IDEAL_CURRENT = range(4)
PRECOND_JACOBI, PRECOND_MULTIGRID = range(2)
FIELD_PHI, FIELD_E_CELL, FIELD_RHO, FIELD_E_POINT, FIELD_SIGMA_V_MAX, FIELD_B_CELL, FIELD_PATCH_SIGMA = range(7)
(PHASE_MOVE, PHASE_CHARGE, PHASE_POISSON, PHASE_EFIELD, PHASE_SORT, PHASE_MCC,
 PHASE_COULOMB, PHASE_COUNT) = range(8)
PHASE_NAMES = ["move", "charge", "poisson", "efield", "sort", "mcc", "coulomb"]

MAX_BOXES = 8
MAX_SPECIES = 4


class ParticlesSoa(C.Structure):
    _fields_ = [("species", C.POINTER(C.c_int32)), ("tet", C.POINTER(C.c_int32)),
                ("bary", C.POINTER(C.c_double)), ("U", C.POINTER(C.c_double))]


class Patch(C.Structure):
    _fields_ = [("kind", C.c_int32), ("phi_bc", C.c_int32), ("phi", C.c_double)]


class Box(C.Structure):
    _fields_ = [("lo", C.c_int32 * 3), ("hi", C.c_int32 * 3), ("patch", Patch)]


class MeshDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int32 * 3),
        ("origin", C.c_double * 3),
        ("length", C.c_double * 3),
        ("side", Patch * 6),
        ("n_boxes", C.c_int32),
        ("box", Box * MAX_BOXES),
    ]


class Species(C.Structure):
    _fields_ = [
        ("mass", C.c_double), ("charge", C.c_double), ("weight", C.c_double),
        ("solve_movement", C.c_int32), ("capacity_hint", C.c_int32),
    ]


class Mcc(C.Structure):
    _fields_ = [
        ("enabled", C.c_int32), ("scatter", C.c_int32), ("create_electron", C.c_int32),
        ("create_ion", C.c_int32), ("ion_species", C.c_int32), ("n_xs", C.c_int32),
        ("gas_density", C.c_double), ("gas_temperature", C.c_double), ("gas_mass", C.c_double),
        ("gas_velocity", C.c_double * 3), ("gas_weight", C.c_double),
        ("ex_threshold", C.c_double), ("iz_threshold", C.c_double),
        ("sigma_v_max_init", C.c_double), ("find_max_energy", C.c_double),
        ("find_energy_step", C.c_double),
        ("xs_energy", C.POINTER(C.c_double)), ("xs_elastic", C.POINTER(C.c_double)),
        ("xs_excitation", C.POINTER(C.c_double)), ("xs_ionization", C.POINTER(C.c_double)),
        ("neutral_parcels", C.c_int32), ("neutral_species", C.c_int32), ("keep_neutrals", C.c_int32),
        ("keep_neutral_velocity", C.c_int32),
    ]


class IonMcc(C.Structure):
    _fields_ = [
        ("enabled", C.c_int32), ("ion_species", C.c_int32), ("n_xs", C.c_int32), ("pad", C.c_int32),
        ("cx_threshold", C.c_double), ("sigma_v_max_init", C.c_double),
        ("find_max_energy", C.c_double), ("find_energy_step", C.c_double),
        ("xs_energy", C.POINTER(C.c_double)), ("xs_elastic", C.POINTER(C.c_double)),
        ("xs_charge_exchange", C.POINTER(C.c_double)),
        ("neutral_parcels", C.c_int32), ("neutral_species", C.c_int32), ("keep_neutral_velocity", C.c_int32),
        ("weight_correction", C.c_int32),
    ]


PAIRING_NANBU_YONEMURA, PAIRING_TAKIZUKA_ABE = range(2)
COLLIDE_NANBU, COLLIDE_PEREZ = range(2)
WEIGHT_CORRECTION_NONE, WEIGHT_CORRECTION_NANBU, WEIGHT_CORRECTION_SENTOKU_KEMP_NR, WEIGHT_CORRECTION_SENTOKU_KEMP = range(4)


class Coulomb(C.Structure):
    _fields_ = [
        ("enabled", C.c_int32), ("pairing", C.c_int32), ("collide", C.c_int32),
        ("allow_intra", C.c_int32), ("coulomb_log", C.c_double),
        ("calculate_bmin", C.c_int32), ("debye_drift", C.c_int32),
        ("weight_correction", C.c_int32), ("pad", C.c_int32),
    ]


class Learned(C.Structure):
    _fields_ = [
        ("enabled", C.c_int32), ("train_steps", C.c_int32), ("train_iters", C.c_int32),
        ("replay", C.c_int32), ("lr", C.c_double), ("refine", C.c_int32), ("pad", C.c_int32),
    ]


XS_HARD_SPHERE, XS_VARIABLE_HARD_SPHERE = range(2)


class Binary(C.Structure):
    _fields_ = [
        ("enabled", C.c_int32), ("cross_section", C.c_int32), ("weight_correction", C.c_int32),
        ("background_species", C.c_int32), ("diameter", C.c_double * MAX_SPECIES),
        ("omega", C.c_double * MAX_SPECIES), ("tref", C.c_double), ("sigma_tcr_max_init", C.c_double),
        ("init_temperature", C.c_double),
    ]


class Circuit(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("anode_patch", C.c_int32), ("cathode_patch", C.c_int32), ("pad", C.c_int32),
        ("R", C.c_double), ("L", C.c_double), ("C", C.c_double),
        ("V", C.c_double), ("omega", C.c_double), ("phase", C.c_double), ("epsilon", C.c_double),
        ("Q", C.c_double * 4), ("sigma", C.c_double),
        ("I", C.c_double), ("J", C.c_double), ("ref_area", C.c_double),
    ]


class Multigrid(C.Structure):
    _fields_ = [
        ("pre_sweeps", C.c_int32), ("post_sweeps", C.c_int32), ("coarsest_cells", C.c_int32),
        ("pad", C.c_int32), ("omega", C.c_double), ("scale_correction", C.c_double),
    ]


class Merging(C.Structure):
    _fields_ = [
        ("enabled", C.c_int32), ("n_species", C.c_int32), ("species", C.c_int32 * MAX_SPECIES),
        ("n_deviation", C.c_double * MAX_SPECIES), ("reduction_factor", C.c_double),
        ("angle_difference", C.c_double), ("velocity_ratio", C.c_double),
        ("cell_parcels_max", C.c_int32), ("max_checks", C.c_int32), ("n_check_neighbors", C.c_int32),
        ("merge_maximum_per_cell", C.c_int32),
    ]


PEREZ_MAX_Z = 64
PEREZ_MAX_IONS = 4


class PerezIon(C.Structure):
    _fields_ = [
        ("species", C.c_int32), ("atomic_number", C.c_int32), ("ionization_limit", C.c_int32), ("pad", C.c_int32),
        ("binding_energy", C.c_double * PEREZ_MAX_Z), ("ionization_energy", C.c_double * PEREZ_MAX_Z),
    ]


class Perez(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("n_ions", C.c_int32), ("ion", PerezIon * PEREZ_MAX_IONS)]


class Config(C.Structure):
    _fields_ = [
        ("pusher", C.c_int32), ("field_weighting", C.c_int32),
        ("charge_distribution", C.c_int32), ("maxwell_solver", C.c_int32),
        ("precision", C.c_int32), ("deposit_mode", C.c_int32),
        ("n_species", C.c_int32), ("electron_species", C.c_int32),
        ("species", Species * MAX_SPECIES),
        ("dt", C.c_double), ("B", C.c_double * 3), ("E_applied", C.c_double * 3),
        ("space_charge", C.c_double),
        ("sync_velocity_at_boundary", C.c_int32), ("track_max_steps", C.c_int32),
        ("pcg_tol", C.c_double), ("pcg_max_iter", C.c_int32), ("pcg_norm", C.c_int32),
        ("sort_interval", C.c_int32), ("pcg_precond", C.c_int32),
        ("seed", C.c_uint64),
        ("mcc", Mcc), ("ion_mcc", IonMcc), ("coulomb", Coulomb), ("learned", Learned),
        ("mg", Multigrid), ("binary", Binary), ("circuit", Circuit), ("merging", Merging), ("perez", Perez),
    ]


# SimpleInjection (picgpu.h)
EMIT_BIRD_MAXWELLIAN_FLUX, EMIT_MOST_PROBABLE_SPEED, EMIT_MAXWELLIAN_FLUX, EMIT_HALF_MAXWELLIAN_FLUX = range(4)
MAX_INJECTORS = 8


class Injection(C.Structure):
    _fields_ = [
        ("patch", C.c_int32), ("velocity_model", C.c_int32), ("n_species", C.c_int32), ("pad", C.c_int32),
        ("species", C.c_int32 * MAX_SPECIES), ("frequency", C.c_double * MAX_SPECIES),
        ("eV", C.c_double * MAX_SPECIES), ("end_time", C.c_double),
    ]


MAX_FREESTREAMS = 8


class FreeStream(C.Structure):
    _fields_ = [
        ("patch", C.c_int32), ("n_species", C.c_int32), ("species", C.c_int32 * MAX_SPECIES),
        ("number_density", C.c_double * MAX_SPECIES), ("temperature", C.c_double), ("velocity", C.c_double * 3),
    ]


EMISSION_THERMIONIC, EMISSION_FOWLER_NORDHEIM = range(2)
MAX_EMISSIONS = 8


class Emission(C.Structure):
    _fields_ = [
        ("patch", C.c_int32), ("model", C.c_int32), ("work_function", C.c_double), ("temperature", C.c_double),
        ("lambda_r", C.c_double), ("weight", C.c_double),
    ]


# picgpu_init.h
INIT_NONE, INIT_EQUIPARTITION, INIT_MAXWELLIAN, INIT_ISOTROPIZATION, INIT_QUASINEUTRAL_PLASMA, \
    INIT_UNIFORM_DISPLACEMENT = range(6)


class Init(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("clear_particles", C.c_int32), ("solve_fields", C.c_int32),
        ("leapfrog", C.c_int32),
        ("number_density", C.c_double * MAX_SPECIES), ("temperature", C.c_double * MAX_SPECIES),
        ("velocity", C.c_double * 3),
        ("drift_velocity", (C.c_double * 3) * MAX_SPECIES), ("thermal_velocity", (C.c_double * 3) * MAX_SPECIES),
        ("tperp_over_tpara", C.c_double), ("cell_count", C.c_double),
        ("ion_species", C.c_int32), ("use_maxwellian", C.c_int32),
        ("species_mask", C.c_int32), ("use_bounds", C.c_int32),
        ("min", C.c_double * 3), ("max", C.c_double * 3), ("particle_numbers", C.c_int64 * 3),
        ("displacement_dir", C.c_double * 3), ("displacement", C.c_double * MAX_SPECIES),
        ("cycles", C.c_double), ("seed", C.c_uint64),
    ]


class InitStats(C.Structure):
    _fields_ = [
        ("added", C.c_int64 * MAX_SPECIES), ("occupancy_avg", C.c_double * MAX_SPECIES),
        ("occupancy_min", C.c_int64 * MAX_SPECIES), ("occupancy_max", C.c_int64 * MAX_SPECIES),
        ("drift", (C.c_double * 3) * MAX_SPECIES), ("temperature", C.c_double * MAX_SPECIES),
        ("number_density", C.c_double * MAX_SPECIES), ("model_temperature", C.c_double * MAX_SPECIES),
        ("model_number_density", C.c_double * MAX_SPECIES),
        ("mesh_volume", C.c_double), ("debye_length", C.c_double), ("average_cell_size", C.c_double),
        ("plasma_frequency_dt", C.c_double), ("place_ms", C.c_double),
    ]


class StepStats(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int64 * MAX_SPECIES),
        ("n_absorbed", C.c_int64 * MAX_SPECIES),
        ("tet_steps", C.c_int64), ("face_crossings", C.c_int64), ("wall_hits", C.c_int64),
        ("pcg_iterations", C.c_int32), ("pcg_iterations_total", C.c_int32),
        ("pcg_residual_l2", C.c_double), ("pcg_residual_of", C.c_double),
        ("pcg_residual_initial", C.c_double),
        ("mcc_candidates", C.c_int64), ("mcc_elastic", C.c_int64),
        ("mcc_excitation", C.c_int64), ("mcc_ionization", C.c_int64),
        ("coulomb_pairs", C.c_int64),
        ("ion_mcc_candidates", C.c_int64), ("ion_mcc_elastic", C.c_int64),
        ("ion_mcc_charge_exchange", C.c_int64),
        ("floating_charge", C.c_double * (MAX_BOXES + 6)),
        ("learned_loss", C.c_double), ("learned_alpha", C.c_double), ("learned_residual", C.c_double),
        ("learned_active", C.c_int32), ("learned_samples", C.c_int32),
        ("learned_fallback", C.c_int32), ("pcg_refinements", C.c_int32),
        ("binary_candidates", C.c_int64), ("binary_collisions", C.c_int64),
        ("binary_background_candidates", C.c_int64), ("binary_background_collisions", C.c_int64),
        ("circuit_voltage", C.c_double), ("circuit_current", C.c_double),
        ("circuit_cathode_current", C.c_double), ("circuit_charge", C.c_double),
        ("mcc_parcel_candidates", C.c_int64), ("mcc_parcel_elastic", C.c_int64),
        ("mcc_parcel_excitation", C.c_int64), ("mcc_parcel_ionization", C.c_int64),
        ("ion_parcel_candidates", C.c_int64), ("ion_parcel_elastic", C.c_int64),
        ("ion_parcel_charge_exchange", C.c_int64),
        ("merged_parcels", C.c_int64), ("merge_checks", C.c_int64), ("merge_kinetic_energy_error", C.c_double),
        ("coulomb_ionizations", C.c_int64), ("coulomb_ionization_electrons", C.c_int64),
    ]

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if hasattr(v, "__len__") else v
        return d


class MeshInfo(C.Structure):
    _fields_ = [("n_cells", C.c_int64), ("n_points", C.c_int64), ("n_tets", C.c_int64),
                ("n_patches", C.c_int64)]


class Diagnostics(C.Structure):
    _fields_ = [
        ("kinetic_energy", C.c_double * MAX_SPECIES),
        ("kinetic_energy_rel", C.c_double * MAX_SPECIES),
        ("momentum", (C.c_double * 3) * MAX_SPECIES),
        ("velocity_sq", (C.c_double * 3) * MAX_SPECIES),
        ("weight_sum", C.c_double * MAX_SPECIES),
        ("field_energy", C.c_double),
    ]
