"""Case builders: mesh, sub-model selection and initial particles.

Each builder stands in for a picFoam case directory (blockMeshDict,
constant/picProperties, system/picInitialiseDict) and the picInitialise
run that fills it: particles are placed uniformly in tets
(UniformInitialization.C:51-127, MaxwellianInitialization.C) with Maxwellian
velocities drawn from numpy's Philox generator.  The workloads are the
benchmark configurations of the particle hot path (seeded synthetic inputs):

  plasma_oscillation_1d   periodic 0.1 m box, 128 cells, 200 e-/cell
  two_species_3d          0.05 m cube, 64^3 cells, e- and Ar+ at 50/cell, B = 0.01 T
  electron_swarm          32x32x256 cells, 10M e-, E = 1e4 V/m, argon-like gas
  coulomb_thermalisation  16^3 cells, 400 e-/cell, T_x = 2 eV, T_yz = 1 eV
  coulomb_relaxation      e- and heavy ions at different temperatures (e-i exchange)
  ion_swarm               Ar+ in argon: isotropic elastic + charge exchange MCC
  swarm_ensemble          64 swarm cases of 16x16x128 cells, 10-1000 Td, 1e5-4e6 e- each
  electrode_box           128^3 cells, two floating boxes, one 100 V box
"""
import ctypes as C
import dataclasses
import math

import numpy as np

from . import abi

C_LIGHT = 299792458.0
MU0 = 4.0 * math.pi * 1e-7
EPS0 = 1.0 / (MU0 * C_LIGHT * C_LIGHT)
E_CHARGE = 1.602176634e-19
K_B = 1.380649e-23
M_E = 9.1093837015e-31
M_AR = 6.6335209e-26


@dataclasses.dataclass
class Case:
    name: str
    mesh: abi.MeshDesc
    cfg: abi.Config
    particles: dict
    keepalive: list
    meta: dict


def patch(kind, phi=0.0, phi_bc=abi.PHI_FIXED_VALUE):
    p = abi.Patch()
    p.kind = kind
    p.phi_bc = phi_bc
    p.phi = phi
    return p


def block_mesh(n, length, sides, origin=(0.0, 0.0, 0.0), boxes=()):
    m = abi.MeshDesc()
    for a in range(3):
        m.n[a] = n[a]
        m.length[a] = length[a]
        m.origin[a] = origin[a]
    for s in range(6):
        m.side[s] = sides[s]
    m.n_boxes = len(boxes)
    for i, (lo, hi, p) in enumerate(boxes):
        for a in range(3):
            m.box[i].lo[a] = lo[a]
            m.box[i].hi[a] = hi[a]
        m.box[i].patch = p
    return m


def base_config(dt, species, pusher=abi.PUSHER_BORIS, precision=abi.PREC_FP64,
                deposit=abi.DEPOSIT_ATOMIC_FP64, maxwell=abi.MAXWELL_ELECTROSTATIC,
                weighting=abi.WEIGHTING_VOLUME, B=(0.0, 0.0, 0.0), E_applied=(0.0, 0.0, 0.0),
                pcg_tol=1e-10, seed=1234, electron_species=0):
    c = abi.Config()
    c.pusher = pusher
    c.field_weighting = weighting
    c.charge_distribution = weighting
    c.maxwell_solver = maxwell
    c.precision = precision
    c.deposit_mode = deposit
    c.n_species = len(species)
    c.electron_species = electron_species
    for i, (mass, charge, weight, move) in enumerate(species):
        c.species[i].mass = mass
        c.species[i].charge = charge
        c.species[i].weight = weight
        c.species[i].solve_movement = 1 if move else 0
    c.dt = dt
    for a in range(3):
        c.B[a] = B[a]
        c.E_applied[a] = E_applied[a]
    c.sync_velocity_at_boundary = 1
    c.track_max_steps = 4096
    c.pcg_tol = pcg_tol
    c.pcg_max_iter = 20000
    c.seed = seed
    return c


def plasma_frequency(n, mass=M_E, charge=E_CHARGE):
    return math.sqrt(n * charge * charge / (EPS0 * mass))


def thermal_speed(T_eV, mass):
    return math.sqrt(T_eV * E_CHARGE / mass)


def uniform_in_cells(rng, cells, per_cell):
    """per_cell particles in each listed cell: random tet, uniform barycentric."""
    cells = np.repeat(np.asarray(cells, dtype=np.int64), per_cell)
    n = cells.size
    tet = (cells * 12 + rng.integers(0, 12, n)).astype(np.int32)
    u = np.sort(rng.random((n, 3)), axis=1)
    bary = np.stack([u[:, 0], u[:, 1] - u[:, 0], u[:, 2] - u[:, 1]], axis=1)
    return tet, bary


def maxwellian(rng, n, T_eV, mass):
    return rng.standard_normal((n, 3)) * thermal_speed(T_eV, mass)


def plasma_oscillation_1d(mesh_api, n_cells=128, per_cell=200, seed=1234, dt_factor=0.05,
                          perturbation=0.01, precision=abi.PREC_FP64,
                          deposit=abi.DEPOSIT_ATOMIC_FP64, pusher=abi.PUSHER_BORIS, pcg_tol=1e-10,
                          T_eV=1.0, n_e=1e14, quiet=False):
    """Periodic 0.1 m box, n_cells x 1 x 1 hexes (thickness = dx, empty y/z),
    electrons over an immobile neutralising background (spaceCharge).
    quiet=True places the electrons evenly (a quiet start)."""
    L = 0.1
    dx = L / n_cells
    sides = [patch(abi.PATCH_CYCLIC), patch(abi.PATCH_CYCLIC),
             patch(abi.PATCH_EMPTY), patch(abi.PATCH_EMPTY),
             patch(abi.PATCH_EMPTY), patch(abi.PATCH_EMPTY)]
    mesh = block_mesh((n_cells, 1, 1), (L, dx, dx), sides)
    N = n_cells * per_cell
    w = n_e * L * dx * dx / N
    wpe = plasma_frequency(n_e)
    dt = dt_factor / wpe
    cfg = base_config(dt, [(M_E, -E_CHARGE, w, True)], pusher=pusher, precision=precision,
                      deposit=deposit, pcg_tol=pcg_tol, seed=seed)
    cfg.space_charge = E_CHARGE * n_e
    rng = np.random.Generator(np.random.Philox(seed))
    x = (np.arange(N) + 0.5) * (L / N) if quiet else rng.random(N) * L
    xyz = np.stack([x, np.full(N, 0.5 * dx), np.full(N, 0.5 * dx)], axis=1)
    m = mesh_api(mesh)
    tet, bary = m.locate(xyz)
    vth = thermal_speed(T_eV, M_E)
    U = rng.standard_normal((N, 3)) * vth
    U[:, 0] += perturbation * vth * np.sin(2 * math.pi * x / L)
    return Case("plasma_oscillation_1d", mesh, cfg, {0: (tet, bary, U)}, [],
                dict(wpe=wpe, dt=dt, n_e=n_e, L=L, vth=vth, N=N, weight=w))


def two_species_3d(n_cells=64, per_cell=50, seed=1234, precision=abi.PREC_MIXED,
                   pusher=abi.PUSHER_BORIS, deposit=abi.DEPOSIT_ATOMIC_FP64, Bz=0.01, n=1e15,
                   T_e=2.0, T_i=0.03, dt_factor=0.1, pcg_tol=1e-10, L=0.05):
    """Cube with grounded absorbing walls, electrons + Ar+, uniform B_z."""
    sides = [patch(abi.PATCH_ABSORB, 0.0) for _ in range(6)]
    mesh = block_mesh((n_cells,) * 3, (L,) * 3, sides)
    n_c = n_cells ** 3
    N = n_c * per_cell
    w = n * L ** 3 / N
    wpe = plasma_frequency(n)
    dt = dt_factor / wpe
    cfg = base_config(dt, [(M_E, -E_CHARGE, w, True), (M_AR, E_CHARGE, w, True)], pusher=pusher,
                      precision=precision, deposit=deposit, B=(0.0, 0.0, Bz), pcg_tol=pcg_tol,
                      seed=seed)
    cfg.sort_interval = 0
    rng = np.random.Generator(np.random.Philox(seed))
    parts = {}
    for s, (T, mass) in enumerate([(T_e, M_E), (T_i, M_AR)]):
        tet, bary = uniform_in_cells(rng, np.arange(n_c), per_cell)
        U = maxwellian(rng, N, T, mass)
        parts[s] = (tet, bary, U)
    return Case("two_species_3d", mesh, cfg, parts, [],
                dict(wpe=wpe, dt=dt, n=n, N=2 * N, weight=w, n_cells=n_c))


def magnetic_rotation(mesh_api, pusher=abi.PUSHER_HIGUERA_CARY, precision=abi.PREC_FP64, beta=0.1, B=1.0,
                      steps_per_orbit=200, n_cells=40, E=(0.0, 0.0, 0.0)):
    """Single electron gyrating in B_z (tutorial magneticRotation: 0.4 mm
    square, 40 x 40 cells, one cell thick and empty along the field, electron
    at (0, -r, 0) with v = 0.1 c along x, MaxwellSolver none).  meta holds the
    gyration radius gamma m v / (e B)."""
    L = 4e-4
    sides = [patch(abi.PATCH_ABSORB), patch(abi.PATCH_ABSORB), patch(abi.PATCH_ABSORB),
             patch(abi.PATCH_ABSORB), patch(abi.PATCH_EMPTY), patch(abi.PATCH_EMPTY)]
    mesh = block_mesh((n_cells, n_cells, 1), (L, L, L / n_cells), sides,
                      origin=(-L / 2, -L / 2, -L / (2 * n_cells)))
    v = beta * C_LIGHT
    gamma = 1.0 / math.sqrt(1.0 - beta * beta)
    r = gamma * M_E * v / (E_CHARGE * B)
    wc = E_CHARGE * B / (gamma * M_E)
    dt = 2 * math.pi / wc / steps_per_orbit
    cfg = base_config(dt, [(M_E, -E_CHARGE, 1.0, True)], pusher=pusher, precision=precision,
                      maxwell=abi.MAXWELL_NONE, B=(0.0, 0.0, B), E_applied=E)
    m = mesh_api(mesh)
    tet, bary = m.locate(np.array([[0.0, -r, 0.0]]))
    U = np.array([[v, 0.0, 0.0]])
    return Case("magnetic_rotation", mesh, cfg, {0: (tet, bary, U)}, [],
                dict(radius=r, v=v, gamma=gamma, wc=wc, dt=dt, L=L))


def xs_tables(n=256, emin=0.01, emax=1000.0, el0=1e-19, ex_th=11.5, ex0=5e-21, iz_th=15.8, iz0=3e-20):
    """Argon-like cross sections tabulated at n log-spaced energies."""
    e = np.logspace(math.log10(emin), math.log10(emax), n)
    el = el0 * (1.0 + e / 10.0) ** -0.5
    ex = np.where(e > ex_th, ex0 * np.log(np.maximum(e / ex_th, 1.0)) / (e / ex_th), 0.0)
    iz = np.where(e > iz_th, iz0 * np.log(np.maximum(e / iz_th, 1.0)) / (e / iz_th), 0.0)
    return e, el, ex, iz


def electron_swarm(nx=32, ny=32, nz=256, N=10_000_000, Ez=1e4, gas_density=1e21, T_gas=300.0,
                   T_e=1.0, seed=1234, precision=abi.PREC_MIXED, dt=None, ion_species=True,
                   size=(0.02, 0.02, 0.16), weight=1.0):
    """Electron swarm in an argon-like background gas, fixed E along z,
    absorbing walls, null-collision MCC with ionisation."""
    sides = [patch(abi.PATCH_ABSORB) for _ in range(6)]
    mesh = block_mesh((nx, ny, nz), size, sides)
    e, el, ex, iz = xs_tables()
    if dt is None:
        # max(nu) dt <= 0.1 at the table maximum of sigma v; v dt <= 0.5 dx
        sv = np.max(np.sqrt(2 * E_CHARGE * e / M_E) * (el + ex + iz))
        dt = min(0.1 / (gas_density * sv), 0.5 * (size[0] / nx) / math.sqrt(2 * E_CHARGE * 200.0 / M_E))
    species = [(M_E, -E_CHARGE, weight, True)]
    if ion_species:
        species.append((M_AR, E_CHARGE, weight, True))
    cfg = base_config(dt, species, precision=precision, maxwell=abi.MAXWELL_NONE,
                      E_applied=(0.0, 0.0, Ez), seed=seed)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (e, el, ex, iz)]
    import ctypes as C
    mc = cfg.mcc
    mc.enabled = 1
    mc.scatter = 0
    mc.create_electron = 1
    mc.create_ion = 1 if ion_species else 0
    mc.ion_species = 1 if ion_species else -1
    mc.n_xs = len(e)
    mc.gas_density = gas_density
    mc.gas_temperature = T_gas
    mc.gas_mass = M_AR
    mc.gas_weight = weight
    mc.ex_threshold = 11.5
    mc.iz_threshold = 15.8
    mc.find_max_energy = 1000.0
    mc.find_energy_step = 0.01
    mc.xs_energy = arrs[0].ctypes.data_as(C.POINTER(C.c_double))
    mc.xs_elastic = arrs[1].ctypes.data_as(C.POINTER(C.c_double))
    mc.xs_excitation = arrs[2].ctypes.data_as(C.POINTER(C.c_double))
    mc.xs_ionization = arrs[3].ctypes.data_as(C.POINTER(C.c_double))
    rng = np.random.Generator(np.random.Philox(seed))
    n_c = nx * ny * nz
    cells = rng.integers(0, n_c, N)
    tet = (cells * 12 + rng.integers(0, 12, N)).astype(np.int32)
    u = np.sort(rng.random((N, 3)), axis=1)
    bary = np.stack([u[:, 0], u[:, 1] - u[:, 0], u[:, 2] - u[:, 1]], axis=1)
    U = maxwellian(rng, N, T_e, M_E)
    # the store in cell order, as picInitialise's per-cell placement leaves it
    o = np.argsort(tet, kind="stable")
    tet, bary, U = tet[o], bary[o], U[o]
    parts = {0: (tet, bary, U)}
    if ion_species:
        parts[1] = (np.zeros(0, np.int32), np.zeros((0, 3)), np.zeros((0, 3)))
    return Case("electron_swarm", mesh, cfg, parts, arrs,
                dict(dt=dt, E_over_N_Td=Ez / gas_density * 1e21, N=N))


def neutral_parcel_ionization(n_cells=(4, 4, 4), L=1e-3, per_cell=(20, 40), T_e_eV=100.0, T_n=300.0, n_n=1e20,
                              sigma_iz=3.43943e-20, threshold=15.76, dt=1e-11, seed=1234, precision=abi.PREC_FP64,
                              keep_neutrals=False, keep_neutral_velocity=False, exact_max=True, ions_per_cell=0,
                              ion_collisions=None):
    """The ionization tutorial's collision set-up: electrons, neutral Ar
    parcels and Ar+ with equal weights in a periodic box, MaxwellSolver
    none, electron-neutral MCC against the parcels (performCollisions) with
    a FixedValue ionisation cross section (threshold 15.76 eV), no elastic or
    excitation.  per_cell = (electrons, neutrals); electrons monoenergetic at
    T_e_eV (isotropic directions).  exact_max starts (sigma c_R)_max at
    sigma_iz times the electron speed.  ions_per_cell places Ar+ parcels at
    the start (1 eV Maxwellian); ion_collisions = (sigma_el, sigma_cx) adds
    ion collisions with the same neutral parcels (IonNeutralCollisionModel
    performCollisions, which runs after the electron step and sees the lists
    without the neutrals that step ionised and deleted)."""
    sides = [patch(abi.PATCH_CYCLIC) for _ in range(6)]
    mesh = block_mesh(n_cells, (L,) * 3, sides)
    n_c = n_cells[0] * n_cells[1] * n_cells[2]
    w = n_n * L ** 3 / (n_c * per_cell[1])
    cfg = base_config(dt, [(M_E, -E_CHARGE, w, True), (M_AR, 0.0, w, True), (M_AR, E_CHARGE, w, True)],
                      maxwell=abi.MAXWELL_NONE, precision=precision, seed=seed)
    e = np.array([0.0, 1e5])
    zero = np.zeros(2)
    iz = np.full(2, sigma_iz)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (e, zero, zero, iz)]
    import ctypes as C
    mc = cfg.mcc
    mc.enabled = 1
    mc.scatter = 1                      # RelativisticElectronNeutral, as the tutorial
    mc.create_electron = 1
    mc.create_ion = 1
    mc.ion_species = 2
    mc.n_xs = 2
    mc.gas_density = 0.0                # BackgroundGasModel none
    mc.gas_mass = M_AR
    mc.gas_weight = w
    mc.ex_threshold = 11.5
    mc.iz_threshold = threshold
    v_e = math.sqrt(2 * E_CHARGE * T_e_eV / M_E)
    mc.sigma_v_max_init = sigma_iz * v_e * 1.01 if exact_max else 0.0
    mc.find_max_energy = 2 * T_e_eV
    mc.find_energy_step = 0.01
    mc.xs_energy, mc.xs_elastic, mc.xs_excitation, mc.xs_ionization = [
        a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]
    mc.neutral_parcels = 1
    mc.neutral_species = 1
    mc.keep_neutrals = 1 if keep_neutrals else 0
    mc.keep_neutral_velocity = 1 if keep_neutral_velocity else 0
    if ion_collisions is not None:
        iarrs = [np.ascontiguousarray(a, dtype=np.float64)
                 for a in ([0.0, 1e6], [ion_collisions[0]] * 2, [ion_collisions[1]] * 2)]
        arrs = arrs + iarrs
        im = cfg.ion_mcc
        im.enabled = 1
        im.ion_species = 2
        im.n_xs = 2
        im.cx_threshold = 0.0
        im.sigma_v_max_init = (ion_collisions[0] + ion_collisions[1]) * math.sqrt(2 * E_CHARGE * 10.0 / M_AR)
        im.xs_energy, im.xs_elastic, im.xs_charge_exchange = [
            a.ctypes.data_as(C.POINTER(C.c_double)) for a in iarrs]
        im.neutral_parcels = 1
        im.neutral_species = 1
        im.keep_neutral_velocity = 1 if keep_neutral_velocity else 0
    rng = np.random.Generator(np.random.Philox(seed))
    te, be = uniform_in_cells(rng, np.arange(n_c), per_cell[0])
    d = rng.standard_normal((len(te), 3))
    Ue = v_e * d / np.linalg.norm(d, axis=1)[:, None]
    tn, bn = uniform_in_cells(rng, np.arange(n_c), per_cell[1])
    Un = rng.standard_normal((len(tn), 3)) * math.sqrt(K_B * T_n / M_AR)
    if ions_per_cell:
        ti, bi = uniform_in_cells(rng, np.arange(n_c), ions_per_cell)
        ions = (ti, bi, rng.standard_normal((len(ti), 3)) * math.sqrt(E_CHARGE * 1.0 / M_AR))
    else:
        ions = (np.zeros(0, np.int32), np.zeros((0, 3)), np.zeros((0, 3)))
    parts = {0: (te, be, Ue), 1: (tn, bn, Un), 2: ions}
    return Case("neutral_parcel_ionization", mesh, cfg, parts, arrs,
                dict(w=w, v_e=v_e, n_n=n_n, V=L ** 3, N_e=len(te), N_n=len(tn), n_c=n_c))


def ion_neutral_parcels(n_cells=(4, 4, 4), L=1e-3, per_cell=(30, 30), T_i_eV=5.0, T_n=300.0, n_n=1e22,
                        sigma_el=5e-19, sigma_cx=3e-19, dt=2e-9, seed=1234, precision=abi.PREC_FP64,
                        keep_neutral_velocity=False, ion_weight_ratio=1.0, weight_correction=0):
    """Ar+ ions and neutral Ar parcels in a periodic box, MaxwellSolver none,
    IonNeutralCollisionModel against the parcels (performCollisions) with
    constant elastic and charge-exchange cross sections.  per_cell = (ions,
    neutrals); the ion weight is ion_weight_ratio times the neutral weight,
    and weight_correction (PICGPU_WEIGHT_CORRECTION_*) corrects elastic pairs
    of unequal weight."""
    sides = [patch(abi.PATCH_CYCLIC) for _ in range(6)]
    mesh = block_mesh(n_cells, (L,) * 3, sides)
    n_c = n_cells[0] * n_cells[1] * n_cells[2]
    w = n_n * L ** 3 / (n_c * per_cell[1])
    cfg = base_config(dt, [(M_AR, 0.0, w, True), (M_AR, E_CHARGE, w * ion_weight_ratio, True)],
                      maxwell=abi.MAXWELL_NONE, precision=precision, seed=seed, electron_species=-1)
    mc = cfg.mcc
    mc.gas_density = 0.0
    mc.gas_mass = M_AR
    mc.gas_temperature = T_n
    mc.gas_weight = w
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in ([0.0, 1e6], [sigma_el] * 2, [sigma_cx] * 2)]
    import ctypes as C
    im = cfg.ion_mcc
    im.enabled = 1
    im.ion_species = 1
    im.n_xs = 2
    im.cx_threshold = 0.0
    vmax = math.sqrt(2 * E_CHARGE * 10 * T_i_eV / M_AR)
    im.sigma_v_max_init = (sigma_el + sigma_cx) * vmax
    im.xs_energy, im.xs_elastic, im.xs_charge_exchange = [a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]
    im.neutral_parcels = 1
    im.neutral_species = 0
    im.keep_neutral_velocity = 1 if keep_neutral_velocity else 0
    im.weight_correction = weight_correction
    rng = np.random.Generator(np.random.Philox(seed))
    tn, bn = uniform_in_cells(rng, np.arange(n_c), per_cell[1])
    Un = rng.standard_normal((len(tn), 3)) * math.sqrt(K_B * T_n / M_AR)
    ti, bi = uniform_in_cells(rng, np.arange(n_c), per_cell[0])
    Ui = rng.standard_normal((len(ti), 3)) * math.sqrt(E_CHARGE * T_i_eV / M_AR)
    return Case("ion_neutral_parcels", mesh, cfg, {0: (tn, bn, Un), 1: (ti, bi, Ui)}, arrs,
                dict(w=w, n_n=n_n, V=L ** 3, sigma=sigma_el + sigma_cx))


def set_coulomb(cfg, pairing=abi.PAIRING_NANBU_YONEMURA, collide=abi.COLLIDE_NANBU, coulomb_log=15.0,
                calculate_bmin=True, debye_drift=True, weight_correction=0, allow_intra=True):
    """CoulombCollisionModel dictionary: coulomb_log 0 computes the logarithm
    from the cell Debye length (calculate_bmin / accountForDrift default on,
    CoulombCollisionModel.C:128-140)."""
    co = cfg.coulomb
    co.enabled = 1
    co.pairing = pairing
    co.collide = collide
    co.allow_intra = 1 if allow_intra else 0
    co.coulomb_log = coulomb_log
    co.calculate_bmin = 1 if calculate_bmin else 0
    co.debye_drift = 1 if debye_drift else 0
    co.weight_correction = weight_correction


def coulomb_thermalisation(n_cells=16, per_cell=400, n=1e18, T=4.0 / 3.0, ratio=0.5, seed=1234,
                           coulomb_log=15.0, precision=abi.PREC_FP64, dt_factor=None, L=None,
                           pairing=abi.PAIRING_NANBU_YONEMURA, collide=abi.COLLIDE_NANBU):
    """Electrons with T_x = 2 eV, T_y = T_z = 1 eV (Isotropization initial
    condition), periodic box, no field solve, intra-species Coulomb
    collisions (NanbuYonemura or TakizukaAbe pairing, Nanbu or Perez
    collide; coulomb_log 0 = from the Debye length)."""
    if L is None:
        L = 1e-4
    sides = [patch(abi.PATCH_CYCLIC) for _ in range(6)]
    mesh = block_mesh((n_cells,) * 3, (L,) * 3, sides)
    n_c = n_cells ** 3
    N = n_c * per_cell
    w = n * L ** 3 / N
    # T_para = T * 3 / (1 + 2 ratio), T_perp = ratio * T_para
    T_x = 3.0 * T / (1.0 + 2.0 * ratio)
    T_yz = ratio * T_x
    ve = thermal_speed(T_x, M_E)
    # the time step is set by a logarithm of 15 whether or not it is computed
    nu = n * E_CHARGE ** 4 * (coulomb_log or 15.0) / (4 * math.pi * EPS0 ** 2 * M_E ** 2 * ve ** 3)
    dt = (dt_factor if dt_factor else 0.02) / nu
    cfg = base_config(dt, [(M_E, -E_CHARGE, w, True)], maxwell=abi.MAXWELL_NONE, precision=precision,
                      seed=seed)
    set_coulomb(cfg, pairing=pairing, collide=collide, coulomb_log=coulomb_log)
    rng = np.random.Generator(np.random.Philox(seed))
    tet, bary = uniform_in_cells(rng, np.arange(n_c), per_cell)
    U = rng.standard_normal((N, 3))
    U[:, 0] *= thermal_speed(T_x, M_E)
    U[:, 1:] *= thermal_speed(T_yz, M_E)
    return Case("coulomb_thermalisation", mesh, cfg, {0: (tet, bary, U)}, [],
                dict(dt=dt, T_x=T_x, T_yz=T_yz, nu=nu, N=N))


def coulomb_relaxation(n_cells=4, e_per_cell=60, i_per_cell=45, n=1e18, T_e=2.0, T_i=0.5, m_i=100.0 * M_E,
                       seed=1234, coulomb_log=10.0, precision=abi.PREC_FP64, L=2e-5,
                       pairing=abi.PAIRING_NANBU_YONEMURA, collide=abi.COLLIDE_NANBU, w_i_factor=1.0,
                       weight_correction=0, dt_factor=0.02, ragged=False):
    """Electrons (T_e) and ions of mass m_i (T_i) in a periodic box, no
    field solve: inter- and intra-species Coulomb collisions relax the two
    temperatures.  Unequal per-cell counts exercise the unequal-group
    pairing; w_i_factor != 1 gives the ions another parcel weight (with
    weight_correction 1 the Nanbu correction applies); ragged draws the
    per-cell counts at random (0..2x the mean) so that empty, single and odd
    cells occur."""
    sides = [patch(abi.PATCH_CYCLIC) for _ in range(6)]
    mesh = block_mesh((n_cells,) * 3, (L,) * 3, sides)
    n_c = n_cells ** 3
    V = L ** 3
    rng = np.random.Generator(np.random.Philox(seed))
    if ragged:
        ce = rng.integers(0, 2 * e_per_cell + 1, n_c)
        ci = rng.integers(0, 2 * i_per_cell + 1, n_c)
    else:
        ce = np.full(n_c, e_per_cell)
        ci = np.full(n_c, i_per_cell)
    Ne, Ni = int(ce.sum()), int(ci.sum())
    w_e = n * V / max(Ne, 1)
    w_i = w_e * w_i_factor
    ve = thermal_speed(T_e, M_E)
    nu = n * E_CHARGE ** 4 * (coulomb_log or 10.0) / (4 * math.pi * EPS0 ** 2 * M_E ** 2 * ve ** 3)
    dt = dt_factor / nu
    cfg = base_config(dt, [(M_E, -E_CHARGE, w_e, True), (m_i, E_CHARGE, w_i, True)], maxwell=abi.MAXWELL_NONE,
                      precision=precision, seed=seed)
    set_coulomb(cfg, pairing=pairing, collide=collide, coulomb_log=coulomb_log,
                weight_correction=weight_correction)

    def place(counts):
        cells = np.repeat(np.arange(n_c), counts)
        m = cells.size
        tet = (cells * 12 + rng.integers(0, 12, m)).astype(np.int32)
        u = np.sort(rng.random((m, 3)), axis=1)
        return tet, np.stack([u[:, 0], u[:, 1] - u[:, 0], u[:, 2] - u[:, 1]], axis=1)

    te, be = place(ce)
    ti, bi = place(ci)
    Ue = maxwellian(rng, Ne, T_e, M_E)
    Ui = maxwellian(rng, Ni, T_i, m_i)
    return Case("coulomb_relaxation", mesh, cfg, {0: (te, be, Ue), 1: (ti, bi, Ui)}, [],
                dict(dt=dt, nu=nu, Ne=Ne, Ni=Ni, counts_e=ce, counts_i=ci))


def ion_swarm(n_cells=(8, 8, 8), N=20000, T_i=1.0, gas_density=1e21, T_gas=300.0, sigma_el=5e-19,
              sigma_cx=5e-19, cx_threshold=0.0, seed=1234, precision=abi.PREC_FP64, size=(0.01, 0.01, 0.01),
              steps_dt=0.01, gas_drift=(0.0, 0.0, 0.0)):
    """Ar+ ions in argon, periodic box, no field: IonNeutralCollisionModel
    with isotropic elastic scattering and charge exchange (constant cross
    sections, List tables of two nodes)."""
    import ctypes as C
    sides = [patch(abi.PATCH_CYCLIC) for _ in range(6)]
    mesh = block_mesh(n_cells, size, sides)
    n_c = n_cells[0] * n_cells[1] * n_cells[2]
    vmax = math.sqrt(2 * E_CHARGE * 30.0 * T_i / M_AR) + 4 * math.sqrt(K_B * T_gas / M_AR)
    sv = (sigma_el + sigma_cx) * vmax
    dt = steps_dt / (gas_density * sv)
    cfg = base_config(dt, [(M_AR, E_CHARGE, 1.0, True)], maxwell=abi.MAXWELL_NONE, precision=precision,
                      seed=seed, electron_species=-1)
    mc = cfg.mcc
    mc.gas_density = gas_density
    mc.gas_temperature = T_gas
    mc.gas_mass = M_AR
    mc.gas_weight = 1.0
    for a in range(3):
        mc.gas_velocity[a] = gas_drift[a]
    arrs = [np.ascontiguousarray(a, dtype=np.float64)
            for a in ([0.0, 1e4], [sigma_el, sigma_el], [sigma_cx, sigma_cx])]
    im = cfg.ion_mcc
    im.enabled = 1
    im.ion_species = 0
    im.n_xs = 2
    im.cx_threshold = cx_threshold
    im.sigma_v_max_init = sv
    im.xs_energy, im.xs_elastic, im.xs_charge_exchange = [
        a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]
    rng = np.random.Generator(np.random.Philox(seed))
    cells = rng.integers(0, n_c, N)
    tet = (cells * 12 + rng.integers(0, 12, N)).astype(np.int32)
    u = np.sort(rng.random((N, 3)), axis=1)
    bary = np.stack([u[:, 0], u[:, 1] - u[:, 0], u[:, 2] - u[:, 1]], axis=1)
    U = maxwellian(rng, N, T_i, M_AR)
    return Case("ion_swarm", mesh, cfg, {0: (tet, bary, U)}, arrs,
                dict(dt=dt, N=N, sv=sv))


def electrode_box(n_cells=128, per_cell=30, n=1e15, T_e=2.0, T_i=0.03, seed=1234,
                  precision=abi.PREC_MIXED, dt_factor=0.1, pcg_tol=1e-8, L=0.1):
    """Cube with grounded absorbing walls, two floating 8^3-cell box
    electrodes and one 100 V box electrode."""
    sides = [patch(abi.PATCH_ABSORB, 0.0) for _ in range(6)]
    k = n_cells // 4
    e = max(n_cells // 16, 1)
    boxes = [((k, k, k), (k + e, k + e, k + e), patch(abi.PATCH_FLOATING)),
             ((3 * k - e, k, k), (3 * k, k + e, k + e), patch(abi.PATCH_FLOATING)),
             ((2 * k - e // 2, 3 * k - e, 2 * k - e // 2), (2 * k + e - e // 2, 3 * k, 2 * k + e - e // 2),
              patch(abi.PATCH_ABSORB, 100.0))]
    mesh = block_mesh((n_cells,) * 3, (L,) * 3, sides, boxes=boxes)
    removed = set()
    for lo, hi, _ in boxes:
        for kk in range(lo[2], hi[2]):
            for j in range(lo[1], hi[1]):
                for i in range(lo[0], hi[0]):
                    removed.add(i + n_cells * (j + n_cells * kk))
    n_c = n_cells ** 3 - len(removed)
    N = n_c * per_cell
    w = n * (L ** 3) / (n_cells ** 3 * per_cell)
    wpe = plasma_frequency(n)
    dt = dt_factor / wpe
    cfg = base_config(dt, [(M_E, -E_CHARGE, w, True), (M_AR, E_CHARGE, w, True)], precision=precision,
                      pcg_tol=pcg_tol, seed=seed)
    rng = np.random.Generator(np.random.Philox(seed))
    parts = {}
    for s, (T, mass) in enumerate([(T_e, M_E), (T_i, M_AR)]):
        tet, bary = uniform_in_cells(rng, np.arange(n_c), per_cell)
        parts[s] = (tet, bary, maxwellian(rng, N, T, mass))
    return Case("electrode_box", mesh, cfg, parts, [], dict(dt=dt, N=2 * N, n_cells=n_c))


def swarm_ensemble(n_cases=64, n=(16, 16, 128), size=(0.01, 0.01, 0.08), counts=None, EN_Td=None,
                   count_range=(1e5, 4e6), count_seed=7, gas_density=1e21, T_gas=300.0, T_e=1.0, seed=1234,
                   ion_species=True, dt=None):
    """Batched electron swarms: n_cases independent copies of the swarm
    geometry (config of electron_swarm scaled to n cells), reduced fields
    E/N log-spaced over 10-1000 Td, particle counts log-uniform over
    count_range drawn from count_seed.  Returns the single-case mesh, the
    config, the per-case fields and the combined particle arrays (tet indices
    of case k offset by k cells_per_case)."""
    one = electron_swarm(nx=n[0], ny=n[1], nz=n[2], N=1, Ez=0.0, gas_density=gas_density, T_gas=T_gas, T_e=T_e,
                         seed=seed, precision=abi.PREC_MIXED, ion_species=ion_species, size=size, dt=dt)
    cfg = one.cfg
    cfg.sort_interval = 20  # keep the store in cell order (deposit locality)
    cpc = n[0] * n[1] * n[2]
    if counts is None:
        r = np.random.Generator(np.random.Philox(count_seed))
        lo, hi = np.log(count_range[0]), np.log(count_range[1])
        counts = np.exp(r.uniform(lo, hi, n_cases)).astype(np.int64)
    counts = np.asarray(counts, dtype=np.int64)
    if EN_Td is None:
        EN_Td = np.logspace(1.0, 3.0, n_cases)
    E = np.zeros((n_cases, 3))
    E[:, 2] = np.asarray(EN_Td) * 1e-21 * gas_density
    rng = np.random.Generator(np.random.Philox(seed))
    N = int(counts.sum())
    case_of = np.repeat(np.arange(n_cases, dtype=np.int64), counts)
    cells = case_of * cpc + rng.integers(0, cpc, N)
    tet = (cells * 12 + rng.integers(0, 12, N)).astype(np.int32)
    u = np.sort(rng.random((N, 3), dtype=np.float32), axis=1)
    bary = np.stack([u[:, 0], u[:, 1] - u[:, 0], u[:, 2] - u[:, 1]], axis=1)
    U = maxwellian(rng, N, T_e, M_E).astype(np.float32)
    parts = {0: (tet, bary, U)}
    if ion_species:
        parts[1] = (np.zeros(0, np.int32), np.zeros((0, 3)), np.zeros((0, 3)))
    return Case("swarm_ensemble", one.mesh, cfg, parts, one.keepalive,
                dict(dt=cfg.dt, n_cases=n_cases, counts=counts, EN_Td=np.asarray(EN_Td), E=E,
                     cells_per_case=cpc, N=N))


def init_config(model, seed=1234, number_density=(), temperature=(), clear=True, solve_fields=False,
                leapfrog=False, electron_volt=False, **kw):
    """An abi.Init (system/picInitialiseDict): number densities [1/m^3] and
    temperatures (K, or eV with electron_volt, as picInitialise's
    electronVolt switch) per species; model coefficients by keyword:
    velocity, drift_velocity, thermal_velocity, tperp_over_tpara, cell_count,
    ion_species, use_maxwellian, species (UniformDisplacement list), min, max,
    particle_numbers, displacement_dir, displacement, cycles."""
    it = abi.Init()
    it.model = model
    it.clear_particles = 1 if clear else 0
    it.solve_fields = 1 if solve_fields else 0
    it.leapfrog = 1 if leapfrog else 0
    it.seed = seed
    for s, n in enumerate(number_density):
        it.number_density[s] = n
    for s, T in enumerate(temperature):
        it.temperature[s] = T * (E_CHARGE / K_B if electron_volt else 1.0)
    for k in ("velocity", "min", "max", "displacement_dir"):
        if k in kw:
            for a in range(3):
                getattr(it, k)[a] = kw[k][a]
    for k in ("drift_velocity", "thermal_velocity"):
        for s, v in enumerate(kw.get(k, ())):
            for a in range(3):
                getattr(it, k)[s][a] = v[a]
    if "particle_numbers" in kw:
        for a in range(3):
            it.particle_numbers[a] = int(kw["particle_numbers"][a])
    if "min" in kw or "max" in kw:
        it.use_bounds = 1
    for s, d in enumerate(kw.get("displacement", ())):
        it.displacement[s] = d
    it.species_mask = sum(1 << s for s in kw.get("species", ()))
    for k in ("tperp_over_tpara", "cell_count", "cycles"):
        if k in kw:
            setattr(it, k, kw[k])
    it.ion_species = kw.get("ion_species", -1)
    it.use_maxwellian = 1 if kw.get("use_maxwellian", True) else 0
    return it


def injection(patch, species, frequency, eV, model=abi.EMIT_MAXWELLIAN_FLUX, end_time=1.0):
    """An abi.Injection (SimpleInjectionCoeffs): injectionTypeIds `species`,
    frequencies [1/s] and eV per species, velocityModel, injectionEndTime."""
    q = abi.Injection()
    q.patch = patch
    q.velocity_model = model
    q.n_species = len(species)
    for j, s in enumerate(species):
        q.species[j] = s
        q.frequency[j] = frequency[j]
        q.eV[j] = eV[j]
    q.end_time = end_time
    return q


def freestream(patch, species, number_density, temperature, velocity=(0.0, 0.0, 0.0)):
    """An abi.FreeStream (FreeStreamCoeffs numberDensities per species [1/m^3],
    boundaryT [K] and boundaryU [m/s] on the patch)."""
    q = abi.FreeStream()
    q.patch = patch
    q.n_species = len(species)
    for j, s in enumerate(species):
        q.species[j] = s
        q.number_density[j] = number_density[j]
    q.temperature = temperature
    for a in range(3):
        q.velocity[a] = velocity[a]
    return q


def emission(patch, model, work_function, temperature=0.0, lambda_r=0.5, weight=0.0):
    """An abi.Emission (ThermionicEmissionCoeffs / FowlerNordheimCoeffs:
    fnW [eV], T [K], lambdaR, nParticle)."""
    q = abi.Emission()
    q.patch = patch
    q.model = model
    q.work_function = work_function
    q.temperature = temperature
    q.lambda_r = lambda_r
    q.weight = weight
    return q


def set_merging(cfg, species, cell_parcels_max=20, reduction_factor=0.7, max_checks=200, n_check_neighbors=4,
                angle_difference=30.0, velocity_ratio=0.5, n_deviation=None, merge_maximum_per_cell=100):
    """ParticleMerging PairMerging dictionary (PairMerging.C:35-68):
    species in merge order, nDeviation per listed species (default: 10
    species weights)."""
    mg = cfg.merging
    mg.enabled = 1
    mg.n_species = len(species)
    for k, s in enumerate(species):
        mg.species[k] = s
        mg.n_deviation[k] = (n_deviation[k] if n_deviation is not None else 10.0 * cfg.species[s].weight)
    mg.reduction_factor = reduction_factor
    mg.angle_difference = angle_difference
    mg.velocity_ratio = velocity_ratio
    mg.cell_parcels_max = cell_parcels_max
    mg.max_checks = max_checks
    mg.n_check_neighbors = n_check_neighbors
    mg.merge_maximum_per_cell = merge_maximum_per_cell


def merging_plasma(n_cells=4, e_per_cell=40, i_per_cell=30, n=1e15, T_e=2.0, T_i=0.5, L=4e-4, seed=1234,
                   precision=abi.PREC_FP64, dt_factor=0.05, ragged=True, **merge):
    """Electrons and Ar+ in a periodic box with the field solve and
    PairMerging of both species; ragged gives the cells 1/4 to 7/4 of the
    mean count, so some cells stay under cellParcelsMax."""
    sides = [patch(abi.PATCH_CYCLIC) for _ in range(6)]
    mesh = block_mesh((n_cells,) * 3, (L,) * 3, sides)
    n_c = n_cells ** 3
    rng = np.random.Generator(np.random.Philox(seed))
    parts = {}
    counts = []
    for s, (per, T, mass) in enumerate([(e_per_cell, T_e, M_E), (i_per_cell, T_i, M_AR)]):
        if ragged:
            cnt = np.maximum(1, (per * (0.25 + 1.5 * rng.random(n_c))).astype(int))
        else:
            cnt = np.full(n_c, per)
        cells = np.repeat(np.arange(n_c), cnt)
        tet = (12 * cells + rng.integers(0, 12, cells.shape[0])).astype(np.int32)
        b = rng.random((cells.shape[0], 4))
        b /= b.sum(axis=1, keepdims=True)
        parts[s] = (tet, np.ascontiguousarray(b[:, 1:]), maxwellian(rng, cells.shape[0], T, mass))
        counts.append(cells.shape[0])
    w = n * L ** 3 / counts[0]
    wpe = plasma_frequency(n)
    cfg = base_config(dt_factor / wpe, [(M_E, -E_CHARGE, w, True), (M_AR, E_CHARGE, w, True)],
                      precision=precision, deposit=abi.DEPOSIT_FIXED_POINT, seed=seed)
    cfg.sort_interval = 0
    set_merging(cfg, [0, 1], **merge)
    return Case("merging_plasma", mesh, cfg, parts, [], dict(counts=counts, weight=w))


def perez_plasma(perez, n_cells=4, e_per_cell=40, i_per_cell=40, n=1e27, T_e=400.0, T_i=1.0, L=2e-8, seed=1234,
                 precision=abi.PREC_FP64, dt=5e-15, collide=abi.COLLIDE_NANBU, w_i_factor=1.0, ragged=True):
    """Hot electrons (T_e in eV) and Ar+ in a periodic box without a field
    solve: Coulomb collisions (NanbuYonemura pairing) with the Perez
    ionisation model `perez` (an abi.Perez for species e = 0, ion = 1; the
    thermalization tutorial's argon coefficients, for instance)."""
    sides = [patch(abi.PATCH_CYCLIC) for _ in range(6)]
    mesh = block_mesh((n_cells,) * 3, (L,) * 3, sides)
    n_c = n_cells ** 3
    rng = np.random.Generator(np.random.Philox(seed))
    parts = {}
    counts = []
    for s, (per, T, mass) in enumerate([(e_per_cell, T_e, M_E), (i_per_cell, T_i, M_AR)]):
        cnt = (np.maximum(1, (per * (0.25 + 1.5 * rng.random(n_c))).astype(int)) if ragged else np.full(n_c, per))
        cells = np.repeat(np.arange(n_c), cnt)
        tet = (12 * cells + rng.integers(0, 12, cells.shape[0])).astype(np.int32)
        b = rng.random((cells.shape[0], 4))
        b /= b.sum(axis=1, keepdims=True)
        parts[s] = (tet, np.ascontiguousarray(b[:, 1:]), maxwellian(rng, cells.shape[0], T, mass))
        counts.append(cells.shape[0])
    w = n * L ** 3 / counts[0]
    cfg = base_config(dt, [(M_E, -E_CHARGE, w, True), (M_AR, E_CHARGE, w * w_i_factor, True)],
                      maxwell=abi.MAXWELL_NONE, precision=precision, seed=seed)
    set_coulomb(cfg, collide=collide, coulomb_log=10.0)
    C.memmove(C.addressof(cfg.perez), C.addressof(perez), C.sizeof(abi.Perez))
    return Case("perez_plasma", mesh, cfg, parts, [], dict(counts=counts, weight=w))


def empty_case(n_cells=(8, 8, 8), length=(0.01, 0.01, 0.01), sides=None, boxes=(), species=None,
               precision=abi.PREC_FP64, dt=1e-12, origin=(0.0, 0.0, 0.0), electron_species=0):
    """A case without particles: block mesh and config for picInitialise runs.
    species: (mass, charge, weight, solveMovement) tuples (default e-, Ar+)."""
    if sides is None:
        sides = [patch(abi.PATCH_ABSORB, 0.0) for _ in range(6)]
    if species is None:
        species = [(M_E, -E_CHARGE, 1e4, True), (M_AR, E_CHARGE, 1e4, True)]
    mesh = block_mesh(n_cells, length, sides, origin=origin, boxes=boxes)
    cfg = base_config(dt, species, precision=precision, deposit=abi.DEPOSIT_FIXED_POINT,
                      electron_species=electron_species)
    return Case("empty", mesh, cfg, {}, [], {})


def circuit_case(model=abi.CIRCUIT_RLC, n=200, length=0.05, width=0.024, R=1.0, C=1e-6, L=0.04, V=100.0,
                 omega=0.0, phase=math.pi / 2, I=-1.0, J=-1.0, ref_area=0.0, sigma=0.0, q0=(0.0,) * 4,
                 per_cell=0, T_e=2.0, T_i=0.03, weight=1e6, dt=1e-11, seed=1234, precision=abi.PREC_FP64,
                 cathode_phi=0.0, anode_phi=0.0):
    """A 1-D gap like the rlcCircuit tutorial: n cells along x over `length`
    (cross-section width x width, empty y/z sides), the cathode ("source") at
    -x and the anode ("collector", fixedValue) at +x, both circuit
    electrodes of `model`: circuitRLC (R, C, L, V sin(omega t + phase)),
    IdealVoltageSource (both fixedValue) or IdealCurrentSource (I / J into
    the cathode's circuitBoundary).  per_cell > 0 fills the gap with e- and
    Ar+ parcels of `weight` at T_e / T_i eV."""
    cathode_bc = {abi.CIRCUIT_RLC: abi.PHI_RLC, abi.CIRCUIT_IDEAL_VOLTAGE: abi.PHI_FIXED_VALUE,
                  abi.CIRCUIT_IDEAL_CURRENT: abi.PHI_CIRCUIT_GRADIENT}[model]
    sides = [patch(abi.PATCH_CIRCUIT, cathode_phi, cathode_bc), patch(abi.PATCH_CIRCUIT, anode_phi),
             patch(abi.PATCH_EMPTY), patch(abi.PATCH_EMPTY), patch(abi.PATCH_EMPTY), patch(abi.PATCH_EMPTY)]
    mesh = block_mesh((n, 1, 1), (length, width, width), sides)
    cfg = base_config(dt, [(M_E, -E_CHARGE, weight, True), (M_AR, E_CHARGE, weight, True)],
                      precision=precision, deposit=abi.DEPOSIT_FIXED_POINT, seed=seed)
    c = cfg.circuit
    c.model = model
    c.cathode_patch, c.anode_patch = 0, 1
    c.R, c.L, c.C, c.V, c.omega, c.phase = R, L, C, V, omega, phase
    for i in range(4):
        c.Q[i] = q0[i]
    c.sigma = sigma
    c.I, c.J, c.ref_area = I, J, ref_area
    particles = {}
    if per_cell > 0:
        rng = np.random.Generator(np.random.Philox(seed))
        for s, (m, T) in enumerate(((M_E, T_e), (M_AR, T_i))):
            tet, bary = uniform_in_cells(rng, np.arange(n), per_cell)
            U = rng.standard_normal((len(tet), 3)) * math.sqrt(T * E_CHARGE / m)
            particles[s] = (tet, bary, U)
    return Case("circuit", mesh, cfg, particles, [], dict(area=width * width))


def neutral_gas(n_cells=4, per_cell=50, n=1e21, T=300.0, T_x=None, d=4.17e-10, L=4e-4, dt=1e-7, seed=1234,
                precision=abi.PREC_FP64, cross_section=abi.XS_HARD_SPHERE, omega=0.5, tref=273.0,
                weight_correction=0, background=None):
    """Neutral argon parcels (charge 0) in a periodic box with binary (DSMC)
    collisions, MaxwellSolver none: BinaryCollisionModel IsotropicScattering
    with hard spheres (or VHS).  T_x != T starts anisotropic; background =
    (n_bg, T_bg) adds collisions with a background argon gas."""
    sides = [patch(abi.PATCH_CYCLIC) for _ in range(6)]
    mesh = block_mesh((n_cells,) * 3, (L,) * 3, sides)
    n_c = n_cells ** 3
    N = n_c * per_cell
    w = n * L ** 3 / N
    cfg = base_config(dt, [(M_AR, 0.0, w, True)], maxwell=abi.MAXWELL_NONE, precision=precision, seed=seed,
                      electron_species=-1)
    b = cfg.binary
    b.enabled = 1
    b.cross_section = cross_section
    b.weight_correction = weight_correction
    b.diameter[0] = d
    b.omega[0] = omega
    b.tref = tref
    b.init_temperature = T
    b.background_species = -1
    if background is not None:
        b.background_species = 0
        cfg.mcc.gas_density = background[0]
        cfg.mcc.gas_temperature = background[1]
        cfg.mcc.gas_mass = M_AR
    rng = np.random.Generator(np.random.Philox(seed))
    tet, bary = uniform_in_cells(rng, np.arange(n_c), per_cell)
    vt = math.sqrt(K_B * T / M_AR)
    vx = math.sqrt(K_B * (T if T_x is None else T_x) / M_AR)
    U = rng.standard_normal((N, 3)) * np.array([vx, vt, vt])
    return Case("neutral_gas", mesh, cfg, {0: (tet, bary, U)}, [], dict(n=n, T=T, w=w, N=N, d=d, V=L ** 3))


def build_ensemble(case, backend=None):
    """Create an ensemble Simulation (one context, n_cases mesh copies)."""
    from .simulation import EnsembleBackend, Simulation
    be = backend if backend is not None else EnsembleBackend(case.meta["n_cases"])
    sim = Simulation(case.mesh, case.cfg, backend=be, keepalive=case.keepalive)
    sim.set_case_efield(case.meta["E"])
    for s, (tet, bary, U) in case.particles.items():
        sim.set_particles(s, tet, bary, U)
    return sim


def build(case, backend=None):
    """Create a Simulation for the case and upload its particles."""
    from .simulation import Simulation
    sim = Simulation(case.mesh, case.cfg, backend=backend, keepalive=case.keepalive)
    for s, (tet, bary, U) in case.particles.items():
        sim.set_particles(s, tet, bary, U)
    return sim
