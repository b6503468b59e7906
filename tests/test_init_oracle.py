"""The oracle's restatement of picInitialise (no GPU): every InitializationModel
places what its picFoam source says it places -- per-tet counts n V / w,
given temperatures and drifts, Tperp/Tpara, cellCount parcels per cell, the
sinusoidally displaced lattice -- the empty-axis constraint holds, the
leapfrog back-step matches the Boris half kick, and the fixed-operation
logarithm and sine of the sampler agree with the C library."""
import math

import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import Mesh, PicError

K_B, E, M_E, M_AR = cases.K_B, cases.E_CHARGE, cases.M_E, cases.M_AR


@pytest.fixture(scope="module")
def oracle(oracle_backend):
    return oracle_backend


def osim(oracle, case):
    return cases.build(case, backend=oracle.OracleBackend(1))


def particles(sim, s):
    tet, bary, U = sim.get_particles(s)
    return tet, bary, U


def test_det_log_and_sin_match_libm(oracle):
    lib = oracle.load()
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.random(2000), 10.0 ** rng.uniform(-300, 0, 2000), [1.0, 0.5, 0.25, 1e-308]])
    err = max(abs(lib.oracle_det_log(float(x)) - math.log(x)) / max(abs(math.log(x)), 1e-300) for x in xs
              if math.log(x) != 0.0)
    assert err < 4e-16
    assert lib.oracle_det_log(1.0) == 0.0
    for x in np.concatenate([rng.uniform(-60, 60, 3000), [0.0, math.pi, 0.5 * math.pi]]):
        assert abs(lib.oracle_det_sin(float(x)) - math.sin(x)) < 2e-15 * max(1.0, abs(x))


def test_equipartition_counts_temperature_drift(oracle):
    case = cases.empty_case(n_cells=(6, 6, 6), length=(0.006, 0.006, 0.006))
    n, T = 2e15, 3.0  # 1/m^3, eV
    init = cases.init_config(abi.INIT_EQUIPARTITION, number_density=(n, n), temperature=(T, 0.1),
                             electron_volt=True, velocity=(1e3, -2e3, 0.0))
    sim = osim(oracle, case)
    st = sim.initialise(init)
    V = 0.006 ** 3
    expect = n * V / 1e4                                # particles per species
    for s in (0, 1):
        assert abs(st.added[s] - expect) < 5 * math.sqrt(expect)
        tet, bary, U = particles(sim, s)
        assert len(tet) == st.added[s]
        # every cell has about n V_cell / w; no empty cell
        assert st.occupancy_min[s] > 0 and st.occupancy_max[s] < 2 * expect / 216
        assert np.all(bary >= 0) and np.all(bary.sum(axis=1) <= 1.0 + 1e-15)
    _, _, Ue = particles(sim, 0)
    assert np.allclose(Ue.mean(axis=0), (1e3, -2e3, 0.0), atol=5 * math.sqrt(K_B * T * E / K_B / M_E / len(Ue)) * 2)
    assert abs(st.temperature[0] / (T * E / K_B) - 1) < 0.03
    assert st.model_temperature[0] == pytest.approx(T * E / K_B)   # given, not calculated
    assert st.debye_length > 0 and st.mesh_volume == pytest.approx(V)
    # same seed: same particles; another seed: others
    sim2 = osim(oracle, case)
    sim2.initialise(init)
    assert all(np.array_equal(a, b) for a, b in zip(particles(sim, 0), particles(sim2, 0)))
    init.seed = 99
    sim2.initialise(init)
    assert not np.array_equal(particles(sim, 0)[2], particles(sim2, 0)[2])


def test_maxwellian_component_spreads(oracle):
    case = cases.empty_case(n_cells=(5, 5, 5), length=(0.005,) * 3)
    vt, vd = (1e5, 2e5, 3e5), (1e4, 0.0, -1e4)
    init = cases.init_config(abi.INIT_MAXWELLIAN, number_density=(4e15, 0.0), thermal_velocity=(vt, (0, 0, 0)),
                             drift_velocity=(vd, (0, 0, 0)))
    sim = osim(oracle, case)
    st = sim.initialise(init)
    assert st.added[1] == 0
    _, _, U = particles(sim, 0)
    assert len(U) > 30000
    assert np.allclose(U.std(axis=0) / vt, 1.0, atol=0.03)
    assert np.allclose(U.mean(axis=0), vd, atol=4 * max(vt) / math.sqrt(len(U)))
    # Maxwellian calculates the temperature (picInitialise.C:146-147)
    assert st.model_temperature[0] == st.temperature[0]


def test_isotropization_tpara_tperp(oracle):
    case = cases.empty_case(n_cells=(6, 6, 6), length=(0.006,) * 3)
    init = cases.init_config(abi.INIT_ISOTROPIZATION, number_density=(3e15, 0.0), temperature=(4.0 / 3.0, 0.0),
                             electron_volt=True, tperp_over_tpara=0.5)
    sim = osim(oracle, case)
    sim.initialise(init)
    _, _, U = particles(sim, 0)
    Ta = M_E * (U ** 2).mean(axis=0) / E      # eV per axis
    assert abs(Ta[0] - 2.0) < 0.05 and abs(Ta[1] - 1.0) < 0.03 and abs(Ta[2] - 1.0) < 0.03


def test_quasineutral_plasma(oracle):
    case = cases.empty_case(n_cells=(4, 4, 4), length=(0.004,) * 3,
                            species=[(M_E, -E, 1e4, True), (M_AR, E, 2e4, True)])
    init = cases.init_config(abi.INIT_QUASINEUTRAL_PLASMA, temperature=(2.0, 0.05), electron_volt=True,
                             cell_count=1e5, ion_species=1, use_maxwellian=False)
    sim = osim(oracle, case)
    st = sim.initialise(init)
    assert st.added[0] == 10 * 64 and st.added[1] == 5 * 64          # cellCount / nParticle per cell
    assert st.occupancy_min[0] == st.occupancy_max[0] == 10
    for s, (m, T) in enumerate(((M_E, 2.0), (M_AR, 0.05))):
        tet, _, U = particles(sim, s)
        assert np.all(tet % 12 != 11)                                 # label((12 - 1) U01): tets 0..10
        sp = np.sqrt((U ** 2).sum(axis=1))
        assert np.allclose(sp, math.sqrt(3 * T * E / m), rtol=1e-14)
        assert np.all(U > 0)                                          # sample01 direction: positive octant
    init.use_maxwellian = 1
    st = sim.initialise(init)
    assert abs(st.temperature[0] / (2.0 * E / K_B) - 1) < 0.15
    init.ion_species = 0
    with pytest.raises(PicError):
        sim.initialise(init)


def test_uniform_displacement_lattice(oracle):
    n, L = 64, 0.1
    dx = L / n
    sides = [cases.patch(abi.PATCH_CYCLIC), cases.patch(abi.PATCH_CYCLIC)] + \
            [cases.patch(abi.PATCH_EMPTY) for _ in range(4)]
    case = cases.empty_case(n_cells=(n, 1, 1), length=(L, dx, dx), sides=sides, origin=(0.0, -dx / 2, -dx / 2),
                            species=[(M_E, -E, 1.0, True)])
    lo, hi = (0.5 * dx, -0.25 * dx, -0.25 * dx), (L - 0.5 * dx, 0.25 * dx, 0.25 * dx)
    init = cases.init_config(abi.INIT_UNIFORM_DISPLACEMENT, temperature=(0.0,), species=(0,), min=lo, max=hi,
                             particle_numbers=(200, 3, 2), cycles=4, displacement=(0.2 * dx,),
                             displacement_dir=(2.0, 0.0, 0.0))
    sim = osim(oracle, case)
    st = sim.initialise(init)
    assert st.added[0] == 200 * 3 * 2
    tet, bary, U = particles(sim, 0)
    assert np.all(U == 0.0)
    mesh = Mesh(case.mesh)
    xyz = mesh.position(tet, bary)
    span = np.array(hi) - np.array(lo)
    delta = span / np.maximum(np.array([200, 3, 2]) - 1, 2)          # max(particleNumbers - 1, 2)
    i, j, k = np.meshgrid(np.arange(200), np.arange(3), np.arange(2), indexing="ij")
    p = np.stack([lo[0] + delta[0] * i, lo[1] + delta[1] * j, lo[2] + delta[2] * k], -1).reshape(-1, 3)
    p[:, 0] += 0.2 * dx * np.sin((p[:, 0] - lo[0]) / span[0] * 4 * math.pi)
    assert np.abs(xyz - p).max() < 1e-12 * L
    # a lattice that leaves the mesh is an error, as mesh.findCell < 0 in picFoam
    init.max[0] = 2 * L
    with pytest.raises(PicError):
        sim.initialise(init)


def test_reduced_dimension_constraint(oracle):
    case = cases.plasma_oscillation_1d(Mesh, n_cells=32, per_cell=1)
    case.particles = {}
    # y and z span [0, dx]: the constrained coordinate 0 lies on the cell face
    init = cases.init_config(abi.INIT_EQUIPARTITION, number_density=(1e14 * 3000,), temperature=(1.0,),
                             electron_volt=True)
    sim = osim(oracle, case)
    st = sim.initialise(init)
    assert st.added[0] > 1000
    tet, bary, U = particles(sim, 0)
    xyz = Mesh(case.mesh).position(tet, bary)
    assert np.abs(xyz[:, 1:]).max() < 1e-15


def test_leapfrog_is_the_boris_half_kick(oracle):
    case = cases.empty_case(n_cells=(3, 3, 3), length=(0.003,) * 3, species=[(M_E, -E, 1e4, True)])
    case.cfg.maxwell_solver = abi.MAXWELL_NONE
    case.cfg.E_applied[0] = 2e4
    case.cfg.dt = 1e-11
    base = cases.init_config(abi.INIT_EQUIPARTITION, number_density=(1e15,), temperature=(1.0,), electron_volt=True)
    a = osim(oracle, case)
    a.initialise(base)
    lf = cases.init_config(abi.INIT_EQUIPARTITION, number_density=(1e15,), temperature=(1.0,), electron_volt=True,
                           leapfrog=True)
    b = osim(oracle, case)
    b.initialise(lf)
    _, _, U0 = particles(a, 0)
    _, _, U1 = particles(b, 0)
    # U1 - U0 = -(q/m) E dt / 2 up to the relativistic factors of the Boris
    # push, O(v^2/c^2) ~ 1e-5 at these speeds
    dv = -(-E / M_E) * 2e4 * 1e-11 / 2
    assert np.allclose(U1[:, 0] - U0[:, 0], dv, rtol=1e-4)
    # the other components change only through the Lorentz factor (v dv / c^2)
    assert np.allclose(U1[:, 1:], U0[:, 1:], rtol=1e-6)
