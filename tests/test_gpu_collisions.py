"""Collision kernels on the GPU against the CPU oracle.

Both sides draw from the same counter-based Philox streams (one per cell and
step) in the same order, so in the FP64 form the runs agree to round-off of
the transcendental functions (pow, log, cos, sin differ by an ulp between
CUDA and the C library); the mixed form is compared statistically.
"""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from test_collisions import constant_xs_swarm

pytestmark = pytest.mark.gpu


def run_pair(case, gpu, oracle_backend, steps, nthreads=4):
    g = cases.build(case, backend=gpu)
    o = cases.build(case, backend=oracle_backend.OracleBackend(nthreads))
    sg, so = [], []
    for _ in range(steps):
        sg.append(g.step(1))
        so.append(o.step(1))
    return g, o, sg, so


def test_mcc_elastic_fp64_matches_oracle(gpu, oracle_backend):
    case = constant_xs_swarm(N=20000)
    g, o, sg, so = run_pair(case, gpu, oracle_backend, 4)
    for a, b in zip(sg, so):
        assert a.mcc_candidates == b.mcc_candidates
        assert abs(a.mcc_elastic - b.mcc_elastic) <= 2
    tg, bg, ug = g.get_particles(0)
    to, bo, uo = o.get_particles(0)
    np.testing.assert_array_equal(tg, to)
    close = np.isclose(ug, uo, rtol=1e-9, atol=1e-9 * np.abs(uo).max()).all(axis=1)
    assert close.mean() > 0.999


def test_mcc_ionisation_fp64_matches_oracle(gpu, oracle_backend):
    case = cases.electron_swarm(nx=4, ny=4, nz=16, N=4000, Ez=0.0, T_e=60.0, precision=abi.PREC_FP64,
                                size=(0.004, 0.004, 0.016))
    for s in range(6):
        case.mesh.side[s].kind = abi.PATCH_CYCLIC
    g, o, sg, so = run_pair(case, gpu, oracle_backend, 10)
    iz_g = sum(s.mcc_ionization for s in sg)
    iz_o = sum(s.mcc_ionization for s in so)
    assert iz_o > 0
    assert abs(iz_g - iz_o) <= max(2, iz_o // 100)
    assert abs(g.count(0) - o.count(0)) <= max(2, iz_o // 100)
    assert abs(g.count(1) - o.count(1)) <= max(2, iz_o // 100)


def test_coulomb_fp64_matches_oracle(gpu, oracle_backend):
    case = cases.coulomb_thermalisation(n_cells=4, per_cell=60, L=2e-5)
    g, o, sg, so = run_pair(case, gpu, oracle_backend, 5)
    for a, b in zip(sg, so):
        assert a.coulomb_pairs == b.coulomb_pairs > 0
    _, _, ug = g.get_particles(0)
    _, _, uo = o.get_particles(0)
    close = np.isclose(ug, uo, rtol=1e-8, atol=1e-8 * np.abs(uo).max()).all(axis=1)
    assert close.mean() > 0.99


def test_coulomb_mixed_isotropisation_rate(gpu, oracle_backend):
    case = cases.coulomb_thermalisation(n_cells=4, per_cell=800, L=2e-5)
    o = cases.build(case, backend=oracle_backend.OracleBackend(4))
    case.cfg.precision = abi.PREC_MIXED
    g = cases.build(case, backend=gpu)

    def anis(sim):
        d = sim.diagnostics()
        v = np.array(d.velocity_sq[0]) / d.weight_sum[0]
        return v[0] / (0.5 * (v[1] + v[2]))

    for _ in range(2):
        g.step(25)
        o.step(25)
        # 51200 electrons: the two runs' anisotropies each carry about 1.2 %
        # of sampling noise (their trajectories decorrelate), so 0.05 is ~3 sigma
        assert abs(anis(g) - anis(o)) < 0.05


def close_fraction(g, o, species, rtol):
    tg, _, ug = g.get_particles(species)
    to, _, uo = o.get_particles(species)
    np.testing.assert_array_equal(tg, to)
    return np.isclose(ug, uo, rtol=rtol, atol=rtol * np.abs(uo).max()).all(axis=1).mean()


def test_ion_mcc_fp64_matches_oracle(gpu, oracle_backend):
    case = cases.ion_swarm(N=20000, T_gas=300.0, sigma_el=5e-19, sigma_cx=2.5e-19, steps_dt=0.05)
    g, o, sg, so = run_pair(case, gpu, oracle_backend, 4)
    for a, b in zip(sg, so):
        assert a.ion_mcc_candidates == b.ion_mcc_candidates > 0
        assert abs(a.ion_mcc_elastic - b.ion_mcc_elastic) <= 2
        assert abs(a.ion_mcc_charge_exchange - b.ion_mcc_charge_exchange) <= 2
    assert close_fraction(g, o, 0, 1e-9) > 0.999


def test_ion_charge_exchange_mixed_thermalises(gpu):
    case = cases.ion_swarm(N=4000, n_cells=(4, 4, 4), T_i=1.0, T_gas=300.0, sigma_el=0.0, sigma_cx=5e-19,
                           steps_dt=0.2, precision=abi.PREC_MIXED)
    sim = cases.build(case, backend=gpu)
    sim.step(200)
    _, _, U = sim.get_particles(0)
    e_mean = 0.5 * cases.M_AR * (U * U).sum(axis=1).mean()
    assert abs(e_mean / (1.5 * cases.K_B * 300.0) - 1.0) < 0.08


def test_relativistic_scatter_fp64_matches_oracle(gpu, oracle_backend):
    case = constant_xs_swarm(N=20000)
    case.cfg.mcc.scatter = 1
    g, o, sg, so = run_pair(case, gpu, oracle_backend, 4)
    for a, b in zip(sg, so):
        assert a.mcc_candidates == b.mcc_candidates
        assert abs(a.mcc_elastic - b.mcc_elastic) <= 2
    assert close_fraction(g, o, 0, 1e-9) > 0.999


@pytest.mark.parametrize("collide", [abi.COLLIDE_NANBU, abi.COLLIDE_PEREZ])
def test_takizuka_abe_fp64_matches_oracle(gpu, oracle_backend, collide):
    # ragged per-cell counts: empty, single, odd and unequal cells
    case = cases.coulomb_relaxation(ragged=True, pairing=abi.PAIRING_TAKIZUKA_ABE, collide=collide)
    g, o, sg, so = run_pair(case, gpu, oracle_backend, 4)
    for a, b in zip(sg, so):
        assert a.coulomb_pairs == b.coulomb_pairs > 0
    for s in range(2):
        assert close_fraction(g, o, s, 1e-8) > 0.99


def test_computed_coulomb_log_fp64_matches_oracle(gpu, oracle_backend):
    case = cases.coulomb_relaxation(ragged=True, coulomb_log=0.0, collide=abi.COLLIDE_PEREZ)
    g, o, sg, so = run_pair(case, gpu, oracle_backend, 4)
    for a, b in zip(sg, so):
        assert a.coulomb_pairs == b.coulomb_pairs > 0
    for s in range(2):
        assert close_fraction(g, o, s, 1e-8) > 0.99


def test_weight_correction_fp64_matches_oracle(gpu, oracle_backend):
    case = cases.coulomb_relaxation(w_i_factor=2.0, weight_correction=1, coulomb_log=0.0)
    g, o, sg, so = run_pair(case, gpu, oracle_backend, 4)
    for a, b in zip(sg, so):
        assert a.coulomb_pairs == b.coulomb_pairs > 0
    for s in range(2):
        assert close_fraction(g, o, s, 1e-8) > 0.99


@pytest.mark.parametrize("wc,collide", [(abi.WEIGHT_CORRECTION_SENTOKU_KEMP_NR, abi.COLLIDE_NANBU),
                                        (abi.WEIGHT_CORRECTION_SENTOKU_KEMP, abi.COLLIDE_PEREZ)])
def test_sentoku_kemp_fp64_matches_oracle(gpu, oracle_backend, wc, collide):
    case = cases.coulomb_relaxation(w_i_factor=2.5, weight_correction=wc, collide=collide, m_i=4.0 * cases.M_E,
                                    T_i=1.0, ragged=True)
    g, o, sg, so = run_pair(case, gpu, oracle_backend, 4)
    for a, b in zip(sg, so):
        assert a.coulomb_pairs == b.coulomb_pairs > 0
    for s in range(2):
        assert close_fraction(g, o, s, 1e-8) > 0.99



@pytest.mark.parametrize("xs,omega,background", [(abi.XS_HARD_SPHERE, 0.5, None),
                                                 (abi.XS_VARIABLE_HARD_SPHERE, 0.81, None),
                                                 (abi.XS_HARD_SPHERE, 0.5, (2e21, 300.0))])
def test_binary_collisions_fp64_match_oracle(gpu, oracle_backend, xs, omega, background):
    """BinaryCollisionModel: the same candidates per step (the NTC counts
    depend on the running (sigma_T c_r)_max), collisions within a few (the
    acceptance draws compare against transcendental results), and velocities
    equal to round-off for nearly all parcels."""
    case = cases.neutral_gas(n_cells=4, per_cell=50, cross_section=xs, omega=omega, background=background,
                             n=1e21 if background is None else 2e19)
    g, o, sg, so = run_pair(case, gpu, oracle_backend, 4)
    for a, b in zip(sg, so):
        assert abs(a.binary_candidates - b.binary_candidates) <= 2
        assert abs(a.binary_collisions - b.binary_collisions) <= 2
        assert abs(a.binary_background_collisions - b.binary_background_collisions) <= 2
    assert sum(a.binary_collisions + a.binary_background_collisions for a in sg) > 50
    assert close_fraction(g, o, 0, 1e-9) > 0.99


def test_binary_collisions_fp32_conserve_energy(gpu):
    case = cases.neutral_gas(n_cells=4, per_cell=50, precision=abi.PREC_MIXED)
    g = cases.build(case, backend=gpu)
    _, _, U0 = g.get_particles(0)
    st = g.step(4)
    _, _, U1 = g.get_particles(0)
    assert st.binary_collisions > 20
    assert abs((U1 * U1).sum() / (U0 * U0).sum() - 1) < 1e-5
