"""Collision models on the CPU oracle: null-collision MCC against a
background gas and binary Coulomb collisions (known answers)."""
import ctypes as C
import math

import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import Mesh


def constant_xs_swarm(sigma=1e-19, n_gas=1e21, N=20000, T_e=10.0, seed=5, steps_dt=0.01, cells=(8, 8, 8)):
    """Periodic box, no field, constant elastic cross section, cold gas:
    the elastic collision rate is n sigma |v|."""
    case = cases.electron_swarm(nx=cells[0], ny=cells[1], nz=cells[2], N=N, Ez=0.0, gas_density=n_gas,
                                T_gas=1e-3, T_e=T_e, seed=seed, precision=abi.PREC_FP64, ion_species=False,
                                size=(0.01, 0.01, 0.01))
    for s in range(6):
        case.mesh.side[s].kind = abi.PATCH_CYCLIC
    e = np.array([0.0, 1e4])
    el = np.array([sigma, sigma])
    zero = np.zeros(2)
    arrs = [np.ascontiguousarray(a) for a in (e, el, zero, zero.copy())]
    mc = case.cfg.mcc
    mc.n_xs = 2
    mc.xs_energy, mc.xs_elastic, mc.xs_excitation, mc.xs_ionization = [
        a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]
    case.keepalive = arrs
    vmax = math.sqrt(2 * cases.E_CHARGE * 200 * T_e / cases.M_E)
    mc.sigma_v_max_init = sigma * vmax
    case.cfg.dt = steps_dt / (n_gas * sigma * vmax)
    return case


def test_mcc_elastic_rate_matches_n_sigma_v(oracle_backend):
    case = constant_xs_swarm()
    sim = cases.build(case, backend=oracle_backend.OracleBackend(4))
    n_gas, sigma, dt = case.cfg.mcc.gas_density, 1e-19, case.cfg.dt
    expected = 0.0
    got = 0
    for _ in range(10):
        _, _, U = sim.get_particles(0)
        expected += n_gas * sigma * dt * np.linalg.norm(U, axis=1).sum()
        st = sim.step(1)
        got += st.mcc_elastic
        assert st.mcc_excitation == 0 and st.mcc_ionization == 0
    assert abs(got - expected) < 4 * math.sqrt(expected)
    # elastic scattering off a cold, heavy gas keeps the electron energy to ~2 m/M
    d = sim.diagnostics()
    assert d.kinetic_energy[0] > 0


def test_mcc_ionisation_grows_population(oracle_backend):
    case = cases.electron_swarm(nx=4, ny=4, nz=16, N=4000, Ez=0.0, T_e=60.0, precision=abi.PREC_FP64,
                                size=(0.004, 0.004, 0.016))
    for s in range(6):
        case.mesh.side[s].kind = abi.PATCH_CYCLIC
    sim = cases.build(case, backend=oracle_backend.OracleBackend(2))
    n0 = sim.count(0)
    st = sim.step(20)
    assert st.mcc_ionization > 0
    assert sim.count(0) == n0 + st.mcc_ionization
    assert sim.count(1) == st.mcc_ionization


def test_coulomb_conserves_momentum_and_energy(oracle_backend):
    case = cases.coulomb_thermalisation(n_cells=4, per_cell=60, L=2e-5)
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    d0 = sim.diagnostics()
    st = sim.step(5)
    assert st.coulomb_pairs > 0
    d1 = sim.diagnostics()
    # Nanbu collide exchanges momentum pairwise with equal weights: total
    # momentum and kinetic energy are conserved to round-off
    p0 = np.array(d0.momentum[0])
    p1 = np.array(d1.momentum[0])
    scale = math.sqrt(2 * cases.M_E * d0.kinetic_energy[0] / d0.weight_sum[0]) * d0.weight_sum[0]
    assert np.abs(p1 - p0).max() < 1e-9 * scale
    assert abs(d1.kinetic_energy[0] / d0.kinetic_energy[0] - 1) < 1e-9


def test_coulomb_isotropises(oracle_backend):
    case = cases.coulomb_thermalisation(n_cells=4, per_cell=200, L=2e-5)
    sim = cases.build(case, backend=oracle_backend.OracleBackend(2))

    def anis():
        d = sim.diagnostics()
        v = np.array(d.velocity_sq[0]) / d.weight_sum[0]
        return v[0] / (0.5 * (v[1] + v[2]))

    a0 = anis()
    assert abs(a0 - 2.0) < 0.1
    sim.step(25)
    a1 = anis()
    sim.step(25)
    a2 = anis()
    # T_x / T_yz relaxes towards 1 monotonically (dt = 0.02 / nu, 50 steps ~ 1 relaxation time)
    assert a0 > a1 > a2 > 1.0
