"""Ion collisions with neutral parcels in the oracle (no GPU)
(IonNeutralCollisionModel::performCollisions): events at the NTC rate,
momentum and energy of the ion-neutral system kept by isotropic elastic
scattering and charge exchange of equal masses, neutral velocities kept
when updateNeutralVelocity is off."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases


def run(oracle_backend, steps, **kw):
    case = cases.ion_neutral_parcels(**kw)
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    stats = [sim.step(1) for _ in range(steps)]
    return case, sim, stats


def momentum_energy(sim, case):
    P, K = np.zeros(3), 0.0
    for s in (0, 1):
        _, _, U = sim.get_particles(s)
        m = case.cfg.species[s].mass
        P += m * U.sum(axis=0)
        K += 0.5 * m * (U * U).sum()
    return P, K


def test_rate_and_conservation(oracle_backend):
    case = cases.ion_neutral_parcels()
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    P0, K0 = momentum_energy(sim, case)
    st = [sim.step(1) for _ in range(3)]
    events = sum(s.ion_mcc_elastic + s.ion_mcc_charge_exchange for s in st)
    cands = sum(s.ion_mcc_candidates for s in st)
    assert events > 300 and cands >= events
    assert sum(s.ion_mcc_elastic for s in st) > 0 and sum(s.ion_mcc_charge_exchange for s in st) > 0
    P1, K1 = momentum_energy(sim, case)
    scale = np.abs(P0).max() + 1e-30 + case.cfg.species[1].mass * 1e4 * 1920
    assert np.abs(P1 - P0).max() <= 1e-9 * scale
    assert K1 == pytest.approx(K0, rel=1e-12)


def test_neutral_velocity_kept_when_asked(oracle_backend):
    case, sim, st = run(oracle_backend, 0, keep_neutral_velocity=True)
    _, _, U0 = sim.get_particles(0)
    st = [sim.step(1) for _ in range(2)]
    assert sum(s.ion_mcc_elastic for s in st) > 0
    _, _, U1 = sim.get_particles(0)
    np.testing.assert_array_equal(U0, U1)
