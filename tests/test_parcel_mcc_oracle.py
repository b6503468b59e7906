"""Electron collisions with neutral parcels in the oracle (no GPU), the
ionization tutorial's set-up (ElectronNeutralCollisionModel::performCollisions,
FixedValue ionisation above 15.76 eV): the ionisation rate against
N_e n_n sigma v dt, electron-ion pairs created and ionised neutrals deleted
(or kept with deleteNeutral off), ions born at the neutral parcel's position
with its velocity, and the checks."""
import math

import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import PicError

SIGMA = 3.43943e-20


def osim(oracle_backend, **kw):
    kw.setdefault("n_n", 1e22)
    kw.setdefault("dt", 4e-11)
    case = cases.neutral_parcel_ionization(**kw)
    return case, cases.build(case, backend=oracle_backend.OracleBackend(1))


def test_ionisation_rate(oracle_backend):
    case, sim = osim(oracle_backend)
    m = case.meta
    st = sim.step(1)
    expect = m["N_e"] * m["n_n"] * SIGMA * m["v_e"] * case.cfg.dt
    assert expect > 50
    assert abs(st.mcc_parcel_ionization - expect) < 4 * math.sqrt(expect)
    # every candidate is above threshold and (sigma c_R)_max is 1 % above sigma v
    assert st.mcc_parcel_ionization <= st.mcc_parcel_candidates and st.mcc_parcel_ionization > 0.95 * st.mcc_parcel_candidates


@pytest.mark.parametrize("keep", [False, True])
def test_pairs_created_and_neutrals_deleted(oracle_backend, keep):
    case, sim = osim(oracle_backend, keep_neutrals=keep)
    m = case.meta
    total = 0
    for _ in range(3):
        total += sim.step(1).mcc_parcel_ionization
    assert total > 100
    assert sim.count(2) == total and sim.count(0) == m["N_e"] + total
    assert sim.count(1) == m["N_n"] - (0 if keep else total)


def test_ions_born_at_the_neutral_parcel(oracle_backend):
    case, sim = osim(oracle_backend, keep_neutrals=True)
    sim.step(1)
    tn, bn, Un = sim.get_particles(1)
    ti, bi, Ui = sim.get_particles(2)
    assert len(ti) > 20
    key = {(int(t), *b.tolist()): u for t, b, u in zip(tn, bn, Un)}
    for t, b, u in zip(ti, bi, Ui):
        un = key[(int(t), *b.tolist())]           # an ion sits on a neutral parcel ...
        np.testing.assert_array_equal(u, un)      # ... with the neutral's scattered velocity


def test_neutral_velocity_kept_when_asked(oracle_backend):
    case, sim = osim(oracle_backend, keep_neutrals=True, keep_neutral_velocity=True)
    _, _, U0 = sim.get_particles(1)
    sim.step(1)
    _, _, U1 = sim.get_particles(1)
    # neutrals move only by tracking, their velocities never change
    np.testing.assert_array_equal(U0, U1)


def test_parcel_mcc_checks(oracle_backend):
    case = cases.neutral_parcel_ionization()
    case.cfg.species[1].charge = 1.0e-19                       # not a neutral species
    with pytest.raises(PicError):
        cases.build(case, backend=oracle_backend.OracleBackend(1))
    case = cases.neutral_parcel_ionization()
    case.cfg.species[2].weight *= 2                             # ion weight differs
    with pytest.raises(PicError):
        cases.build(case, backend=oracle_backend.OracleBackend(1))
