"""Perez ionisation in the oracle (PerezIonizationModel.C:129-385, inside the
Coulomb pairing), with the argon coefficients of picFoam's thermalization
tutorial (tests/golden/tutorials/thermalization_perez.json): known answers
without a GPU.

* electrons of a few hundred eV ionise Ar+ further: ion charge modifiers
  rise, never past the ionisation limit (5), and each ionisation that
  raises a charge adds an electron parcel with the ion's nParticle, so the
  total charge (species charge x charge modifier x nParticle) is kept;
* the colliding electrons lose energy to the ionisation;
* an ionisation limit of 1 (Ar+ already at it) or the model switched off
  ionises nothing.
"""
import ctypes as C
import json
import os
import sys

import numpy as np
import pytest

from picfoam_gb300 import abi, cases

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import tutorial_cases  # noqa: E402


def argon():
    with open(os.path.join(HERE, "golden", "tutorials", "thermalization_perez.json")) as f:
        d = json.load(f)
    return tutorial_cases.from_json(abi.Perez(), d["cfg"]["perez"])


def charge(sim, case):
    q = 0.0
    for s in range(case.cfg.n_species):
        w, z = sim.get_parcel_attributes(s)
        q += case.cfg.species[s].charge * float(np.sum(w * z))
    return q


def kinetic(sim, case, s):
    _, _, U = sim.get_particles(s)
    w, _ = sim.get_parcel_attributes(s)
    return 0.5 * case.cfg.species[s].mass * float(np.sum(w * (U * U).sum(axis=1)))


def test_fixture_carries_argon():
    pz = argon()
    assert pz.enabled == 1 and pz.n_ions == 1
    ion = pz.ion[0]
    assert (ion.species, ion.atomic_number, ion.ionization_limit) == (1, 18, 5)
    assert ion.ionization_energy[0] == pytest.approx(15.7596117)


def test_ionisation_keeps_charge_and_limit(oracle_backend):
    case = cases.perez_plasma(argon())
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    q0 = charge(sim, case)
    n0 = sim.count(0)
    ions = 0
    added = 0
    for _ in range(4):
        st = sim.step(1)
        ions += st.coulomb_ionizations
        added += st.coulomb_ionization_electrons
    assert ions > 0 and added >= ions
    assert sim.count(0) == n0 + added
    _, z = sim.get_parcel_attributes(1)
    assert z.max() > 1 and z.max() <= 5 and z.min() >= 1
    w_e, z_e = sim.get_parcel_attributes(0)
    assert np.all(z_e == 1)
    # the new electrons (appended behind the old ones) carry the ion weight
    np.testing.assert_array_equal(w_e[n0:], case.cfg.species[1].weight)
    assert charge(sim, case) == pytest.approx(q0, rel=1e-12, abs=1e-12 * abs(q0) + 1e-30)


def test_ionisation_costs_electron_energy(oracle_backend):
    out = []
    for on in (0, 1):
        pz = argon()
        pz.enabled = on
        case = cases.perez_plasma(pz)
        sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
        sim.step(2)
        out.append((kinetic(sim, case, 0) + kinetic(sim, case, 1), sim.count(0)))
    assert out[1][1] > out[0][1]                 # ionisation added electrons
    assert out[1][0] < out[0][0]                 # and took kinetic energy


def test_no_ionisation_at_the_limit(oracle_backend):
    pz = argon()
    pz.ion[0].ionization_limit = 1               # Ar+ is at Z* = 1 already
    case = cases.perez_plasma(pz)
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    n0 = sim.count(0)
    st = sim.step(2)
    assert st.coulomb_ionizations == 0 and sim.count(0) == n0
