"""Perez ionisation on the GPU against the oracle, through the C ABI
(PerezIonizationModel.C:129-385 inside the Coulomb pairing; argon from the
thermalization tutorial's PerezIonizationCoeffs).

Both sides draw the same Philox streams (the ionisation draws of a collision
from the stream of its ordinal), so in the FP64 form they make the same
ionisations: the same counts, the same charge modifiers, the same new
electron parcels (appended in picFoam's sequential order) with the ions'
nParticle, and velocities equal to round-off of the transcendental
functions; with unequal electron and ion weights as well (then an
ionisation changes the ion with probability wE / wP and the electron with
wP / wE).  In the FP32 form the ionisation count agrees statistically.
"""
import json
import os
import sys

import numpy as np
import pytest

from picfoam_gb300 import abi, cases

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import tutorial_cases  # noqa: E402

pytestmark = pytest.mark.gpu


def argon():
    with open(os.path.join(HERE, "golden", "tutorials", "thermalization_perez.json")) as f:
        return tutorial_cases.from_json(abi.Perez(), json.load(f)["cfg"]["perez"])


@pytest.mark.parametrize("w_i_factor,collide", [(1.0, abi.COLLIDE_NANBU), (2.0, abi.COLLIDE_PEREZ)])
def test_perez_ionisation_fp64_matches_oracle(gpu, oracle_backend, w_i_factor, collide):
    case = cases.perez_plasma(argon(), w_i_factor=w_i_factor, collide=collide)
    g = cases.build(case, backend=gpu)
    o = cases.build(case, backend=oracle_backend.OracleBackend(4))
    total = 0
    for _ in range(3):
        sg, so = g.step(1), o.step(1)
        assert sg.coulomb_pairs == so.coulomb_pairs > 0
        assert (sg.coulomb_ionizations, sg.coulomb_ionization_electrons) == \
               (so.coulomb_ionizations, so.coulomb_ionization_electrons)
        total += sg.coulomb_ionizations
    assert total > 0
    for s in range(2):
        tg, bg, ug = g.get_particles(s)
        to, bo, uo = o.get_particles(s)
        np.testing.assert_array_equal(tg, to)
        close = np.isclose(ug, uo, rtol=1e-8, atol=1e-8 * np.abs(uo).max()).all(axis=1)
        assert close.mean() > 0.99
        for a, b in zip(g.get_parcel_attributes(s), o.get_parcel_attributes(s)):
            np.testing.assert_array_equal(a, b)


def test_perez_ionisation_fp32_rate(gpu, oracle_backend):
    case = cases.perez_plasma(argon(), precision=abi.PREC_MIXED, e_per_cell=60, i_per_cell=60)
    g = cases.build(case, backend=gpu)
    case.cfg.precision = abi.PREC_FP64
    o = cases.build(case, backend=oracle_backend.OracleBackend(4))
    ng = no = 0
    for _ in range(3):
        ng += g.step(1).coulomb_ionizations
        no += o.step(1).coulomb_ionizations
    assert no > 50
    # independent-looking counts: within 4 sigma of each other
    assert abs(ng - no) <= 4.0 * np.sqrt(2.0 * no)
    _, z = g.get_parcel_attributes(1)
    assert z.min() >= 1 and z.max() <= 5
