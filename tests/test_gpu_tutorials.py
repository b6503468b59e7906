"""picFoam's tutorial cases on the GPU against the oracle, from the fixtures
tests/golden/tutorials/*.json (the tutorials' case directories mapped by
ofcase.load_case; tests/golden/make_tutorial_cases.py writes them).

Collisionless tutorials, FP64 with the order-independent fixed-point charge
deposit: particles, potential and absorbed counts bit for bit after several
steps.  Tutorials with collisions draw the same Philox streams on both sides:
the same collision counts, velocities equal to the round-off of the
transcendental functions for nearly every particle.
"""
import os
import sys

import numpy as np
import pytest

from picfoam_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import tutorial_cases  # noqa: E402

pytestmark = pytest.mark.gpu

FIXTURES = os.path.join(HERE, "golden", "tutorials")


def pair(name, gpu, oracle_backend, precision=abi.PREC_FP64, nthreads=4):
    cases = []
    for prec, be in ((precision, gpu), (abi.PREC_FP64, oracle_backend.OracleBackend(nthreads))):
        c = tutorial_cases.load(os.path.join(FIXTURES, name + ".json"), precision=prec)
        c.cfg.deposit_mode = abi.DEPOSIT_FIXED_POINT
        cases.append(c.build(backend=be))
    return cases


@pytest.mark.parametrize("name,steps", [("plasmaOscillation", 4), ("magneticRotation", 400), ("rlcCircuit", 10),
                                        ("floatingBoundary", 10), ("electricAcceleration", 50)])
def test_collisionless_tutorials_bit_exact(gpu, oracle_backend, name, steps):
    g, o = pair(name, gpu, oracle_backend)
    for _ in range(2):
        sg, so = g.step(steps // 2), o.step(steps // 2)
        assert list(sg.n_absorbed) == list(so.n_absorbed)
        assert (sg.tet_steps, sg.face_crossings) == (so.tet_steps, so.face_crossings)
    for s in range(g.cfg.n_species):
        for a, b in zip(g.get_particles(s), o.get_particles(s)):
            np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(g.field(abi.FIELD_PHI), o.field(abi.FIELD_PHI))
    if name == "rlcCircuit":
        assert sg.circuit_voltage == so.circuit_voltage and sg.circuit_current == so.circuit_current


def close_fraction(g, o, s, rtol=1e-8):
    tg, _, ug = g.get_particles(s)
    to, _, uo = o.get_particles(s)
    np.testing.assert_array_equal(tg, to)
    if len(uo) == 0:
        return 1.0
    return np.isclose(ug, uo, rtol=rtol, atol=rtol * np.abs(uo).max()).all(axis=1).mean()


@pytest.mark.parametrize("name", ["thermalization", "thermalization_binaryCollision", "ionization"])
def test_collision_tutorials_match_oracle(gpu, oracle_backend, name):
    g, o = pair(name, gpu, oracle_backend)
    for _ in range(3):
        sg, so = g.step(1), o.step(1)
        assert sg.coulomb_pairs == so.coulomb_pairs
        assert sg.binary_candidates == so.binary_candidates
        assert (sg.mcc_parcel_candidates, sg.mcc_parcel_ionization) == \
               (so.mcc_parcel_candidates, so.mcc_parcel_ionization)
    assert sg.coulomb_pairs + sg.binary_collisions + sg.mcc_parcel_ionization > 0
    for s in range(g.cfg.n_species):
        assert close_fraction(g, o, s) > 0.99


def test_plasma_oscillation_tutorial_fp32_close(gpu, oracle_backend):
    """The FP32 form on plasmaOscillation: the tutorial's lattice puts every
    particle on the centre line of its cell (y and z at the cell centres),
    which is an edge of the cell's tets, so the tet a rounding picks there is
    arbitrary; positions and velocities are compared instead: within 2e-5 of
    the cell size and 2e-5 relative after 4 steps."""
    from picfoam_gb300.simulation import Mesh
    g, o = pair("plasmaOscillation", gpu, oracle_backend, precision=abi.PREC_MIXED)
    desc = tutorial_cases.load(os.path.join(FIXTURES, "plasmaOscillation.json")).mesh
    m = Mesh(desc)
    h = min(desc.length[a] / desc.n[a] for a in range(3))
    g.step(4)
    o.step(4)
    for s in range(2):
        tg, bg, ug = g.get_particles(s)
        to, bo, uo = o.get_particles(s)
        assert len(tg) == len(to)
        assert (tg // 12 == to // 12).mean() > 0.999             # the same cells
        np.testing.assert_allclose(m.position(tg, bg), m.position(to, bo), rtol=0, atol=2e-5 * h)
        np.testing.assert_allclose(ug, uo, rtol=2e-5, atol=2e-5 * max(np.abs(uo).max(), 1e-30))
