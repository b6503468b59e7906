"""The tutorial fixtures of tests/golden/tutorials (no GPU): each rebuilds a
case the oracle steps, and, where picFoam's tutorials are present
(PICFOAM_TUTORIALS), each still equals what ofcase.load_case maps the
tutorial to, so the fixtures cannot go stale."""
import glob
import json
import os
import sys

import pytest

from picfoam_gb300 import ofcase

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import tutorial_cases  # noqa: E402

FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "tutorials", "*.json")))
REF = os.environ.get("PICFOAM_TUTORIALS", "")


def test_all_tutorials_have_fixtures():
    names = {os.path.basename(p)[:-5] for p in FIXTURES}
    assert {"plasmaOscillation", "thermalization", "thermalization_binaryCollision", "ionization",
            "magneticRotation", "rlcCircuit", "floatingBoundary", "electricAcceleration"} <= names


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-5] for p in FIXTURES])
def test_fixture_runs_on_the_oracle(oracle_backend, path):
    case = tutorial_cases.load(path)
    sim = case.build(backend=oracle_backend.OracleBackend(4))
    assert sum(sim.count(s) for s in range(case.cfg.n_species)) > 0
    sim.step(1)


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="PICFOAM_TUTORIALS is not set to picFoam's tutorials")
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-5] for p in FIXTURES])
def test_fixture_matches_the_tutorial(path):
    name = os.path.basename(path)[:-5]
    with open(path) as f:
        stored = json.load(f)
    fresh = tutorial_cases.dump(ofcase.load_case(os.path.join(REF, name), allow_unsupported=True))
    assert json.loads(json.dumps(fresh)) == stored
