"""A picFoam case directory run on the GPU: the case written by
tests/test_ofcase.py (permuted block axes, SimpleInjection, a floating
electrode, Maxwellian start with leapfrog) stepped on the GPU and in the
oracle -- particles and potential bit for bit -- and the case runner
writing its time directories."""
import os

import numpy as np
import pytest

from picfoam_gb300 import abi, ofcase, run

from test_ofcase import make_case

pytestmark = pytest.mark.gpu


def test_case_directory_matches_oracle(gpu, oracle_backend, tmp_path):
    make_case(str(tmp_path))
    c = ofcase.load_case(str(tmp_path))
    g = c.build(backend=gpu)
    o = c.build(backend=oracle_backend.OracleBackend(1))
    for sim in (g, o):
        sim.step(3)
    for s in (0, 1):
        tg, bg, ug = g.get_particles(s)
        to, bo, uo = o.get_particles(s)
        assert len(tg) > 100
        assert np.array_equal(tg, to) and np.array_equal(bg, bo) and np.array_equal(ug, uo)
    assert np.array_equal(g.field(abi.FIELD_PHI), o.field(abi.FIELD_PHI))


def test_case_runner_writes_time_directories(gpu, tmp_path):
    make_case(str(tmp_path))
    assert run.main([str(tmp_path), "--write-mesh"]) == 0
    for t in ("2e-12", "4e-12"):
        d = os.path.join(str(tmp_path), t)
        assert os.path.exists(os.path.join(d, "phiE")) and os.path.exists(os.path.join(d, "lagrangian", "pic", "U"))
    assert os.path.exists(os.path.join(str(tmp_path), "constant", "polyMesh", "faces"))
    phi = ofcase.read_field(os.path.join(str(tmp_path), "4e-12", "phiE"))
    assert np.all(np.isfinite(phi)) and phi.shape == (120,)
