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


@pytest.mark.parametrize("mixed", [False, True])
def test_restart_continues_bit_for_bit_on_gpu(tmp_path, mixed):
    """startFrom latestTime on the GPU: written at step 2 and continued, the
    run ends where the uninterrupted one does, bit for bit (FP64 and the
    FP32 store alike: the state is written with 17 digits)."""
    from picfoam_gb300 import foam
    from test_ofcase import make_case as make
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    make(a, injection=False)
    make(b, injection=False)
    extra = ["--mixed"] if mixed else []
    assert run.main([a, "--steps", "4"] + extra) == 0
    assert run.main([b, "--steps", "2"] + extra) == 0
    assert run.main([b, "--restart", "--steps", "2"] + extra) == 0
    la, lb = (os.path.join(p, "4e-12", "lagrangian", "pic") for p in (a, b))
    for name in ("picgpuTet", "picgpuBarycentric", "U", "typeId"):
        np.testing.assert_array_equal(ofcase.read_list(os.path.join(la, name)),
                                      ofcase.read_list(os.path.join(lb, name)))
    np.testing.assert_array_equal(ofcase.read_field(os.path.join(a, "4e-12", "phiE")),
                                  ofcase.read_field(os.path.join(b, "4e-12", "phiE")))
    sa = foam.read(os.path.join(a, "4e-12", "uniform", "picgpuState"))
    sb = foam.read(os.path.join(b, "4e-12", "uniform", "picgpuState"))
    np.testing.assert_array_equal(foam.numeric_list(sa["patchSigma"]), foam.numeric_list(sb["patchSigma"]))
