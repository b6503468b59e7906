"""FreeStream on the GPU against the oracle: PIC steps with a drifting stream
from a side patch and a box patch (both species, both rejection scalings)
-- FP64 form bit for bit (particles and potential), the FP32 form to its
rounding; graph stepping refuses FreeStream."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import PicError

pytestmark = pytest.mark.gpu

E, M_E, M_AR, K_B = cases.E_CHARGE, cases.M_E, cases.M_AR, cases.K_B


def make(precision=abi.PREC_FP64):
    box = ((3, 3, 3), (5, 5, 5), cases.patch(abi.PATCH_ABSORB, -3.0))
    case = cases.empty_case(n_cells=(8, 8, 8), length=(0.008,) * 3, boxes=[box], precision=precision, dt=2e-12,
                            species=[(M_E, -E, 1e3, True), (M_AR, E, 1e3, True)])
    case.cfg.B[2] = 0.05
    return case


MODELS = [cases.freestream(0, (0, 1), (4e15, 4e15), 3.0 * E / K_B, velocity=(3e5, 1e5, 0.0)),
          cases.freestream(6, (0,), (2e16,), 2.0 * E / K_B, velocity=(0.0, 0.0, -3e6))]


def run(backend, case, steps):
    sim = cases.build(case, backend=backend)
    sim.set_freestream(MODELS)
    sim.initialise_fields()
    for _ in range(steps):
        sim.step(1)
    return sim


def test_freestream_steps_match_oracle(gpu, oracle_backend):
    g = run(gpu, make(), 5)
    o = run(oracle_backend.OracleBackend(1), make(), 5)
    for s in (0, 1):
        tg, bg, ug = g.get_particles(s)
        to, bo, uo = o.get_particles(s)
        assert len(tg) > 50
        assert np.array_equal(tg, to) and np.array_equal(bg, bo) and np.array_equal(ug, uo)
    assert np.array_equal(g.field(abi.FIELD_PHI), o.field(abi.FIELD_PHI))


def test_fp32_form_close_to_oracle(gpu, oracle_backend):
    g = run(gpu, make(precision=abi.PREC_MIXED), 2)
    o = run(oracle_backend.OracleBackend(1), make(), 2)
    for s in (0, 1):
        tg, _, ug = g.get_particles(s)
        to, _, uo = o.get_particles(s)
        assert len(tg) == len(to) > 20
        same = tg == to
        assert same.mean() > 0.99
        assert np.abs(ug[same] - uo[same]).max() <= 1e-4 * np.abs(uo).max()


def test_graph_stepping_refuses_freestream(gpu):
    case = make(precision=abi.PREC_MIXED)
    case.cfg.maxwell_solver = abi.MAXWELL_NONE
    sim = cases.build(case, backend=gpu)
    sim.set_freestream(MODELS[:1])
    with pytest.raises(PicError):
        sim.step_graph(4, 2)
