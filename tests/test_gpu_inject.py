"""SimpleInjection on the GPU against the oracle: several PIC steps with
emission from side and box patches, every velocity model, a floating
injector, the half-step velocity sync in the self-consistent field -- FP64
form bit for bit (particles and potential); the FP32 form to its rounding."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import PicError

pytestmark = pytest.mark.gpu

E, M_E, M_AR = cases.E_CHARGE, cases.M_E, cases.M_AR


def make(precision=abi.PREC_FP64, floating=False, box=False):
    sides = [cases.patch(abi.PATCH_FLOATING if floating else abi.PATCH_ABSORB, 0.0)] + \
            [cases.patch(abi.PATCH_ABSORB, 0.0), cases.patch(abi.PATCH_WALL, 0.0, abi.PHI_ZERO_GRADIENT),
             cases.patch(abi.PATCH_WALL, 0.0, abi.PHI_ZERO_GRADIENT), cases.patch(abi.PATCH_ABSORB, 5.0),
             cases.patch(abi.PATCH_ABSORB, 0.0)]
    boxes = [((3, 3, 3), (5, 5, 5), cases.patch(abi.PATCH_ABSORB, -2.0))] if box else []
    case = cases.empty_case(n_cells=(8, 8, 8), length=(0.008,) * 3, sides=sides, boxes=boxes,
                            species=[(M_E, -E, 2e3, True), (M_AR, E, 2e3, True)], precision=precision,
                            dt=2e-12)
    case.cfg.B[1] = 0.02
    return case


def run(backend, case, injectors, steps):
    sim = cases.build(case, backend=backend)
    sim.set_injection(injectors)
    sim.initialise_fields()
    for _ in range(steps):
        sim.step(1)
    return sim


def particles(sim, s):
    return sim.get_particles(s)


@pytest.mark.parametrize("model", [abi.EMIT_MAXWELLIAN_FLUX, abi.EMIT_BIRD_MAXWELLIAN_FLUX,
                                   abi.EMIT_HALF_MAXWELLIAN_FLUX, abi.EMIT_MOST_PROBABLE_SPEED])
def test_injection_steps_match_oracle(gpu, oracle_backend, model):
    case = make(box=True)
    # 30 + 10 parcels per step from the -x side, 20 from the box
    inj = [cases.injection(0, (0, 1), (3e16, 1e16), (3.0, 0.5), model=model),
           cases.injection(6, (0,), (2e16,), (1.0,), model=model)]
    g = run(gpu, case, inj, 4)
    o = run(oracle_backend.OracleBackend(1), case, inj, 4)
    for s in (0, 1):
        tg, bg, ug = particles(g, s)
        to, bo, uo = particles(o, s)
        assert len(tg) > 30
        assert np.array_equal(tg, to) and np.array_equal(bg, bo) and np.array_equal(ug, uo)
    assert np.array_equal(g.field(abi.FIELD_PHI), o.field(abi.FIELD_PHI))


def test_floating_injector_matches_oracle(gpu, oracle_backend):
    case = make(floating=True)
    inj = [cases.injection(0, (0,), (5e16,), (2.0,))]
    g = cases.build(case, backend=gpu)
    o = cases.build(case, backend=oracle_backend.OracleBackend(1))
    for sim in (g, o):
        sim.set_injection(inj)
        sim.initialise_fields()
    for _ in range(3):
        sg, so = g.step(1), o.step(1)
        assert sg.floating_charge[0] == so.floating_charge[0]
    assert sg.floating_charge[0] > 0
    assert np.array_equal(particles(g, 0)[2], particles(o, 0)[2])
    assert np.array_equal(g.field(abi.FIELD_PHI), o.field(abi.FIELD_PHI))


def test_fp32_form_close_to_oracle(gpu, oracle_backend):
    inj = [cases.injection(0, (0, 1), (3e16, 1e16), (3.0, 0.5))]
    g = run(gpu, make(precision=abi.PREC_MIXED), inj, 2)
    o = run(oracle_backend.OracleBackend(1), make(), inj, 2)
    for s in (0, 1):
        tg, bg, ug = particles(g, s)
        to, bo, uo = particles(o, s)
        assert len(tg) == len(to) > 15
        assert np.mean(tg == to) > 0.99
        same = tg == to
        assert np.abs(ug[same] - uo[same]).max() <= 1e-4 * np.abs(uo).max()


def test_graph_stepping_refuses_injection(gpu):
    case = make()
    case.cfg.maxwell_solver = abi.MAXWELL_NONE
    case.cfg.precision = abi.PREC_MIXED
    sim = cases.build(case, backend=gpu)
    sim.set_injection([cases.injection(0, (0,), (1e15,), (1.0,))])
    with pytest.raises(PicError):
        sim.step_graph(4, 2)
