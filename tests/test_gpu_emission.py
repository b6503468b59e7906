"""EmissionModels on the GPU against the oracle: thermionic and
Fowler-Nordheim emission from the cathode of a 30 kV gap, several PIC steps
-- FP64 form bit for bit (particles, potential); the FP32 form to within a
parcel or two."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases

pytestmark = pytest.mark.gpu

E, M_E, M_AR = cases.E_CHARGE, cases.M_E, cases.M_AR


def make(precision=abi.PREC_FP64):
    sides = [cases.patch(abi.PATCH_ABSORB, -3.0e4), cases.patch(abi.PATCH_ABSORB, 0.0)] + \
            [cases.patch(abi.PATCH_WALL, 0.0, abi.PHI_ZERO_GRADIENT)] * 2 + [cases.patch(abi.PATCH_EMPTY)] * 2
    return cases.empty_case(n_cells=(16, 4, 1), length=(1e-5, 1e-5, 1e-5), sides=sides, dt=1e-14,
                            precision=precision, species=[(M_E, -E, 1.0, True), (M_AR, E, 1.0, True)])


MODELS = [cases.emission(0, abi.EMISSION_FOWLER_NORDHEIM, 4.5),
          cases.emission(0, abi.EMISSION_THERMIONIC, 2.5, temperature=2200.0, lambda_r=0.5)]


def run(backend, case, steps):
    sim = cases.build(case, backend=backend)
    sim.set_emission(MODELS)
    sim.initialise_fields()
    stats = [sim.step(1) for _ in range(steps)]
    return sim, stats


def test_emission_steps_match_oracle(gpu, oracle_backend):
    g, sg = run(gpu, make(), 4)
    o, so = run(oracle_backend.OracleBackend(1), make(), 4)
    for a, b in zip(sg, so):
        assert list(a.n_absorbed) == list(b.n_absorbed)
    tg, bg, ug = g.get_particles(0)
    to, bo, uo = o.get_particles(0)
    assert len(tg) > 50
    assert np.array_equal(tg, to) and np.array_equal(bg, bo) and np.array_equal(ug, uo)
    assert np.array_equal(g.field(abi.FIELD_PHI), o.field(abi.FIELD_PHI))


def test_fp32_form_close_to_oracle(gpu, oracle_backend):
    g, _ = run(gpu, make(precision=abi.PREC_MIXED), 2)
    o, _ = run(oracle_backend.OracleBackend(1), make(), 2)
    assert abs(g.count(0) - o.count(0)) <= 2
    assert g.count(0) > 20
