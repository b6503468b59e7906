"""EmissionModels in the oracle (no GPU): thermionic emission's
Richardson-Dushman count per step with the remainder carried and its
maxwellianFlux velocities, the emitted charge taken off a floating cathode,
Fowler-Nordheim emission from the summed face current of a strong outward
field (none for an inward field), the case loader reading a circuit's
EmissionModels, and the checks."""
import math
import os

import numpy as np
import pytest

from picfoam_gb300 import abi, cases, ofcase
from picfoam_gb300.simulation import PicError

E, M_E, M_AR, K_B = cases.E_CHARGE, cases.M_E, cases.M_AR, cases.K_B
A0 = 1201732.101


def gap(n=8, length=1e-5, width=1e-5, cathode=None, anode_phi=0.0, dt=1e-14, w=1.0):
    cathode = cathode or cases.patch(abi.PATCH_ABSORB, 0.0)
    sides = [cathode, cases.patch(abi.PATCH_ABSORB, anode_phi)] + [cases.patch(abi.PATCH_EMPTY)] * 4
    case = cases.empty_case(n_cells=(n, 1, 1), length=(length, width, width), sides=sides, dt=dt,
                            species=[(M_E, -E, w, True), (M_AR, E, w, True)])
    return case


def osim(oracle_backend, case, models):
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    sim.set_emission(models)
    sim.initialise_fields()
    return sim


def test_thermionic_counts_and_velocities(oracle_backend):
    T, W, lam, dt, w = 2500.0, 2.0, 0.5, 1e-14, 1.0
    case = gap(dt=dt, w=w)
    case.cfg.pusher = abi.PUSHER_NONE
    case.cfg.maxwell_solver = abi.MAXWELL_NONE
    sim = osim(oracle_backend, case, [cases.emission(0, abi.EMISSION_THERMIONIC, W, temperature=T, lambda_r=lam)])
    j = lam * A0 * T * T * math.exp(-(W * E / (T * K_B)))
    A = 1e-10
    rem, total = 0.0, 0
    for _ in range(5):
        sim.step(1)
        ne = j * A * dt / (w * E) + rem
        n = int(ne)
        rem = ne - n
        total += n
        assert sim.count(0) + 0 == total
    assert total > 1000
    _, _, U = sim.get_particles(0)
    vt = math.sqrt(K_B * T / M_E)
    assert np.all(U[:, 0] > 0)
    assert U[:, 0].mean() == pytest.approx(math.sqrt(math.pi / 2) * vt, rel=0.03)


def test_floating_cathode_loses_the_emitted_charge(oracle_backend):
    case = gap(cathode=cases.patch(abi.PATCH_FLOATING))
    sim = osim(oracle_backend, case, [cases.emission(0, abi.EMISSION_THERMIONIC, 2.0, temperature=2500.0)])
    st = sim.step(1)
    n = sim.count(0)
    assert n > 0
    # particleEjection: -q w per electron, so the patch gains + n e w
    assert st.floating_charge[0] == pytest.approx(n * E, rel=1e-12)


def fowler_nordheim(Emag, W):
    y = 3.7947e-5 * math.sqrt(Emag) / W
    v = 0.956 - 1.062 * y * y
    return 1.541434e-6 * Emag * Emag / W * math.exp(-6.830889776e9 * v * W ** 1.5 / Emag)


@pytest.mark.parametrize("ny", [1, 3])
def test_fowler_nordheim_from_the_summed_face_current(oracle_backend, ny):
    W, dt, w, V, L = 4.5, 1e-12, 1.0, -3.0e4, 1e-5
    n = 8
    sides = [cases.patch(abi.PATCH_ABSORB, V), cases.patch(abi.PATCH_ABSORB, 0.0)] + \
            [cases.patch(abi.PATCH_WALL, 0.0, abi.PHI_ZERO_GRADIENT)] * 2 + [cases.patch(abi.PATCH_EMPTY)] * 2
    case = cases.empty_case(n_cells=(n, ny, 1), length=(L, 1e-5, 1e-5), sides=sides, dt=dt,
                            species=[(M_E, -E, w, True), (M_AR, E, w, True)])
    case.cfg.pusher = abi.PUSHER_NONE
    sim = osim(oracle_backend, case, [cases.emission(0, abi.EMISSION_FOWLER_NORDHEIM, W)])
    Emag = abs(V) / L             # cathode at -30 kV: E points into the cathode (outward normal -x)
    j = ny * fowler_nordheim(Emag, W)   # the reference sums the face current densities
    expect = j * 1e-10 * dt / (w * E)
    st = sim.step(1)
    assert sim.count(0) + st.n_absorbed[0] == pytest.approx(expect, abs=1.0)
    assert sim.count(0) > 10
    # reversed field: nothing leaves the cathode
    sides[0] = cases.patch(abi.PATCH_ABSORB, -V)
    case2 = cases.empty_case(n_cells=(n, ny, 1), length=(L, 1e-5, 1e-5), sides=sides, dt=dt,
                             species=[(M_E, -E, w, True), (M_AR, E, w, True)])
    sim2 = osim(oracle_backend, case2, [cases.emission(0, abi.EMISSION_FOWLER_NORDHEIM, W)])
    sim2.step(2)
    assert sim2.count(0) == 0


def test_emission_checks(oracle_backend):
    case = gap()
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    with pytest.raises(PicError):
        sim.set_emission([cases.emission(0, abi.EMISSION_THERMIONIC, 2.0, temperature=2500.0, weight=5.0)])
    with pytest.raises(PicError):
        sim.set_emission([cases.emission(2, abi.EMISSION_THERMIONIC, 2.0, temperature=2500.0)])   # empty patch
    with pytest.raises(PicError):
        sim.set_emission([cases.emission(0, abi.EMISSION_THERMIONIC, 2.0, temperature=0.0)])
    sim.set_emission([cases.emission(0, abi.EMISSION_FOWLER_NORDHEIM, 4.5, weight=1.0)])


def test_case_loader_reads_emission_models(tmp_path):
    from test_ofcase import make_case
    make_case(str(tmp_path))
    pp = os.path.join(str(tmp_path), "constant", "picProperties")
    text = open(pp).read().replace(
        "collector { type FloatingPotential; }",
        "\"source|collector\" { type IdealVoltageSource; IdealVoltageSourceCoeffs {"
        " EmissionModels (Thermionic FowlerNordheim);"
        " ThermionicCoeffs { lambdaR 0.5; T 2000; fnW 2.5; } FowlerNordheimCoeffs { fnW 4.5; }"
        " source { type cathode; } collector { type anode; } } }").replace(
        "source { type SimpleInjection;", "unused { type SimpleInjection;")
    open(pp, "w").write(text)
    phi = os.path.join(str(tmp_path), "0", "phiE")
    open(phi, "w").write(open(phi).read().replace("collector { type circuitBoundary; value uniform 0; }",
                                                  "collector { type fixedValue; value uniform 0; }"))
    with pytest.raises(ofcase.UnsupportedCase):
        ofcase.load_case(str(tmp_path))                      # "unused" is not a patch
    open(pp, "w").write(text.replace("unused { type SimpleInjection;", "sides { type SimpleInjection;"))
    c = ofcase.load_case(str(tmp_path))
    assert c.cfg.circuit.model == abi.CIRCUIT_IDEAL_VOLTAGE
    th, fn = c.emissions
    assert th.model == abi.EMISSION_THERMIONIC and th.temperature == 2000 and th.work_function == 2.5
    assert fn.model == abi.EMISSION_FOWLER_NORDHEIM and fn.patch == 0 and fn.work_function == 4.5
