"""Circuit boundary models in the oracle (no GPU): circuitRLC with the
RLCBoundary potential (the backward-difference circuit equation step by step,
the cathode face value, R-C charging of the gap), IdealCurrentSource (the
surface charge it feeds, J and refArea scaling, the area-weighted voltage),
IdealVoltageSource (running-average currents from the emitted charge),
electrodes absorbing charged and reflecting neutral parcels, and the
constructor checks."""
import math

import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import PicError

E, M_E, M_AR = cases.E_CHARGE, cases.M_E, cases.M_AR
EPS0 = 1.0 / (4e-7 * math.pi * 299792458.0 ** 2)


def osim(oracle_backend, case):
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    sim.initialise_fields()
    return sim


def rlc_coefficients(R, L, C, dt):
    return (2.25 * L / dt / dt + 1.5 * R / dt + 1.0 / C, -6.0 * L / dt / dt - 2.0 * R / dt,
            5.5 * L / dt / dt + 0.5 * R / dt, -2.0 * L / dt / dt, 0.25 * L / dt / dt)


@pytest.mark.parametrize("R,L,omega", [(1.0, 0.04, 0.0), (50.0, 1e-3, 2e9)])
def test_rlc_backward_difference_equation(oracle_backend, R, L, omega):
    dt, V, C = 1e-11, 100.0, 1e-6
    case = cases.circuit_case(n=32, R=R, L=L, C=C, V=V, omega=omega, dt=dt)
    sim = osim(oracle_backend, case)
    a = rlc_coefficients(R, L, C, dt)
    Q = [0.0] * 4
    for k in range(12):
        st = sim.step(1)
        t = (k + 1) * dt
        src = V * math.sin(omega * t + math.pi / 2)
        lhs = a[0] * st.circuit_charge + a[1] * Q[0] + a[2] * Q[1] + a[3] * Q[2] + a[4] * Q[3]
        assert lhs == pytest.approx(src - st.circuit_voltage, rel=1e-9, abs=1e-9 * V)
        assert st.circuit_current == pytest.approx((st.circuit_charge - Q[0]) / dt, rel=1e-12)
        Q = [st.circuit_charge] + Q[:3]
    # the reported voltage is the RLCBoundary face value (1 - coeff1 d) phi_P
    phi = sim.field(abi.FIELD_PHI)
    d = 0.5 * 0.05 / 32
    k_rlc = a[0] * EPS0 * 0.024 ** 2
    assert st.circuit_voltage == pytest.approx((1.0 - d / (k_rlc + d)) * phi[0], rel=1e-12)


def test_rc_charging_of_the_vacuum_gap(oracle_backend):
    # L = 0: the gap (C_gap = eps0 A / gap) charges through R with
    # tau = R C_gap C / (C_gap + C) towards V C / (C_gap + C)
    R, C, V, dt, n, length, width = 1e3, 1e-6, 100.0, 1e-11, 50, 0.05, 0.024
    case = cases.circuit_case(n=n, R=R, L=0.0, C=C, V=V, dt=dt, length=length, width=width)
    sim = osim(oracle_backend, case)
    c_gap = EPS0 * width ** 2 / length
    c_ser = c_gap * C / (c_gap + C)
    tau = R * c_ser
    volts = [sim.step(1).circuit_voltage for _ in range(200)]
    assert np.all(np.diff(volts) > 0)
    # exponential approach once the second-order start-up has passed
    rate = math.log((V - volts[39]) / (V - volts[79])) / (40 * dt)
    assert rate == pytest.approx(1.0 / tau, rel=0.03)
    st = sim.step(1)
    assert st.circuit_voltage == pytest.approx(V * C / (c_gap + C), rel=1e-3)
    assert st.circuit_charge == pytest.approx(c_ser * V, rel=0.03)
    phi = sim.field(abi.FIELD_PHI)
    assert np.all(np.diff(phi) < 0)                  # linear fall towards the 0 V anode
    assert np.allclose(np.diff(phi), np.diff(phi).mean(), rtol=1e-6)


@pytest.mark.parametrize("I,J,ref_area", [(2e-3, -1.0, 0.0), (2e-3, -1.0, 1e-4), (-1.0, 5.0, 0.0)])
def test_ideal_current_source_surface_charge(oracle_backend, I, J, ref_area):
    dt, width = 1e-11, 0.024
    A = width * width
    sigma0 = 1e-9
    case = cases.circuit_case(model=abi.CIRCUIT_IDEAL_CURRENT, n=16, I=I, J=J, ref_area=ref_area, sigma=sigma0,
                              dt=dt, width=width)
    sim = osim(oracle_backend, case)
    I_eff = J * A if J > 0 else (I * A / ref_area if ref_area > 0 else I)
    sigma = sigma0
    for k in range(6):
        st = sim.step(1)
        sigma = sigma + (0.0 - I_eff * dt) / A
        assert st.circuit_charge == pytest.approx(sigma * A, rel=1e-12)
    phi = sim.field(abi.FIELD_PHI)
    assert st.circuit_voltage == pytest.approx(phi[0], rel=1e-12)   # one face: |S| phi_P / |S|
    # the cathode's circuitBoundary gradient sigma / eps0 (outward normal -x)
    # sets the field in the gap
    assert (phi[0] - phi[1]) / (0.05 / 16) == pytest.approx(sigma / EPS0, rel=1e-9)


def test_ideal_voltage_source_running_average_currents(oracle_backend):
    dt, w = 1e-11, 1e6
    case = cases.circuit_case(model=abi.CIRCUIT_IDEAL_VOLTAGE, n=16, dt=dt, weight=w, cathode_phi=-10.0)
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    per_step = 3
    sim.set_injection([cases.injection(0, (0,), (per_step * w / dt,), (1e-6,), model=abi.EMIT_HALF_MAXWELLIAN_FLUX)])
    sim.initialise_fields()
    qc = [0.0, 0.0, 0.0]
    avg = 0.0
    for k in range(5):
        st = sim.step(1)
        assert st.n_absorbed[0] == 0
        acc = per_step * E * w            # particleEjection takes q w off the cathode's accumulator
        qc = [qc[0] - acc, qc[0], qc[1]]
        beta = dt / ((k + 1) * dt)
        avg = (1 - beta) * avg + beta * ((2.0 * (qc[0] - qc[1]) + 0.5 * (qc[2] - qc[0])) / dt)
        assert st.circuit_cathode_current == pytest.approx(avg, rel=1e-12)
        assert st.circuit_current == 0.0
    assert sim.count(0) == 15


def test_electrodes_absorb_charged_and_reflect_neutral_parcels(oracle_backend):
    case = cases.circuit_case(model=abi.CIRCUIT_RLC, n=8, length=0.008, dt=1e-9)
    cfg = case.cfg
    cfg.species[1].charge = 0.0                          # second species neutral
    rng = np.random.Generator(np.random.Philox(5))
    tet, bary = cases.uniform_in_cells(rng, np.arange(8), 20)
    U = np.zeros((len(tet), 3))
    U[:, 0] = rng.choice([-1.0, 1.0], len(tet)) * 2e6   # every parcel crosses a cell per step
    case.particles = {0: (tet, bary, U.copy()), 1: (tet, bary, U * 1e-1)}
    sim = osim(oracle_backend, case)
    absorbed = 0
    for _ in range(6):
        st = sim.step(1)
        absorbed += st.n_absorbed[0]
    assert absorbed > 0 and sim.count(0) == 160 - absorbed
    assert sim.count(1) == 160                         # neutral parcels bounce off both electrodes
    _, _, Un = sim.get_particles(1)
    assert np.allclose(np.abs(Un[:, 0]), 2e5)


def test_circuit_checks(oracle_backend):
    def create(case):
        return cases.build(case, backend=oracle_backend.OracleBackend(1))

    bad = cases.circuit_case(model=abi.CIRCUIT_RLC)
    bad.mesh.side[0].phi_bc = abi.PHI_FIXED_VALUE               # RLC needs the RLCBoundary cathode
    with pytest.raises(PicError):
        create(bad)
    bad = cases.circuit_case(model=abi.CIRCUIT_IDEAL_CURRENT)
    bad.cfg.circuit.I = bad.cfg.circuit.J = -1.0                   # neither I nor J
    with pytest.raises(PicError):
        create(bad)
    bad = cases.circuit_case(model=abi.CIRCUIT_RLC)
    bad.cfg.circuit.model = abi.CIRCUIT_NONE                      # circuit patches without a model
    with pytest.raises(PicError):
        create(bad)
    bad = cases.circuit_case(model=abi.CIRCUIT_RLC)
    bad.mesh.side[1].phi_bc = abi.PHI_ZERO_GRADIENT               # anode must be fixedValue
    with pytest.raises(PicError):
        create(bad)
    bad = cases.empty_case()
    bad.mesh.side[0].phi_bc = abi.PHI_RLC                         # RLCBoundary off a circuit electrode
    with pytest.raises(PicError):
        create(bad)
