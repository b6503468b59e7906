"""Circuit boundary models on the GPU against the oracle: circuitRLC (with an
AC source), IdealCurrentSource and IdealVoltageSource with a plasma in the
gap and electrons emitted from the cathode -- particles, potential and the
circuit's voltage, current and charge bit for bit in the FP64 form, to
rounding in the FP32 form; graph stepping refuses circuits."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import PicError

pytestmark = pytest.mark.gpu


def make(model, precision=abi.PREC_FP64):
    kw = dict(n=24, length=0.012, width=0.004, per_cell=12, T_e=10.0, weight=2e5, dt=1e-10, precision=precision)
    if model == abi.CIRCUIT_RLC:
        return cases.circuit_case(model=model, R=20.0, L=1e-9, C=1e-12, V=50.0, omega=3e9, **kw)
    if model == abi.CIRCUIT_IDEAL_CURRENT:
        return cases.circuit_case(model=model, I=5e-3, sigma=2e-9, **kw)
    return cases.circuit_case(model=model, cathode_phi=-20.0, anode_phi=5.0, **kw)


def run(backend, case, steps, emit=True):
    sim = cases.build(case, backend=backend)
    if emit:
        sim.set_injection([cases.injection(0, (0,), (2e16,), (2.0,))])
    sim.initialise_fields()
    stats = [sim.step(1) for _ in range(steps)]
    return sim, stats


@pytest.mark.parametrize("model", [abi.CIRCUIT_RLC, abi.CIRCUIT_IDEAL_CURRENT, abi.CIRCUIT_IDEAL_VOLTAGE])
def test_circuit_steps_match_oracle(gpu, oracle_backend, model):
    case = make(model)
    g, sg = run(gpu, case, 6)
    o, so = run(oracle_backend.OracleBackend(1), case, 6)
    for a, b in zip(sg, so):
        for f in ("circuit_voltage", "circuit_current", "circuit_cathode_current", "circuit_charge"):
            assert getattr(a, f) == getattr(b, f), f
        assert list(a.n_absorbed) == list(b.n_absorbed)
    assert sum(s.n_absorbed[0] + s.n_absorbed[1] for s in sg) > 0
    for s in (0, 1):
        tg, bg, ug = g.get_particles(s)
        to, bo, uo = o.get_particles(s)
        assert np.array_equal(tg, to) and np.array_equal(bg, bo) and np.array_equal(ug, uo)
    assert np.array_equal(g.field(abi.FIELD_PHI), o.field(abi.FIELD_PHI))
    assert np.array_equal(g.field(abi.FIELD_E_CELL), o.field(abi.FIELD_E_CELL))


def test_rlc_multigrid_matches_jacobi(gpu):
    case = make(abi.CIRCUIT_RLC)
    case.particles = {}
    case.cfg.pcg_tol = 1e-12
    _, sj = run(gpu, case, 4, emit=False)
    case.cfg.pcg_precond = abi.PRECOND_MULTIGRID
    _, sm = run(gpu, case, 4, emit=False)
    for a, b in zip(sj, sm):
        assert a.circuit_voltage == pytest.approx(b.circuit_voltage, rel=1e-9)
        assert a.circuit_charge == pytest.approx(b.circuit_charge, rel=1e-9)


def test_fp32_form_close_to_oracle(gpu, oracle_backend):
    g, sg = run(gpu, make(abi.CIRCUIT_RLC, precision=abi.PREC_MIXED), 3)
    o, so = run(oracle_backend.OracleBackend(1), make(abi.CIRCUIT_RLC), 3)
    for a, b in zip(sg, so):
        assert a.circuit_voltage == pytest.approx(b.circuit_voltage, rel=1e-5, abs=1e-6)
        assert a.circuit_charge == pytest.approx(b.circuit_charge, rel=1e-5)


def test_graph_stepping_refuses_circuits(gpu):
    case = make(abi.CIRCUIT_IDEAL_VOLTAGE, precision=abi.PREC_MIXED)
    case.cfg.maxwell_solver = abi.MAXWELL_NONE
    sim = cases.build(case, backend=gpu)
    with pytest.raises(PicError):
        sim.step_graph(4, 2)
