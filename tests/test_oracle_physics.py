"""Known-answer tests of the CPU oracle (pinning the restatement without
reference outputs): gyration radius, E x B drift, plasma frequency, energy
conservation, Poisson manufactured solution, wall and patch behaviour."""
import math

import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import Mesh


def oracle(case, ob, nthreads=1, precond=0):
    return cases.build(case, backend=ob.OracleBackend(nthreads, precond))


@pytest.mark.parametrize("pusher", [abi.PUSHER_BORIS, abi.PUSHER_VAY, abi.PUSHER_HIGUERA_CARY])
def test_gyration_radius_and_period(oracle_backend, pusher):
    case = cases.magnetic_rotation(Mesh, pusher=pusher, steps_per_orbit=400)
    r = case.meta["radius"]
    sim = oracle(case, oracle_backend)
    m = Mesh(case.mesh)
    pts = []
    for _ in range(400):
        sim.step(1)
        tet, bary, U = sim.get_particles(0)
        assert len(tet) == 1
        pts.append(m.position(tet, bary)[0])
        # the relativistic pushers keep |u| (and |v|) in a pure B field
        assert abs(np.linalg.norm(U[0]) - case.meta["v"]) < 1e-9 * case.meta["v"]
    pts = np.array(pts)
    centre = pts[:, :2].mean(axis=0)
    radius = np.linalg.norm(pts[:, :2] - centre, axis=1)
    assert abs(radius.mean() - r) < 0.01 * r
    assert radius.std() < 0.01 * r
    # back near the start after one period
    assert np.linalg.norm(pts[-1, :2] - pts[0, :2]) < 0.05 * r
    assert np.all(np.abs(pts[:, 2]) < 1e-12)  # stays on the mesh-centre plane


def test_e_cross_b_drift(oracle_backend):
    B = 1.0
    E = (2e5, 0.0, 0.0)
    case = cases.magnetic_rotation(Mesh, pusher=abi.PUSHER_BORIS, beta=0.01, B=B, E=E, steps_per_orbit=100)
    sim = oracle(case, oracle_backend)
    m = Mesh(case.mesh)
    n_orbits = 4
    pts = []
    for _ in range(100 * n_orbits):
        sim.step(1)
        tet, bary, _ = sim.get_particles(0)
        pts.append(m.position(tet, bary)[0])
    pts = np.array(pts)
    T = 100 * case.meta["dt"]
    # drift over whole orbits: v_d = E x B / B^2 = (0, -E_x/B, 0) for B along z
    drift = (pts[-1] - pts[99]) / ((n_orbits - 1) * T)
    vd = -E[0] / B
    assert abs(drift[1] - vd) < 0.02 * abs(vd)
    assert abs(drift[0]) < 0.02 * abs(vd)


def test_cold_plasma_oscillation_frequency(oracle_backend):
    case = cases.plasma_oscillation_1d(Mesh, n_cells=64, per_cell=20, T_eV=1e-6, quiet=True,
                                       perturbation=1e3, dt_factor=0.05)
    sim = oracle(case, oracle_backend)
    sim.initialise_fields()
    fe = []
    for _ in range(400):
        sim.step(1)
        fe.append(sim.diagnostics().field_energy)
    fe = np.array(fe)
    # field energy oscillates at 2 omega_pe
    peaks = [i for i in range(1, len(fe) - 1) if fe[i] > fe[i - 1] and fe[i] >= fe[i + 1]]
    assert len(peaks) >= 4
    period_steps = (peaks[-1] - peaks[0]) / (len(peaks) - 1)
    w = 2 * math.pi / (2 * period_steps * case.meta["dt"])
    assert abs(w / case.meta["wpe"] - 1.0) < 0.02


def test_energy_conservation_1d(oracle_backend):
    # 128 cells (dx ~ lambda_D) at 200/cell: total energy stays within 1e-3
    # over 200 steps (2.3 plasma periods)
    case = cases.plasma_oscillation_1d(Mesh, n_cells=128, per_cell=200)
    sim = oracle(case, oracle_backend)
    sim.initialise_fields()
    tot = []
    for _ in range(200):
        sim.step(1)
        d = sim.diagnostics()
        tot.append(d.kinetic_energy[0] + d.field_energy)
    tot = np.array(tot)
    assert np.abs(tot / tot[0] - 1).max() < 1e-3


def test_poisson_manufactured_solution(oracle_backend):
    # phi = sin(pi x/L) sin(pi y/L) sin(pi z/L) in a grounded cube:
    # rho = 3 (pi/L)^2 eps0 phi; second-order convergence of the FV solution
    errs = []
    for n in (8, 16):
        L = 1.0
        case = cases.two_species_3d(n_cells=n, per_cell=1, L=L, precision=abi.PREC_FP64, pcg_tol=1e-12)
        sim = oracle(case, oracle_backend)
        cc, _ = Mesh(case.mesh).cells()
        k = math.pi / L
        exact = np.sin(k * cc[:, 0]) * np.sin(k * cc[:, 1]) * np.sin(k * cc[:, 2])
        rho = 3 * k * k * cases.EPS0 * exact
        phi, st = sim.solve_poisson(rho)
        assert st.pcg_residual_l2 <= 1e-12
        errs.append(np.abs(phi - exact).max())
    assert errs[1] < errs[0] / 3.0


def test_dic_and_jacobi_agree(oracle_backend):
    case = cases.electrode_box(n_cells=16, per_cell=1, precision=abi.PREC_FP64, pcg_tol=1e-12)
    rng = np.random.default_rng(0)
    sj = oracle(case, oracle_backend, precond=0)
    sd = oracle(case, oracle_backend, precond=1)
    rho = rng.standard_normal(sj.sizes()[0]) * 1e-6
    pj, stj = sj.solve_poisson(rho)
    pd, std = sd.solve_poisson(rho)
    np.testing.assert_allclose(pj, pd, rtol=0, atol=1e-9 * np.abs(pj).max())
    assert std.pcg_iterations < stj.pcg_iterations


def test_absorbing_walls_remove_particles(oracle_backend):
    case = cases.two_species_3d(n_cells=4, per_cell=20, L=0.002, precision=abi.PREC_FP64, dt_factor=1.0)
    sim = oracle(case, oracle_backend)
    sim.initialise_fields()
    n0 = sim.count(0)
    st = sim.step(5)
    assert st.n_absorbed[0] > 0
    assert sim.count(0) == n0 - st.n_absorbed[0]


def test_specular_wall_keeps_particles_and_speed(oracle_backend):
    case = cases.two_species_3d(n_cells=4, per_cell=20, L=0.002, precision=abi.PREC_FP64, dt_factor=1.0)
    for s in range(6):
        case.mesh.side[s].kind = abi.PATCH_WALL
    case.cfg.species[0].charge = 0.0  # neutral: no field, speed must be kept exactly
    case.cfg.species[1].charge = 0.0
    case.cfg.maxwell_solver = abi.MAXWELL_NONE
    sim = oracle(case, oracle_backend)
    _, _, U0 = sim.get_particles(0)
    st = sim.step(20)
    assert st.wall_hits > 0 and st.n_absorbed[0] == 0
    _, _, U1 = sim.get_particles(0)
    np.testing.assert_allclose(np.linalg.norm(U1, axis=1), np.linalg.norm(U0, axis=1), rtol=1e-12)


def test_floating_electrode_collects_charge(oracle_backend):
    case = cases.electrode_box(n_cells=16, per_cell=4, precision=abi.PREC_FP64, dt_factor=1.0, L=0.004)
    sim = oracle(case, oracle_backend)
    sim.initialise_fields()
    st = sim.step(6)
    # electrons are faster than ions: the floating boxes charge negatively
    q = np.array(st.floating_charge)
    assert q[6] < 0 and q[7] < 0


def test_threads_give_identical_results(oracle_backend):
    case = cases.two_species_3d(n_cells=6, per_cell=10, L=0.003, precision=abi.PREC_FP64,
                                deposit=abi.DEPOSIT_FIXED_POINT, dt_factor=0.5)
    a = oracle(case, oracle_backend, nthreads=1)
    b = oracle(case, oracle_backend, nthreads=4)
    for s in (a, b):
        s.initialise_fields()
        s.step(3)
    for sp in (0, 1):
        for x, y in zip(a.get_particles(sp), b.get_particles(sp)):
            np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(a.field(abi.FIELD_PHI), b.field(abi.FIELD_PHI))


def test_cell_magnetic_field_acts_per_cell(oracle_backend):
    """PICGPU_FIELD_B_CELL in the oracle: a per-cell field equal everywhere to
    the uniform B reproduces the uniform run bit for bit; the gyration then
    follows the cell values (a field of twice the strength halves the radius)."""
    runs = []
    for mode in ("uniform", "per_cell", "double"):
        case = cases.magnetic_rotation(Mesh, pusher=abi.PUSHER_BORIS, steps_per_orbit=200)
        if mode != "uniform":
            case.cfg.B[2] = 0.0
        sim = oracle(case, oracle_backend)
        n = sim.sizes()[0]
        if mode != "uniform":
            sim.set_field(abi.FIELD_B_CELL, np.tile([0.0, 0.0, 1.0 if mode == "per_cell" else 2.0], n))
        m = Mesh(case.mesh)
        pts = []
        for _ in range(100):
            sim.step(1)
            tet, bary, U = sim.get_particles(0)
            pts.append(m.position(tet, bary)[0])
        runs.append((np.array(pts), U))
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])
    d_single = np.ptp(runs[0][0][:, 1])          # half an orbit: the diameter along y
    d_double = np.ptp(runs[2][0][:, 1])          # a whole orbit at half the radius
    assert abs(d_double / d_single - 0.5) < 0.02
