"""The multigrid-preconditioned PCG (pcg_precond = MULTIGRID): on the same
charge density it reaches the same tolerance as the Jacobi PCG -- whose
solves match the oracle bit for bit -- with far fewer iterations, on meshes
with Dirichlet walls and box electrodes, fully periodic (singular) meshes,
odd cell counts and reduced dimensions; its solves are bit-reproducible."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import Mesh, PicError

pytestmark = pytest.mark.gpu

TOL = 1e-10


def with_precond(case, precond, **mg):
    case.cfg.pcg_precond = precond
    case.cfg.pcg_tol = TOL
    case.cfg.pcg_max_iter = 20000
    for k, v in mg.items():
        setattr(case.cfg.mg, k, v)
    return case


def rho_field(n, seed):
    rng = np.random.default_rng(seed)
    return 1e-7 * (rng.standard_normal(n) + 0.5)


def solve_both(gpu, make, seed=3, **mg):
    sj = cases.build(with_precond(make(), abi.PRECOND_JACOBI), backend=gpu)
    sm = cases.build(with_precond(make(), abi.PRECOND_MULTIGRID, **mg), backend=gpu)
    n = sj.sizes()[0]
    rho = rho_field(n, seed)
    pj, stj = sj.solve_poisson(rho)
    pm, stm = sm.solve_poisson(rho)
    sj.close()
    sm.close()
    return pj, stj, pm, stm


def close_potentials(pj, pm, singular=False):
    if singular:  # defined up to a constant
        pj = pj - pj.mean()
        pm = pm - pm.mean()
    scale = np.abs(pj).max()
    assert scale > 0
    return np.abs(pj - pm).max() / scale


def electrode(n=32):
    return lambda: cases.electrode_box(n_cells=n, per_cell=1, seed=2)


def periodic_cube(n=(24, 24, 24)):
    def make():
        sides = [cases.patch(abi.PATCH_CYCLIC) for _ in range(6)]
        mesh = cases.block_mesh(n, (0.01, 0.01, 0.01), sides)
        cfg = cases.base_config(1e-12, [(cases.M_E, -cases.E_CHARGE, 1.0, True)])
        return cases.Case("periodic", mesh, cfg, {}, [], {})
    return make


def odd_mixed(n=(27, 18, 11)):
    def make():
        sides = [cases.patch(abi.PATCH_CYCLIC), cases.patch(abi.PATCH_CYCLIC),
                 cases.patch(abi.PATCH_ABSORB, 0.0), cases.patch(abi.PATCH_ABSORB, 5.0),
                 cases.patch(abi.PATCH_WALL, 0.0, abi.PHI_ZERO_GRADIENT),
                 cases.patch(abi.PATCH_WALL, 0.0, abi.PHI_ZERO_GRADIENT)]
        box = ((5, 4, 3), (9, 7, 6), cases.patch(abi.PATCH_ABSORB, -3.0))
        mesh = cases.block_mesh(n, (0.027, 0.018, 0.011), sides, boxes=[box])
        cfg = cases.base_config(1e-12, [(cases.M_E, -cases.E_CHARGE, 1.0, True)])
        return cases.Case("odd", mesh, cfg, {}, [], {})
    return make


def line_1d(n=2048):
    def make():
        return cases.plasma_oscillation_1d(Mesh, n_cells=n, per_cell=1)
    return make


def test_electrode_box_same_potential_fewer_iterations(gpu):
    pj, stj, pm, stm = solve_both(gpu, electrode(32))
    assert stm.pcg_residual_l2 <= TOL and stj.pcg_residual_l2 <= TOL
    assert close_potentials(pj, pm) < 1e-7
    assert stm.pcg_iterations * 4 <= stj.pcg_iterations, (stm.pcg_iterations, stj.pcg_iterations)


def test_periodic_singular(gpu):
    pj, stj, pm, stm = solve_both(gpu, periodic_cube())
    assert stm.pcg_residual_l2 <= TOL
    assert close_potentials(pj, pm, singular=True) < 1e-7
    assert stm.pcg_iterations < stj.pcg_iterations


def test_odd_counts_box_and_mixed_walls(gpu):
    pj, stj, pm, stm = solve_both(gpu, odd_mixed())
    assert stm.pcg_residual_l2 <= TOL
    assert close_potentials(pj, pm) < 1e-7
    assert stm.pcg_iterations < stj.pcg_iterations


def test_reduced_dimension(gpu):
    pj, stj, pm, stm = solve_both(gpu, line_1d())
    assert stm.pcg_residual_l2 <= TOL
    assert close_potentials(pj, pm, singular=True) < 1e-7


@pytest.mark.parametrize("mg", [dict(pre_sweeps=1, post_sweeps=1), dict(coarsest_cells=64),
                                dict(scale_correction=1.0, omega=0.6), dict(pre_sweeps=3, post_sweeps=0)])
def test_settings(gpu, mg):
    pj, stj, pm, stm = solve_both(gpu, electrode(24), **mg)
    assert stm.pcg_residual_l2 <= TOL
    assert close_potentials(pj, pm) < 1e-7


def test_bit_reproducible_and_warm_started(gpu):
    sim = cases.build(with_precond(electrode(32)(), abi.PRECOND_MULTIGRID), backend=gpu)
    rho = rho_field(sim.sizes()[0], 9)
    p1, s1 = sim.solve_poisson(rho)
    p2, s2 = sim.solve_poisson(rho)
    assert np.array_equal(p1, p2) and s1.pcg_iterations == s2.pcg_iterations
    # from the converged potential nothing is left to do
    p3, s3 = sim.solve_poisson(rho, phi0=p1)
    assert s3.pcg_iterations <= 3
    sim.close()


def test_steps_with_multigrid_match_jacobi(gpu):
    """A few PIC steps of the electrode box: the particle histories agree to
    the solve tolerance whichever preconditioner solves the potential."""
    runs = []
    for pre in (abi.PRECOND_JACOBI, abi.PRECOND_MULTIGRID):
        case = cases.electrode_box(n_cells=24, per_cell=4, seed=8)
        case.cfg.pcg_precond = pre
        sim = cases.build(case, backend=gpu)
        st = sim.step(3)
        runs.append((sim.field(abi.FIELD_PHI), st.pcg_iterations))
        sim.close()
    (pj, ij), (pm, im) = runs
    assert np.abs(pj - pm).max() <= 1e-5 * np.abs(pj).max()
    assert im < ij


def test_rejects_bad_settings(gpu):
    with pytest.raises(PicError):
        cases.build(with_precond(electrode(16)(), abi.PRECOND_MULTIGRID, pre_sweeps=9), backend=gpu)
    case = electrode(16)()
    case.cfg.pcg_precond = 7
    with pytest.raises(PicError):
        cases.build(case, backend=gpu)
