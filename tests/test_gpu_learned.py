"""The learned Poisson warm start inside picgpu_step: after its training
solves the net's start is closer to the solution than the previous
potential, and the FP64 PCG still converges to the same tolerance and the
same potential."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases

pytestmark = pytest.mark.gpu

PCG_TOL = 1e-8  # electrode_box's pcg_tol


def run(gpu, learned, steps, train_steps=40):
    case = cases.electrode_box(n_cells=32, per_cell=20, seed=5)
    if learned:
        case.cfg.learned.enabled = 1
        case.cfg.learned.train_steps = train_steps
        case.cfg.learned.train_iters = 8
        case.cfg.learned.refine = 1
        case.cfg.learned.lr = 2e-3
    sim = cases.build(case, backend=gpu)
    stats = [sim.step(1) for _ in range(steps)]
    return sim, stats


def test_learned_warm_start_beats_previous_potential(gpu):
    steps, T = 50, 40
    plain, sp = run(gpu, False, steps)
    learned, sl = run(gpu, True, steps, T)
    # training phase: plain starts, samples collected, loss reported; a
    # solve that starts far from its solution (the first) is not a pair
    first = next(k for k, s in enumerate(sl) if s.learned_active)
    assert T <= first <= T + 2
    assert all(s.learned_active == 0 for s in sl[:first])
    assert sl[first - 1].learned_samples > 0 and 0 < sl[first - 1].learned_loss < 1.0
    after = sl[first:]
    assert all(s.learned_active == 1 for s in after)
    # the net's start residual is clearly below the previous potential's
    # (0.3-0.65 of it over the measured runs: an online training outcome)
    for s in after:
        assert s.pcg_residual_initial < 0.75 * s.learned_residual
        assert s.pcg_residual_l2 <= PCG_TOL and s.pcg_iterations > 0
    # no more iterations than the plain start on average
    assert np.mean([s.pcg_iterations for s in after]) <= np.mean([s.pcg_iterations for s in sp[first:]]) + 1
    # same physics: the particle histories are identical up to the solve
    # tolerance, so the potentials agree to well within the field scale
    phi_p, phi_l = plain.field(abi.FIELD_PHI), learned.field(abi.FIELD_PHI)
    assert np.abs(phi_p - phi_l).max() <= 1e-3 * np.abs(phi_p).max()


def test_learned_needs_supported_grid(gpu):
    from picfoam_gb300.simulation import PicError
    case = cases.electrode_box(n_cells=24, per_cell=2)
    case.cfg.learned.enabled = 1
    with pytest.raises(PicError):
        cases.build(case, backend=gpu)
