"""picgpu_initialise against the oracle's picInitialise: every
InitializationModel places the same particles bit for bit in the FP64 store
(the FP32 store holds the oracle's values rounded to float), the statistics
agree, appending keeps the existing particles, the field solve and the
leapfrog back-step match, and a lattice outside the mesh is an error."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import Mesh, PicError

pytestmark = pytest.mark.gpu

E, M_E, M_AR = cases.E_CHARGE, cases.M_E, cases.M_AR


def run_both(gpu, oracle_backend, case, init):
    g = cases.build(case, backend=gpu)
    o = cases.build(case, backend=oracle_backend.OracleBackend(1))
    sg = g.initialise(init)
    so = o.initialise(init)
    return g, o, sg, so


def same_particles(g, o, ns, fp32=False):
    for s in range(ns):
        tg, bg, ug = g.get_particles(s)
        to, bo, uo = o.get_particles(s)
        assert np.array_equal(tg, to), s
        if fp32:
            assert np.array_equal(bg, bo.astype(np.float32).astype(np.float64)), s
            assert np.array_equal(ug, uo.astype(np.float32).astype(np.float64)), s
        else:
            assert np.array_equal(bg, bo), s
            assert np.array_equal(ug, uo), s


def same_stats(sg, so, ns):
    for s in range(ns):
        assert sg.added[s] == so.added[s]
        assert sg.occupancy_min[s] == so.occupancy_min[s] and sg.occupancy_max[s] == so.occupancy_max[s]
        # T = m/(3k) (<U^2> - |drift|^2): sums in another order (device atomics),
        # cancellation when the drift is large (the positive-octant directions)
        assert sg.temperature[s] == pytest.approx(so.temperature[s], rel=1e-6, abs=1e-9)
        assert sg.number_density[s] == pytest.approx(so.number_density[s], rel=1e-12)
    assert sg.debye_length == pytest.approx(so.debye_length, rel=1e-9)


MODELS = {
    "equipartition": dict(model=abi.INIT_EQUIPARTITION, number_density=(2e15, 1e15), temperature=(3.0, 0.1),
                          electron_volt=True, velocity=(1e3, -2e3, 0.0)),
    "maxwellian": dict(model=abi.INIT_MAXWELLIAN, number_density=(2e15, 2e15),
                       thermal_velocity=((1e5, 2e5, 3e5), (300.0, 300.0, 300.0)),
                       drift_velocity=((1e4, 0.0, -1e4), (0.0, 0.0, 50.0))),
    "isotropization": dict(model=abi.INIT_ISOTROPIZATION, number_density=(2e15, 0.0), temperature=(4 / 3, 0.0),
                           electron_volt=True, tperp_over_tpara=0.5),
    "quasineutral": dict(model=abi.INIT_QUASINEUTRAL_PLASMA, temperature=(2.0, 0.05), electron_volt=True,
                         cell_count=1e5, ion_species=1, use_maxwellian=True),
    "quasineutral_speed": dict(model=abi.INIT_QUASINEUTRAL_PLASMA, temperature=(2.0, 0.05), electron_volt=True,
                               cell_count=1e5, ion_species=1, use_maxwellian=False),
}


@pytest.mark.parametrize("name", sorted(MODELS))
@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_models_match_oracle(gpu, oracle_backend, name, precision):
    kw = dict(MODELS[name])
    model = kw.pop("model")
    case = cases.empty_case(n_cells=(6, 5, 7), length=(0.006, 0.005, 0.007), precision=precision,
                            boxes=[((2, 2, 2), (4, 3, 4), cases.patch(abi.PATCH_ABSORB, 1.0))])
    init = cases.init_config(model, seed=77, **kw)
    g, o, sg, so = run_both(gpu, oracle_backend, case, init)
    assert sum(sg.added[s] for s in range(2)) > 1000
    same_particles(g, o, 2, fp32=precision == abi.PREC_MIXED)
    same_stats(sg, so, 2)


def test_uniform_displacement_matches_oracle(gpu, oracle_backend):
    n, L = 64, 0.1
    dx = L / n
    sides = [cases.patch(abi.PATCH_CYCLIC), cases.patch(abi.PATCH_CYCLIC)] + \
            [cases.patch(abi.PATCH_EMPTY) for _ in range(4)]
    case = cases.empty_case(n_cells=(n, 1, 1), length=(L, dx, dx), sides=sides, origin=(0.0, -dx / 2, -dx / 2),
                            species=[(M_E, -E, 1.0, True), (M_AR, E, 1.0, False)])
    init = cases.init_config(abi.INIT_UNIFORM_DISPLACEMENT, temperature=(1e4, 300.0), species=(0, 1),
                             min=(0.5 * dx, -0.25 * dx, -0.25 * dx), max=(L - 0.5 * dx, 0.25 * dx, 0.25 * dx),
                             particle_numbers=(600, 4, 4), cycles=4, displacement=(0.3 * dx, 0.0),
                             displacement_dir=(1.0, 0.0, 0.0))
    g, o, sg, so = run_both(gpu, oracle_backend, case, init)
    assert sg.added[0] == sg.added[1] == 600 * 16
    same_particles(g, o, 2)
    same_stats(sg, so, 2)
    init.max[0] = 2 * L
    with pytest.raises(PicError):
        g.initialise(init)


def test_reduced_dimension_constraint_matches_oracle(gpu, oracle_backend):
    case = cases.plasma_oscillation_1d(Mesh, n_cells=48, per_cell=1)
    case.particles = {}
    init = cases.init_config(abi.INIT_EQUIPARTITION, number_density=(3e17,), temperature=(1.0,), electron_volt=True)
    g, o, sg, so = run_both(gpu, oracle_backend, case, init)
    assert sg.added[0] > 1000
    same_particles(g, o, 1)
    tet, bary, _ = g.get_particles(0)
    assert np.abs(Mesh(case.mesh).position(tet, bary)[:, 1:]).max() < 1e-15


def test_append_keeps_existing_particles(gpu, oracle_backend):
    case = cases.empty_case(n_cells=(4, 4, 4), length=(0.004,) * 3)
    first = cases.init_config(abi.INIT_EQUIPARTITION, seed=1, number_density=(1e15, 1e15), temperature=(1.0, 0.1),
                              electron_volt=True)
    g = cases.build(case, backend=gpu)
    o = cases.build(case, backend=oracle_backend.OracleBackend(1))
    g.initialise(first)
    o.initialise(first)
    n0 = g.count(0)
    more = cases.init_config(abi.INIT_MAXWELLIAN, seed=2, clear=False, number_density=(8e15, 0.0),
                             thermal_velocity=((1e5, 1e5, 1e5), (0, 0, 0)))
    sg = g.initialise(more)
    o.initialise(more)
    assert g.count(0) == n0 + sg.added[0] and sg.added[0] > 4 * n0
    same_particles(g, o, 2)


def test_fields_and_leapfrog_match_oracle(gpu, oracle_backend):
    """Electrode-type box: charge deposit, Poisson solve and the -dt/2 push,
    all bit for bit (FP64 form, fixed-point deposit)."""
    case = cases.empty_case(n_cells=(12, 12, 12), length=(0.012,) * 3,
                            boxes=[((4, 4, 4), (8, 8, 8), cases.patch(abi.PATCH_ABSORB, 20.0))])
    case.cfg.dt = 2e-11
    case.cfg.B[2] = 0.01
    init = cases.init_config(abi.INIT_EQUIPARTITION, seed=5, number_density=(3e14, 2.5e14), temperature=(2.0, 0.03),
                             electron_volt=True, solve_fields=True, leapfrog=True)
    g, o, sg, so = run_both(gpu, oracle_backend, case, init)
    same_particles(g, o, 2)
    assert np.array_equal(g.field(abi.FIELD_PHI), o.field(abi.FIELD_PHI))
    assert np.array_equal(g.field(abi.FIELD_E_CELL), o.field(abi.FIELD_E_CELL))
    # and the run continues identically
    g.step(2)
    o.step(2)
    same_particles(g, o, 2)
