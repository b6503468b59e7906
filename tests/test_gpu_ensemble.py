"""Batched ensembles stepped by CUDA graphs.

The collision random streams are keyed by (cell, step) and every kernel of
a step is per particle, per cell or an integer sum, so a graph-stepped run
reproduces the regular step exactly, and case 0 of an ensemble (whose cells
keep their single-case numbers) reproduces the same case run alone.
"""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import EnsembleBackend

pytestmark = pytest.mark.gpu


def small_ensemble(n_cases, counts, EN_Td, seed=3):
    return cases.swarm_ensemble(n_cases=n_cases, n=(8, 8, 32), size=(0.005, 0.005, 0.02), counts=counts,
                                EN_Td=EN_Td, T_e=4.0, seed=seed)


def particle_set(sim, species):
    tet, bary, U = sim.get_particles(species)
    keys = np.concatenate([tet[:, None].astype(np.float64), bary, U], axis=1)
    order = np.lexsort(keys.T[::-1])
    return keys[order]


def case_rows(keys, k, cells_per_case):
    cell = keys[:, 0].astype(np.int64) // 12
    return keys[(cell // cells_per_case) == k]


def test_graph_step_reproduces_regular_step(gpu):
    case = small_ensemble(1, [20000], [3e3])
    # Re-sorting renumbers particles: two that later meet in one cell can
    # swap their order in its list, and MCC picks by list position.  The two
    # paths re-sort at different times, so exact equality needs no re-sort.
    case.cfg.sort_interval = 0
    # regular context: the same case with a uniform applied field
    case.cfg.E_applied[2] = case.meta["E"][0, 2]
    reg = cases.build(case)
    st_r = abi.StepStats()
    for _ in range(20):
        s = reg.step(1)
        st_r.mcc_candidates += s.mcc_candidates
        st_r.mcc_ionization += s.mcc_ionization
        st_r.mcc_elastic += s.mcc_elastic
    ens = cases.build_ensemble(case)
    st_g = ens.step_graph(20, 5)
    assert st_g.mcc_candidates == st_r.mcc_candidates > 0
    assert st_g.mcc_elastic == st_r.mcc_elastic
    assert st_g.mcc_ionization == st_r.mcc_ionization
    for s in range(2):
        assert ens.count(s) == reg.count(s)
        np.testing.assert_array_equal(particle_set(ens, s), particle_set(reg, s))
    bps, blk, _ = ens.graph_tuning()
    assert bps in (3, 4, 5, 6, 8) and blk in (64, 128, 256)


def test_ensemble_case_zero_matches_single_case(gpu):
    single = small_ensemble(1, [15000], [3e3])
    pair = small_ensemble(2, [15000, 30000], [3e3, 3e2])
    # case 0 of the pair starts with exactly the particles of the single run
    tet1, b1, u1 = single.particles[0]
    tet2, b2, u2 = pair.particles[0]
    cpc = pair.meta["cells_per_case"]
    sel = tet2 // 12 < cpc
    tet2, b2, u2 = tet2[sel], b2[sel], u2[sel]
    pair.particles[0] = (np.concatenate([tet1, pair.particles[0][0][~sel]]),
                         np.concatenate([b1, pair.particles[0][1][~sel]]),
                         np.concatenate([u1, pair.particles[0][2][~sel]]))
    a = cases.build_ensemble(single)
    b = cases.build_ensemble(pair)
    a.step_graph(10, 5)
    b.step_graph(10, 5)
    for s in range(2):
        ka = particle_set(a, s)
        kb = case_rows(particle_set(b, s), 0, cpc)
        np.testing.assert_array_equal(ka, kb)


def test_ensemble_per_case_statistics(gpu):
    EN = [30.0, 300.0, 3000.0]
    case = small_ensemble(3, [8000, 16000, 12000], EN)
    sim = cases.build_ensemble(case)
    st = sim.step_graph(30, 5)
    out, iz = sim.case_stats(0, 3)
    assert int(out[:, 0].sum()) == sim.count(0) == st.n_particles[0]
    assert int(iz.sum()) == st.mcc_ionization
    # the drift along z is opposite to E and grows with E/N
    vz = out[:, 3] / out[:, 0]
    assert np.all(vz < 0)
    assert -vz[0] < -vz[1] < -vz[2]
