"""PairMerging in the oracle (PairMerging::mergeParticles,
PICMCCFVM/submodels/ParticleMerging/PairMerging/PairMerging.C:71-259):
known answers without a GPU.

* a merge keeps the real particles (nParticle summed) and the momentum
  (weighted mean velocity), loses kinetic energy (the reported error is the
  after - before difference, <= 0), and keeps the charge;
* cells above cellParcelsMax shrink towards reductionFactor of their count
  (at most mergeMaximumPerCell merges), the others are left alone;
* the merged parcel sits in its partners' cell with charge modifier 1;
* settings picFoam refuses are refused.
"""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import Mesh, PicError


def still(case):
    """No field and no movement: the step does nothing but merge."""
    case.cfg.maxwell_solver = abi.MAXWELL_NONE
    for s in range(case.cfg.n_species):
        case.cfg.species[s].solve_movement = 0


def totals(sim, case):
    out = []
    for s in range(case.cfg.n_species):
        tet, bary, U = sim.get_particles(s)
        w, z = sim.get_parcel_attributes(s)
        out.append((w.sum(), (w[:, None] * U).sum(axis=0), 0.5 * case.cfg.species[s].mass * (w * (U * U).sum(1)).sum(),
                    (w * z).sum(), len(w)))
    return out


def test_merging_conserves_weight_and_momentum(oracle_backend):
    case = cases.merging_plasma()
    still(case)                      # the step changes nothing but the merges
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    before = totals(sim, case)
    st = sim.step(1)
    after = totals(sim, case)
    assert st.merged_parcels > 0 and st.merge_checks >= st.merged_parcels
    dE = 0.0
    for (w0, p0, e0, q0, n0), (w1, p1, e1, q1, n1) in zip(before, after):
        assert w1 == pytest.approx(w0, rel=1e-13)
        np.testing.assert_allclose(p1, p0, rtol=1e-9, atol=1e-12 * np.abs(p0).max() + 1e-300)
        assert q1 == pytest.approx(q0, rel=1e-13)
        assert e1 <= e0 * (1 + 1e-13)
        dE += e1 - e0
    assert st.merge_kinetic_energy_error < 0
    assert st.merge_kinetic_energy_error == pytest.approx(dE, rel=1e-6)
    assert sum(b[4] - a[4] for b, a in zip(before, after)) == st.merged_parcels


def test_merging_reduces_crowded_cells_only(oracle_backend):
    case = cases.merging_plasma(cell_parcels_max=30, reduction_factor=0.8, merge_maximum_per_cell=3)
    still(case)
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    counts0 = [np.bincount(sim.get_particles(s)[0] // 12, minlength=64) for s in range(2)]
    sim.step(1)
    counts1 = [np.bincount(sim.get_particles(s)[0] // 12, minlength=64) for s in range(2)]
    for c0, c1 in zip(counts0, counts1):
        quiet = c0 <= 30
        np.testing.assert_array_equal(c1[quiet], c0[quiet])
        crowded = ~quiet
        assert crowded.any()
        merges = c0[crowded] - c1[crowded]
        assert np.all(merges >= 0) and np.all(merges <= 3)          # mergeMaximumPerCell
        assert merges.sum() > 0


def test_merged_parcels_stay_in_their_cell(oracle_backend):
    case = cases.merging_plasma()
    still(case)
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    n0 = [sim.count(s) for s in range(2)]
    cells0 = [set(np.unique(sim.get_particles(s)[0] // 12)) for s in range(2)]
    m = Mesh(case.mesh)
    sim.step(1)
    for s in range(2):
        tet, bary, U = sim.get_particles(s)
        w, z = sim.get_parcel_attributes(s)
        new = w > case.cfg.species[s].weight * 1.5          # merged parcels carry at least two weights
        assert new.any()
        assert np.all(z == 1)
        assert set(np.unique(tet[new] // 12)) <= cells0[s]
        # inside the tet: barycentric coordinates within [0, 1]
        y0 = 1.0 - bary.sum(axis=1)
        assert np.all(bary >= 0) and np.all(y0 >= -1e-12)
        assert len(tet) < n0[s]
        assert np.all(np.isfinite(m.position(tet, bary)))


def test_bad_merging_settings_refused(oracle_backend):
    case = cases.merging_plasma(cell_parcels_max=4, reduction_factor=0.5, n_check_neighbors=4)
    with pytest.raises(PicError):
        cases.build(case, backend=oracle_backend.OracleBackend(1))
