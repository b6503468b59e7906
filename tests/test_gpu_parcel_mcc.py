"""Electron collisions with neutral parcels on the GPU against the oracle:
the ionization tutorial's set-up over several steps -- FP64 form: the same
counters, the same parcels of every species (ionised neutrals deleted, ions
created) in the same cells, velocities and coordinates to the round-off of
the transcendental functions of the relativistic scattering; the FP32 form's
ionisation count close to the oracle's; graph stepping refuses the
neutral-parcel collisions."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import PicError

pytestmark = pytest.mark.gpu


def make(precision=abi.PREC_FP64, n_n=1e22, **kw):
    return cases.neutral_parcel_ionization(n_n=n_n, dt=4e-11, precision=precision, **kw)


@pytest.mark.parametrize("keep", [False, True])
def test_parcel_mcc_matches_oracle(gpu, oracle_backend, keep):
    case = make(keep_neutrals=keep)
    g = cases.build(case, backend=gpu)
    o = cases.build(case, backend=oracle_backend.OracleBackend(1))
    for _ in range(3):
        sg, so = g.step(1), o.step(1)
        assert (sg.mcc_parcel_candidates, sg.mcc_parcel_ionization) == (so.mcc_parcel_candidates, so.mcc_parcel_ionization)
    assert sg.mcc_parcel_ionization > 20
    for s in (0, 1, 2):
        tg, bg, ug = g.get_particles(s)
        to, bo, uo = o.get_particles(s)
        assert len(tg) == len(to)
        np.testing.assert_array_equal(tg, to)
        for a, b in ((ug, uo), (bg, bo)):
            close = np.isclose(a, b, rtol=1e-9, atol=1e-9 * max(np.abs(b).max(), 1e-300)).all(axis=1)
            assert close.mean() > 0.999


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_ion_parcels_after_neutral_deletion_match_oracle(gpu, oracle_backend, precision):
    # electron - parcel ionisation deletes neutrals, then the ion - parcel
    # step draws from the same per-cell lists: its candidate count uses the
    # neutrals left, and no deleted neutral is drawn
    kw = dict(ions_per_cell=20, ion_collisions=(2e-17, 1e-17), n_n=3e22)
    g = cases.build(make(precision=precision, **kw), backend=gpu)
    o = cases.build(make(**kw), backend=oracle_backend.OracleBackend(1))
    deleted = 0
    for _ in range(3):
        sg, so = g.step(1), o.step(1)
        if precision == abi.PREC_FP64:
            assert (sg.mcc_parcel_candidates, sg.ion_parcel_candidates) == \
                   (so.mcc_parcel_candidates, so.ion_parcel_candidates)
            assert (sg.mcc_parcel_ionization, sg.ion_parcel_elastic, sg.ion_parcel_charge_exchange) == \
                   (so.mcc_parcel_ionization, so.ion_parcel_elastic, so.ion_parcel_charge_exchange)
        else:
            # FP32 velocities move the running (sigma c_R)_max and the remainders by rounding
            assert abs(sg.mcc_parcel_candidates - so.mcc_parcel_candidates) <= 0.02 * so.mcc_parcel_candidates + 2
            assert abs(sg.ion_parcel_candidates - so.ion_parcel_candidates) <= 0.02 * so.ion_parcel_candidates + 2
        deleted += so.mcc_parcel_ionization
        assert sg.mcc_candidates == 0 and sg.ion_mcc_candidates == 0    # no background gas
    assert deleted > 100 and so.ion_parcel_elastic + so.ion_parcel_charge_exchange > 50
    if precision != abi.PREC_FP64:
        return
    for s in (0, 1, 2):
        tg, bg, ug = g.get_particles(s)
        to, bo, uo = o.get_particles(s)
        np.testing.assert_array_equal(tg, to)
        close = np.isclose(ug, uo, rtol=1e-9, atol=1e-9 * max(np.abs(uo).max(), 1e-300)).all(axis=1)
        assert close.mean() > 0.999


def test_fp32_form_close_to_oracle(gpu, oracle_backend):
    g = cases.build(make(precision=abi.PREC_MIXED), backend=gpu)
    o = cases.build(make(), backend=oracle_backend.OracleBackend(1))
    ng = sum(g.step(1).mcc_parcel_ionization for _ in range(2))
    no = sum(o.step(1).mcc_parcel_ionization for _ in range(2))
    assert abs(ng - no) <= 4 * np.sqrt(no) and no > 50
    assert g.count(2) == ng and g.count(1) == make().meta["N_n"] - ng


def test_graph_stepping_refuses_parcel_mcc(gpu):
    case = make(precision=abi.PREC_MIXED)
    sim = cases.build(case, backend=gpu)
    with pytest.raises(PicError):
        sim.step_graph(4, 2)
