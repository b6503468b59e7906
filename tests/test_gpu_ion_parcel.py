"""Ion collisions with neutral parcels on the GPU against the oracle: the
same candidate and event counts, the same parcels, velocities to the
round-off of the scattering's transcendental functions."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases

pytestmark = pytest.mark.gpu


def test_ion_parcel_collisions_match_oracle(gpu, oracle_backend):
    case = cases.ion_neutral_parcels()
    g = cases.build(case, backend=gpu)
    o = cases.build(case, backend=oracle_backend.OracleBackend(1))
    for _ in range(3):
        sg, so = g.step(1), o.step(1)
        assert (sg.ion_mcc_candidates, sg.ion_mcc_elastic, sg.ion_mcc_charge_exchange) == \
               (so.ion_mcc_candidates, so.ion_mcc_elastic, so.ion_mcc_charge_exchange)
    assert sg.ion_mcc_elastic + sg.ion_mcc_charge_exchange > 50
    for s in (0, 1):
        tg, bg, ug = g.get_particles(s)
        to, bo, uo = o.get_particles(s)
        np.testing.assert_array_equal(tg, to)
        close = np.isclose(ug, uo, rtol=1e-9, atol=1e-9 * np.abs(uo).max()).all(axis=1)
        assert close.mean() > 0.999
