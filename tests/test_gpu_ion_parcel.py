"""Ion collisions with neutral parcels on the GPU against the oracle: the
same candidate and event counts, the same parcels, velocities to the
round-off of the scattering's transcendental functions; equal weights, and
unequal weights under each WeightCorrection model."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ratio,model", [
    (1.0, abi.WEIGHT_CORRECTION_NONE),
    (2.0, abi.WEIGHT_CORRECTION_NANBU),
    (3.0, abi.WEIGHT_CORRECTION_SENTOKU_KEMP_NR),
    (0.5, abi.WEIGHT_CORRECTION_SENTOKU_KEMP),
])
def test_ion_parcel_collisions_match_oracle(gpu, oracle_backend, ratio, model):
    case = cases.ion_neutral_parcels(ion_weight_ratio=ratio, weight_correction=model)
    g = cases.build(case, backend=gpu)
    o = cases.build(case, backend=oracle_backend.OracleBackend(1))
    for _ in range(3):
        sg, so = g.step(1), o.step(1)
        assert (sg.ion_parcel_candidates, sg.ion_parcel_elastic, sg.ion_parcel_charge_exchange) == \
               (so.ion_parcel_candidates, so.ion_parcel_elastic, so.ion_parcel_charge_exchange)
    assert sg.ion_parcel_elastic + sg.ion_parcel_charge_exchange > 50
    for s in (0, 1):
        tg, bg, ug = g.get_particles(s)
        to, bo, uo = o.get_particles(s)
        np.testing.assert_array_equal(tg, to)
        close = np.isclose(ug, uo, rtol=1e-9, atol=1e-9 * np.abs(uo).max()).all(axis=1)
        assert close.mean() > 0.999
