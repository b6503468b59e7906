"""Per-parcel weight and charge state in the oracle (PICParcel nParticle_ and
chargeModifier_, PICParcel.H:182-195): known answers without a GPU.

* nParticle scales a parcel's charge deposit (VolumeWeighting.C:114): twice
  the weight of every parcel gives exactly twice the charge density;
* the charge modifier scales the parcel's charge (PICCloud.C:368), so the
  push and the deposit: modifier 2 on the ions doubles their charge and
  their velocity change in the field; modifier 0 leaves a parcel unpushed
  (PICParcel.C:55) and uncharged;
* the attributes follow their parcels through steps that remove parcels,
  and the diagnostics sum the parcels' own weights.
"""
import numpy as np

from picfoam_gb300 import abi, cases


def build(ob, **kw):
    case = cases.two_species_3d(n_cells=6, per_cell=10, precision=abi.PREC_FP64, L=0.003, **kw)
    return case, cases.build(case, backend=ob.OracleBackend(1))


def test_defaults_without_attributes(oracle_backend):
    case, sim = build(oracle_backend)
    for s in range(2):
        w, z = sim.get_parcel_attributes(s)
        assert len(w) == sim.count(s)
        np.testing.assert_array_equal(w, case.cfg.species[s].weight)
        np.testing.assert_array_equal(z, 1)


def test_double_weight_doubles_charge_density(oracle_backend):
    rho = []
    for factor in (1.0, 2.0):
        case, sim = build(oracle_backend)
        for s in range(2):
            n = sim.count(s)
            sim.set_parcel_attributes(s, np.full(n, factor * case.cfg.species[s].weight), np.ones(n, np.int32))
        sim.initialise_fields()
        rho.append(sim.field(abi.FIELD_RHO))
    assert np.abs(rho[0]).max() > 0
    np.testing.assert_array_equal(rho[1], 2.0 * rho[0])


def test_charge_modifier_scales_charge_and_push(oracle_backend):
    out = []
    for z in (1, 2, 0):
        case, sim = build(oracle_backend, Bz=0.0)
        n = sim.count(1)
        sim.set_parcel_attributes(1, np.full(n, case.cfg.species[1].weight), np.full(n, z, np.int32))
        sim.set_particles(0, np.zeros(0, np.int32), np.zeros((0, 3)), np.zeros((0, 3)))
        sim.initialise_fields()
        rho = sim.field(abi.FIELD_RHO)
        _, _, U0 = sim.get_particles(1)
        sim.set_field(abi.FIELD_E_CELL, np.tile([1e4, 0.0, 0.0], sim.sizes()[0]))
        E_pt = np.tile([1e4, 0.0, 0.0], sim.field(abi.FIELD_E_POINT).shape[0])
        sim.set_field(abi.FIELD_E_POINT, E_pt)
        sim.move()
        _, _, U1 = sim.get_particles(1)
        out.append((rho, U1 - U0))
    np.testing.assert_allclose(out[1][0], 2.0 * out[0][0], rtol=1e-14, atol=0)
    np.testing.assert_array_equal(out[2][0], 0.0)
    dv1, dv2, dv0 = out[0][1][:, 0], out[1][1][:, 0], out[2][1][:, 0]
    assert np.all(dv1 > 0)
    np.testing.assert_allclose(dv2, 2.0 * dv1, rtol=1e-9)
    np.testing.assert_array_equal(dv0, 0.0)


def test_attributes_follow_their_parcels(oracle_backend):
    case, sim = build(oracle_backend, T_e=50.0)
    n = sim.count(0)
    w0 = case.cfg.species[0].weight * (1.0 + np.arange(n) / n)
    z0 = (np.arange(n) % 3 + 1).astype(np.int32)
    sim.set_parcel_attributes(0, w0, z0)
    sim.initialise_fields()
    d = sim.diagnostics()
    assert abs(d.weight_sum[0] - np.sum(w0)) < 1e-12 * np.sum(w0)
    sim.step(3)
    w1, z1 = sim.get_parcel_attributes(0)
    assert 0 < len(w1) < n          # hot electrons leave through the absorbing walls
    # the survivors keep their attributes in their order
    idx = np.searchsorted(w0, w1)
    np.testing.assert_array_equal(w0[idx], w1)
    np.testing.assert_array_equal(z0[idx], z1)
    assert np.all(np.diff(idx) > 0)
