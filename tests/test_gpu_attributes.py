"""Per-parcel weight and charge state on the GPU against the oracle, through
the C ABI (picgpu_set_parcel_attributes / picgpu_get_parcel_attributes;
PICParcel nParticle_, chargeModifier_, PICParcel.H:182-195).

* FP64 store, fixed-point deposit: parcels with their own nParticle (1 to 3
  species weights) and charge modifiers (0 to 3) move and deposit bit for
  bit like the oracle's, over steps that remove parcels at absorbing walls;
  the attributes follow their parcels; on floating electrodes the patch
  charge sums parcels of unequal charge in arbitrary order (round-off);
* FP32 store: the same set-up agrees with the FP64 oracle to the FP32 form's
  tolerance, including parcels heavier than 64 species weights (their
  fixed-point weights take the 64-bit path);
* bad attributes and counts are refused.
"""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import PicError

pytestmark = pytest.mark.gpu


def attributes(sim, case, seed, heavy=False):
    rng = np.random.default_rng(seed)
    out = {}
    for s in range(case.cfg.n_species):
        n = sim.count(s)
        w = case.cfg.species[s].weight * rng.choice([1.0, 1.5, 2.0, 3.0], n)
        if heavy:
            w[::7] = case.cfg.species[s].weight * 100.0
        z = rng.choice([0, 1, 1, 2, 3], n).astype(np.int32)
        out[s] = (w, z)
    return out


def electrode(precision):
    case = cases.electrode_box(n_cells=16, per_cell=6, precision=precision, dt_factor=0.5, L=0.004)
    case.cfg.deposit_mode = abi.DEPOSIT_FIXED_POINT
    return case


def walls(precision):
    case = cases.two_species_3d(n_cells=8, per_cell=20, precision=precision, deposit=abi.DEPOSIT_FIXED_POINT,
                                dt_factor=0.5, L=0.004, T_e=8.0)
    return case


def pair(case, gpu, oracle_backend, seed, heavy=False, precision=None):
    g = cases.build(case, backend=gpu)
    if precision is not None:
        case.cfg.precision = precision
    o = cases.build(case, backend=oracle_backend.OracleBackend(1))
    for s, (w, z) in attributes(g, case, seed, heavy).items():
        g.set_parcel_attributes(s, w, z)
        o.set_parcel_attributes(s, w, z)
    g.initialise_fields()
    o.initialise_fields()
    return g, o


def test_attributes_fp64_bit_exact(gpu, oracle_backend):
    case = walls(abi.PREC_FP64)
    g, o = pair(case, gpu, oracle_backend, 7)
    np.testing.assert_array_equal(g.field(abi.FIELD_RHO), o.field(abi.FIELD_RHO))
    removed = 0
    for _ in range(3):
        sg, so = g.step(3), o.step(3)
        assert list(sg.n_absorbed) == list(so.n_absorbed)
        removed += sum(sg.n_absorbed)
        for s in range(case.cfg.n_species):
            for a, b in zip(g.get_particles(s), o.get_particles(s)):
                np.testing.assert_array_equal(a, b)
            for a, b in zip(g.get_parcel_attributes(s), o.get_parcel_attributes(s)):
                np.testing.assert_array_equal(a, b)
        for f in (abi.FIELD_RHO, abi.FIELD_PHI, abi.FIELD_E_CELL):
            np.testing.assert_array_equal(g.field(f), o.field(f))
    assert removed > 0
    dg, do = g.diagnostics(), o.diagnostics()
    for s in range(case.cfg.n_species):
        assert dg.weight_sum[s] == pytest.approx(do.weight_sum[s], rel=1e-12)


def test_attributes_floating_electrodes_fp64(gpu, oracle_backend):
    """Parcels of unequal nParticle x charge charge the floating boxes: the
    device adds them with atomics in arbitrary order, so the patch charge,
    and through its boundary condition the potential, agree to round-off;
    the parcels' fate (which ones the boxes and walls remove) is the same."""
    case = electrode(abi.PREC_FP64)
    g, o = pair(case, gpu, oracle_backend, 7)
    np.testing.assert_array_equal(g.field(abi.FIELD_RHO), o.field(abi.FIELD_RHO))
    sg, so = g.step(1), o.step(1)
    assert list(sg.n_absorbed) == list(so.n_absorbed)
    np.testing.assert_allclose(list(sg.floating_charge), list(so.floating_charge), rtol=1e-12, atol=1e-30)
    pg, po = g.field(abi.FIELD_PHI), o.field(abi.FIELD_PHI)
    assert np.abs(pg - po).max() <= 1e-12 * np.abs(po).max()
    for s in range(case.cfg.n_species):
        for a, b in zip(g.get_parcel_attributes(s), o.get_parcel_attributes(s)):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("heavy", [False, True])
def test_attributes_fp32_close(gpu, oracle_backend, heavy):
    case = walls(abi.PREC_MIXED)
    g, o = pair(case, gpu, oracle_backend, 11, heavy, precision=abi.PREC_FP64)
    rg, ro = g.field(abi.FIELD_RHO), o.field(abi.FIELD_RHO)
    # the FP32 store rounds the coordinates; the 2^-25 fixed point the weights
    assert np.abs(rg - ro).max() <= 1e-5 * np.abs(ro).max()
    g.move()
    o.move()
    for s in range(case.cfg.n_species):
        tg, _, ug = g.get_particles(s)
        to, _, uo = o.get_particles(s)
        assert abs(len(tg) - len(to)) <= max(2, len(to) // 1000)
        if len(tg) != len(to):
            continue
        same = tg == to
        assert same.mean() > 0.999
        np.testing.assert_allclose(ug[same], uo[same], rtol=2e-5, atol=2e-5 * np.abs(uo).max())
        wg, zg = g.get_parcel_attributes(s)
        wo, zo = o.get_parcel_attributes(s)
        np.testing.assert_array_equal(wg[same], wo[same])
        np.testing.assert_array_equal(zg[same], zo[same])
    rg, ro = g.field(abi.FIELD_RHO), o.field(abi.FIELD_RHO)
    assert np.abs(rg - ro).max() <= 2e-3 * np.abs(ro).max()


def test_attributes_refused(gpu):
    case = walls(abi.PREC_FP64)
    g = cases.build(case, backend=gpu)
    n = g.count(0)
    w = np.full(n, case.cfg.species[0].weight)
    z = np.ones(n, np.int32)
    with pytest.raises(PicError):
        g.set_parcel_attributes(0, w[:-1], z[:-1])          # not the parcel count
    with pytest.raises(PicError):
        g.set_parcel_attributes(0, -w, z)                    # nParticle <= 0
    with pytest.raises(PicError):
        g.set_parcel_attributes(0, w, np.full(n, 2000, np.int32))  # modifier too large
    # nothing was set: the defaults
    wg, zg = g.get_parcel_attributes(0)
    np.testing.assert_array_equal(wg, case.cfg.species[0].weight)
    np.testing.assert_array_equal(zg, 1)


@pytest.mark.parametrize("wc,collide,cl", [(1, abi.COLLIDE_NANBU, 0.0), (abi.WEIGHT_CORRECTION_SENTOKU_KEMP_NR,
                                                                       abi.COLLIDE_PEREZ, 15.0)])
def test_coulomb_with_parcel_attributes_fp64_matches_oracle(gpu, oracle_backend, wc, collide, cl):
    """NanbuYonemura pairing with per-parcel weights and charges: the pair
    densities sum the parcels' nParticle (NanbuYonemuraPairing.C:96-141,
    198-260), the collide models use the parcels' charges and the weight
    corrections their nParticle (NanbuCorrection.C:63-67,
    SentokuKempNonRelCorrection.C:65-100); the Debye length sums per parcel
    (CoulombCollisionModel.C:270-277)."""
    case = cases.coulomb_relaxation(ragged=True, weight_correction=wc, collide=collide, coulomb_log=cl,
                                    m_i=4.0 * cases.M_E, T_i=1.0)
    g = cases.build(case, backend=gpu)
    o = cases.build(case, backend=oracle_backend.OracleBackend(4))
    for s, (w, z) in attributes(g, case, 5).items():
        z = np.maximum(z, 1)          # charged parcels take part
        g.set_parcel_attributes(s, w, z)
        o.set_parcel_attributes(s, w, z)
    for _ in range(3):
        sg, so = g.step(1), o.step(1)
        assert sg.coulomb_pairs == so.coulomb_pairs > 0
    for s in range(2):
        tg, _, ug = g.get_particles(s)
        to, _, uo = o.get_particles(s)
        np.testing.assert_array_equal(tg, to)
        close = np.isclose(ug, uo, rtol=1e-8, atol=1e-8 * np.abs(uo).max()).all(axis=1)
        assert close.mean() > 0.99
