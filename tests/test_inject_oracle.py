"""SimpleInjection in the oracle (no GPU): frequency / weight * dt parcels per
step with the remainder carried, nothing after injectionEndTime, parcels
placed 10-50 % of the way from the patch towards the first cell centres,
the four velocity models' normal-component distributions, the ejected
charge of a floating patch, emission from a box electrode, and a cyclic
patch rejected."""
import math

import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import Mesh, PicError

E, M_E, M_AR, K_B = cases.E_CHARGE, cases.M_E, cases.M_AR, cases.K_B


def osim(oracle_backend, case):
    return cases.build(case, backend=oracle_backend.OracleBackend(1))


def box_case(n=(8, 8, 8), L=0.008, sides=None, boxes=(), pusher=abi.PUSHER_BORIS, dt=1e-12):
    case = cases.empty_case(n_cells=n, length=(L,) * 3, sides=sides, boxes=boxes,
                            species=[(M_E, -E, 1e4, True), (M_AR, E, 1e4, True)], dt=dt)
    case.cfg.pusher = pusher
    return case


def test_counts_remainder_and_end_time(oracle_backend):
    case = box_case()
    sim = osim(oracle_backend, case)
    # 2.5 electron and 0.3 ion parcels per step
    f_e, f_i = 2.5 * 1e4 / 1e-12, 0.3 * 1e4 / 1e-12
    sim.set_injection([cases.injection(0, (0, 1), (f_e, f_i), (1e-6, 1e-6), model=abi.EMIT_MOST_PROBABLE_SPEED,
                                       end_time=6.5e-12)])
    for k, (ne, ni) in enumerate([(2, 0), (5, 0), (7, 0), (10, 1), (12, 1), (15, 1)]):
        sim.step(1)
        assert (sim.count(0), sim.count(1)) == (ne, ni), k
    sim.step(2)                     # t = 7, 8 dt > injectionEndTime
    assert (sim.count(0), sim.count(1)) == (15, 1)


def test_positions_between_face_and_centre_plane(oracle_backend):
    n, L = 8, 0.008
    dx = L / n
    case = box_case(pusher=abi.PUSHER_NONE)
    sim = osim(oracle_backend, case)
    # near-zero speed: after one step the parcels sit where they were emitted
    sim.set_injection([cases.injection(1, (0,), (4000 * 1e4 / 1e-12,), (1e-8,), model=abi.EMIT_MOST_PROBABLE_SPEED)])
    sim.step(1)
    tet, bary, U = sim.get_particles(0)
    assert len(tet) == 4000
    xyz = Mesh(case.mesh).position(tet, bary)
    d = L - xyz[:, 0]                           # patch 1 is the +x side
    assert d.min() >= 0.1 * dx / 2 * (1 - 1e-9) and d.max() <= 0.5 * dx / 2 * (1 + 1e-9)
    assert abs(d.mean() / (0.3 * dx / 2) - 1) < 0.02
    cells = tet // 12
    assert np.all(cells % n == n - 1)          # owner cells of the +x faces
    # uniform over the face: each of the 64 faces gets about 4000 / 64
    hist = np.bincount(cells // n, minlength=n * n)
    assert hist.min() > 30 and hist.max() < 100
    assert np.all(U[:, 0] < 0) and np.allclose(U[:, 1:], 0.0)   # inward normal is -x


@pytest.mark.parametrize("model,mean_over_vt", [
    (abi.EMIT_MAXWELLIAN_FLUX, math.sqrt(math.pi / 2)),
    (abi.EMIT_BIRD_MAXWELLIAN_FLUX, math.sqrt(math.pi / 2)),
    (abi.EMIT_HALF_MAXWELLIAN_FLUX, math.sqrt(2 / math.pi)),
    (abi.EMIT_MOST_PROBABLE_SPEED, math.sqrt(2.0)),
])
def test_velocity_models(oracle_backend, model, mean_over_vt):
    case = box_case(n=(4, 4, 4), L=0.04)
    sim = osim(oracle_backend, case)
    T = 2.0
    sim.set_injection([cases.injection(2, (0,), (20000 * 1e4 / 1e-12,), (T,), model=model)])
    sim.step(1)
    _, _, U = sim.get_particles(0)
    vt = math.sqrt(T * E / M_E)
    un = U[:, 1]                                # patch 2 is -y: inward normal +y
    assert np.all(un > 0)
    assert abs(un.mean() / (mean_over_vt * vt) - 1) < 0.02
    if model == abi.EMIT_MOST_PROBABLE_SPEED:
        assert np.allclose(un, math.sqrt(2.0) * vt, rtol=1e-12) and np.allclose(U[:, [0, 2]], 0.0)
    else:
        assert abs(U[:, 0].std() / vt - 1) < 0.03 and abs(U[:, 2].std() / vt - 1) < 0.03
        assert abs(U[:, 0].mean()) < 0.03 * vt


def test_floating_patch_takes_the_ejected_charge(oracle_backend):
    sides = [cases.patch(abi.PATCH_FLOATING)] + [cases.patch(abi.PATCH_ABSORB, 0.0) for _ in range(5)]
    case = box_case(sides=sides)
    sim = osim(oracle_backend, case)
    sim.set_injection([cases.injection(0, (0,), (7 * 1e4 / 1e-12,), (1.0,))])
    st = sim.step(1)
    # seven electrons left the patch: +7 e w (nothing came back within a step)
    assert st.floating_charge[0] == pytest.approx(7 * E * 1e4, rel=1e-12)


def test_box_electrode_emits_into_adjacent_cells(oracle_backend):
    n = 8
    box = ((3, 3, 3), (5, 5, 5), cases.patch(abi.PATCH_ABSORB, 0.0))
    case = box_case(boxes=[box], pusher=abi.PUSHER_NONE)
    sim = osim(oracle_backend, case)
    sim.set_injection([cases.injection(6, (0,), (3000 * 1e4 / 1e-12,), (1e-8,))])
    sim.step(1)
    tet, _, U = sim.get_particles(0)
    assert len(tet) == 3000
    m = Mesh(case.mesh)
    cc, _ = m.cells()
    c = cc[tet // 12]
    lo, hi = 3 * 0.001, 5 * 0.001
    inside = np.all((c > lo - 0.001) & (c < hi + 0.001), axis=1)
    assert np.all(inside)                      # the shell of cells around the box
    # the owner cells touch one box face: the velocity component along that
    # face's outward normal (the emitter's inward normal) is positive
    below, above = c < lo, c > hi
    assert np.all(below.sum(axis=1) + above.sum(axis=1) == 1)
    un = (U * above).sum(axis=1) - (U * below).sum(axis=1)
    assert np.all(un > 0)


def test_rejects_cyclic_patch(oracle_backend):
    sides = [cases.patch(abi.PATCH_CYCLIC), cases.patch(abi.PATCH_CYCLIC)] + \
            [cases.patch(abi.PATCH_ABSORB, 0.0) for _ in range(4)]
    sim = osim(oracle_backend, box_case(sides=sides))
    with pytest.raises(PicError):
        sim.set_injection([cases.injection(0, (0,), (1e16,), (1.0,))])
