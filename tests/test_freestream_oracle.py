"""FreeStream in the oracle (no GPU): the per-face accumulators against Bird's
eq. 4.22 flux (with and without drift, remainders carried), parcels placed on
the patch faces uniformly, the normal-speed and tangential distributions of a
drifting Maxwellian flux (eq. 12.5 acceptance-rejection, both scalings), a
box electrode emitting through all its faces, and the checks."""
import math

import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import Mesh, PicError

E, M_E, M_AR, K_B = cases.E_CHARGE, cases.M_E, cases.M_AR, cases.K_B


def osim(oracle_backend, case, models):
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    sim.set_freestream(models)
    return sim


def box_case(n=8, L=0.008, boxes=(), dt=1e-12, weight=1e4):
    case = cases.empty_case(n_cells=(n,) * 3, length=(L,) * 3, boxes=boxes, dt=dt,
                            species=[(M_E, -E, weight, True), (M_AR, E, weight, True)])
    case.cfg.pusher = abi.PUSHER_NONE
    case.cfg.maxwell_solver = abi.MAXWELL_NONE
    return case


def flux_per_area(n, T, m, un):
    """Bird eq. 4.22: n c_mp (e^{-s^2} + sqrt(pi) s (1 + erf s)) / (2 sqrt(pi))."""
    c = math.sqrt(2 * K_B * T / m)
    s = un / c
    return n * c * (math.exp(-s * s) + math.sqrt(math.pi) * s * (1 + math.erf(s))) / (2 * math.sqrt(math.pi))


def mean_normal_speed(T, m, un):
    """Flux-weighted mean normal speed of a drifting Maxwellian, by quadrature,
    over the interval eq. 12.5's rejection samples: thermal part within
    +-3 c_mp (+-(|s| + 1) c_mp when s < -3)."""
    vt = math.sqrt(K_B * T / m)
    c = math.sqrt(2.0) * vt
    s = un / c
    top = c * (s + (abs(s) + 1 if s < -3 else 3.0))
    v = np.linspace(0, top, 400001)
    f = v * np.exp(-(v - un) ** 2 / (2 * vt * vt))
    return float(np.trapezoid(v * f, v) / np.trapezoid(f, v))


@pytest.mark.parametrize("drift", [0.0, 4e5, -6e5])
def test_counts_follow_the_flux(oracle_backend, drift):
    n, T, L, dt, w, steps = 1e18, 2.0 * E / K_B, 0.008, 1e-12, 1e4, 20
    case = box_case(L=L, dt=dt, weight=w)
    sim = osim(oracle_backend, case, [cases.freestream(0, (0, 1), (n, n), T, velocity=(drift, 0.0, 0.0))])
    st = sim.step(steps)
    for s, m in ((0, M_E), (1, M_AR)):
        expect = flux_per_area(n, T, m, drift) * L * L * dt / w * steps   # patch 0 (-x): inward normal +x
        got = sim.count(s) + st.n_absorbed[s]     # a few leave through the side walls near the edges
        assert abs(got - expect) <= 4 * math.sqrt(0.25 * 64 * steps) + 1, (s, got, expect)
    assert sim.count(0) > 100


def test_parcels_start_on_the_faces(oracle_backend):
    case = box_case(n=4, L=0.004)
    # a near-zero temperature: the parcels barely move in their first step
    sim = osim(oracle_backend, case, [cases.freestream(3, (0,), (1e24,), 1e-6)])
    sim.step(1)
    tet, bary, U = sim.get_particles(0)
    assert len(tet) > 2000
    xyz = Mesh(case.mesh).position(tet, bary)
    assert np.all(np.abs(xyz[:, 1] - 0.004) < 1e-10)      # patch 3 is +y (moved ~4 m/s x 1 ps)
    assert np.all(U[:, 1] < 0)
    hist = np.histogram2d(xyz[:, 0], xyz[:, 2], bins=4, range=[[0, 0.004], [0, 0.004]])[0]
    assert hist.min() > 0.8 * hist.mean() and hist.max() < 1.2 * hist.mean()
    cells = tet // 12
    assert np.all((cells // 4) % 4 == 3)                   # owner cells of the +y faces


@pytest.mark.parametrize("drift_n,drift_t", [(0.0, (0.0, 0.0)), (3e5, (2e5, -1e5)), (-1.5e6, (0.0, 0.0)),
                                             (-3.0e6, (1e5, 0.0))])
def test_velocity_distribution(oracle_backend, drift_n, drift_t):
    # s = -3.57 for the last case: the |s| + 1 scaling of the rejection interval
    T = 2.0 * E / K_B
    vt = math.sqrt(K_B * T / M_E)
    L, dt, w = 0.04, 1e-12, 1e4
    case = box_case(n=4, L=L, dt=dt, weight=w)
    # patch 4 is -z: inward normal +z, tangents in the x-y plane
    U_d = (drift_t[0], drift_t[1], drift_n)
    dens = 30000 * w / (flux_per_area(1.0, T, M_E, drift_n) * L * L * dt)
    sim = osim(oracle_backend, case, [cases.freestream(4, (0,), (dens,), T, velocity=U_d)])
    sim.step(1)
    _, _, U = sim.get_particles(0)
    assert len(U) > 20000
    un = U[:, 2]
    assert np.all(un > 0)
    assert un.mean() == pytest.approx(mean_normal_speed(T, M_E, drift_n), rel=0.015)
    for a in (0, 1):
        assert U[:, a].mean() == pytest.approx(U_d[a], abs=0.02 * vt)
        assert U[:, a].std() == pytest.approx(vt, rel=0.02)


def test_box_patch_emits_through_every_face(oracle_backend):
    box = ((3, 3, 3), (5, 5, 5), cases.patch(abi.PATCH_ABSORB, 0.0))
    case = box_case(boxes=[box])
    sim = osim(oracle_backend, case, [cases.freestream(6, (0,), (1e20,), 2.0 * E / K_B)])
    sim.step(1)
    tet, bary, U = sim.get_particles(0)
    m = Mesh(case.mesh)
    cc, _ = m.cells()
    c = cc[tet // 12]
    lo, hi = 0.003, 0.005
    below, above = c < lo, c > hi
    outside = below.sum(axis=1) + above.sum(axis=1)
    assert np.all(outside >= 1)                     # nothing inside the box
    one = outside == 1                              # still in a face-adjacent cell (a few crossed an edge)
    assert one.mean() > 0.99
    un = (U * above).sum(axis=1) - (U * below).sum(axis=1)
    assert np.all(un[one] > 0)
    per_side = [(below[:, a]).sum() for a in range(3)] + [(above[:, a]).sum() for a in range(3)]
    assert min(per_side) > 0.8 * np.mean(per_side)


def test_freestream_checks(oracle_backend):
    sides = [cases.patch(abi.PATCH_WALL, 0.0)] + [cases.patch(abi.PATCH_ABSORB, 0.0) for _ in range(5)]
    case = cases.empty_case(sides=sides)
    sim = cases.build(case, backend=oracle_backend.OracleBackend(1))
    with pytest.raises(PicError):
        sim.set_freestream([cases.freestream(0, (0,), (1e15,), 300.0)])   # wall patch
    with pytest.raises(PicError):
        sim.set_freestream([cases.freestream(1, (0,), (1e15,), 0.0)])     # zero boundaryT
    with pytest.raises(PicError):
        sim.set_freestream([cases.freestream(1, (3,), (1e15,), 300.0)])   # no such species
    sim.set_freestream([cases.freestream(1, (0,), (1e15,), 300.0)])
