"""The whole-population entry points of the C ABI on the GPU:
picgpu_upload_particles / picgpu_download_particles round-trip a mixed
population of both species through the context, and picgpu_get_fields
returns what picgpu_get_field does for phi, E and rho."""
import ctypes as C

import numpy as np
import pytest

from picfoam_gb300 import abi, cases

pytestmark = pytest.mark.gpu


def test_soa_round_trip_and_fields(gpu):
    case = cases.two_species_3d(n_cells=6, per_cell=10, precision=abi.PREC_FP64, L=0.003)
    sim = cases.build(case, backend=gpu)
    lib = sim.lib
    P = C.POINTER
    lib.picgpu_upload_particles.argtypes = [C.c_void_p, P(abi.ParticlesSoa), C.c_size_t]
    lib.picgpu_download_particles.argtypes = [C.c_void_p, P(abi.ParticlesSoa), C.c_size_t, P(C.c_size_t)]
    lib.picgpu_get_fields.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double), P(C.c_double)]
    # interleave the two species' parcels in one set
    parts = [sim.get_particles(s) for s in (0, 1)]
    n0, n1 = len(parts[0][0]), len(parts[1][0])
    order = np.random.default_rng(3).permutation(n0 + n1)
    species = np.concatenate([np.zeros(n0, np.int32), np.ones(n1, np.int32)])[order]
    tet = np.concatenate([parts[0][0], parts[1][0]]).astype(np.int32)[order]
    bary = np.ascontiguousarray(np.concatenate([parts[0][1], parts[1][1]])[order])
    U = np.ascontiguousarray(np.concatenate([parts[0][2], parts[1][2]])[order])

    def soa(sp, t, b, u):
        return abi.ParticlesSoa(sp.ctypes.data_as(P(C.c_int32)), t.ctypes.data_as(P(C.c_int32)),
                                b.ctypes.data_as(P(C.c_double)), u.ctypes.data_as(P(C.c_double)))

    assert lib.picgpu_upload_particles(sim._h, C.byref(soa(species, tet, bary, U)), len(tet)) == 0
    assert (sim.count(0), sim.count(1)) == (n0, n1)
    N = n0 + n1
    out = [np.zeros(N, np.int32), np.zeros(N, np.int32), np.zeros((N, 3)), np.zeros((N, 3))]
    n = C.c_size_t(0)
    assert lib.picgpu_download_particles(sim._h, C.byref(soa(*out)), N - 1, C.byref(n)) != 0
    assert n.value == N
    assert lib.picgpu_download_particles(sim._h, C.byref(soa(*out)), N, C.byref(n)) == 0
    assert n.value == N and np.all(out[0][:n0] == 0) and np.all(out[0][n0:] == 1)
    for s, sl in ((0, slice(0, n0)), (1, slice(n0, N))):
        keep = species == s
        np.testing.assert_array_equal(out[1][sl], tet[keep])        # stable grouping by species
        np.testing.assert_array_equal(out[2][sl], bary[keep])
        np.testing.assert_array_equal(out[3][sl], U[keep])
    sim.step(2)
    nc = 6 ** 3
    phi, E, rho = np.zeros(nc), np.zeros(3 * nc), np.zeros(nc)
    f = lambda a: a.ctypes.data_as(P(C.c_double))
    assert lib.picgpu_get_fields(sim._h, f(phi), f(E), f(rho)) == 0
    np.testing.assert_array_equal(phi, sim.field(abi.FIELD_PHI))
    np.testing.assert_array_equal(E, sim.field(abi.FIELD_E_CELL).ravel())
    np.testing.assert_array_equal(rho, sim.field(abi.FIELD_RHO))
    assert lib.picgpu_get_fields(sim._h, None, None, f(rho)) == 0
