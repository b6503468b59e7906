"""Known-answer checks of the oracle's own mesh (no GPU).

The oracle states the block mesh of the hot path by itself (oracle/omesh.hpp,
from OpenFOAM's polyMesh conventions and the tet decomposition picFoam's
VolumeWeighting walks); these checks pin it from first principles rather
than against the library: the twelve tets fill the cell, barycentric
coordinates round-trip through positions and give unit vectors at the tet
vertices, the Gauss Laplacian of a linear potential vanishes away from
boundaries, VolumeWeighting's distance weights and the cell -> point
interpolation weights are partitions of unity, a cell's face area vectors
close, and every tet move across a face can be undone.
"""
import ctypes as C

import numpy as np
import pytest

from picfoam_gb300 import abi, cases

NAMES = ["tet volumes", "position round trip", "vertex coordinates", "laplacian of a linear field",
         "distance weights", "interpolation weights", "closed faces", "tet moves"]


def selfcheck(oracle_backend, mesh):
    lib = oracle_backend.load()
    out = (C.c_double * 8)()
    n = lib.oracle_mesh_selfcheck(C.byref(mesh), out, 8)
    assert n == 8
    return dict(zip(NAMES, list(out)))


def side(kind):
    return cases.patch(kind)


MESHES = {
    "cube": cases.block_mesh((6, 6, 6), (0.05, 0.05, 0.05), [side(abi.PATCH_ABSORB)] * 6),
    "anisotropic_with_boxes": cases.block_mesh(
        (12, 9, 7), (0.03, 0.011, 0.02), [side(abi.PATCH_ABSORB)] * 2 + [side(abi.PATCH_WALL)] * 2 +
        [side(abi.PATCH_ABSORB)] * 2, origin=(-0.01, 0.002, 0.3),
        boxes=[((2, 2, 2), (4, 5, 3), side(abi.PATCH_FLOATING)), ((7, 1, 4), (10, 3, 6), side(abi.PATCH_WALL))]),
    "cyclic": cases.block_mesh((8, 5, 4), (0.02, 0.02, 0.01), [side(abi.PATCH_CYCLIC)] * 4 +
                               [side(abi.PATCH_ABSORB)] * 2),
    "line_with_empty_sides": cases.block_mesh((32, 1, 1), (0.1, 7.8125e-4, 7.8125e-4),
                                              [side(abi.PATCH_CYCLIC)] * 2 + [side(abi.PATCH_EMPTY)] * 4),
}


@pytest.mark.parametrize("name", list(MESHES))
def test_oracle_mesh_known_answers(oracle_backend, name):
    r = selfcheck(oracle_backend, MESHES[name])
    assert r["tet volumes"] < 1e-14
    assert r["position round trip"] < 1e-12
    assert r["vertex coordinates"] < 1e-13
    assert r["laplacian of a linear field"] < 1e-12
    assert r["distance weights"] < 1e-14
    assert r["interpolation weights"] < 1e-14
    assert r["closed faces"] < 1e-14
    assert r["tet moves"] == 0.0


def test_oracle_mesh_rejects_bad_descriptions(oracle_backend):
    lib = oracle_backend.load()
    out = (C.c_double * 8)()
    bad = cases.block_mesh((4, 2, 4), (0.01, 0.01, 0.01), [side(abi.PATCH_ABSORB)] * 2 +
                           [side(abi.PATCH_EMPTY)] * 2 + [side(abi.PATCH_ABSORB)] * 2)
    assert lib.oracle_mesh_selfcheck(C.byref(bad), out, 8) == -1   # an empty direction two cells thick
    every_cell_removed = cases.block_mesh((2, 2, 2), (0.01, 0.01, 0.01), [side(abi.PATCH_ABSORB)] * 6,
                                          boxes=[((0, 0, 0), (2, 2, 2), side(abi.PATCH_WALL))])
    assert lib.oracle_mesh_selfcheck(C.byref(every_cell_removed), out, 8) == -1
    assert np.isfinite(list(out)).all()
