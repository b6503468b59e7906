"""Particle transfers from and to page-locked host arrays
(picgpu_host_alloc): the direct DMA path gives the same particles as the
pinned ring that pageable arrays take, bit for bit, for stores above the
ring's 8 MB threshold."""
import numpy as np
import pytest

from picfoam_gb300 import abi, cases
from picfoam_gb300.simulation import pinned_empty

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [abi.PREC_MIXED, abi.PREC_FP64])
def test_pinned_transfers_match_pageable(gpu, precision):
    case = cases.two_species_3d(n_cells=24, per_cell=40, precision=precision)
    a = cases.build(case, backend=gpu)                  # pageable arrays (ring)
    b = cases.build(case, backend=gpu)
    for s, (tet, bary, U) in case.particles.items():
        n = len(tet)
        pin = (pinned_empty(n, np.int32), pinned_empty((n, 3), np.float64), pinned_empty((n, 3), np.float64))
        for dst, src in zip(pin, (tet, bary, U)):
            dst[...] = src
        b.set_particles(s, *pin)                        # page-locked arrays (direct)
    for _ in range(2):
        a.move()
        b.move()
    for s in case.particles:
        n = b.count(s)
        out = (pinned_empty(n, np.int32), pinned_empty((n, 3), np.float64), pinned_empty((n, 3), np.float64))
        got = b.get_particles(s, out=out)
        ref = a.get_particles(s)
        assert len(ref[0]) == n
        for x, y in zip(got, ref):
            np.testing.assert_array_equal(x, y)
    a.close()
    b.close()
