"""picgpu_solve_ldu_noalloc: the allocation-free PCG entry point.

Callers that cannot call cudaMalloc (a plugin inside a framework whose memory
pool owns the device, or a loop that must not hit cudaMalloc's device-wide
synchronisation) hand the solver their own device buffers; the solver's
working vectors come from a fixed __device__ array.  This test drives the
entry point through the C ABI and checks it against picgpu_solve_poisson on
the same Poisson problem, for two calls in a row (the second starting from
the first call's answer, so stale scratch contents would show).
"""
import ctypes as C

import numpy as np
import pytest

from picfoam_gb300 import abi, cases, native

pytestmark = pytest.mark.gpu


def laplacian_ell(n, L):
    """-laplacian of an n^3 cube with grounded walls in the cell-face form
    the entry point takes (diag, off[6n], nbr[6n])."""
    dx = L / n
    nc = n ** 3
    idx = np.arange(nc)
    i, j, k = idx % n, (idx // n) % n, idx // (n * n)
    nbr = np.full((nc, 6), -1, np.int32)
    off = np.zeros((nc, 6))
    diag = np.zeros(nc)
    a, a_wall = dx, 2.0 * dx  # |S|/|d| between centres, |S|/(dx/2) to a wall
    for f, (coord, step, stride) in enumerate([(i, -1, 1), (i, 1, 1), (j, -1, n), (j, 1, n),
                                               (k, -1, n * n), (k, 1, n * n)]):
        inside = (coord + step >= 0) & (coord + step < n)
        nbr[inside, f] = (idx + step * stride)[inside]
        off[inside, f] = -a
        diag += np.where(inside, a, a_wall)
    return diag, off.ravel(), nbr.ravel(), dx ** 3


def test_noalloc_pcg_matches_solve_poisson(gpu):
    torch = pytest.importorskip("torch")
    n, L, tol = 16, 0.004, 1e-13
    case = cases.two_species_3d(n_cells=n, per_cell=1, precision=abi.PREC_FP64, pcg_tol=tol, L=L)
    sim = cases.build(case, backend=gpu)
    lib = native.load()
    diag, off, nbr, V = laplacian_ell(n, L)
    dev = torch.device("cuda")
    d_diag = torch.tensor(diag, device=dev)
    d_off = torch.tensor(off, device=dev)
    d_nbr = torch.tensor(nbr, device=dev)
    d_x = torch.zeros(n ** 3, dtype=torch.float64, device=dev)
    rng = np.random.default_rng(11)
    phi_prev = np.zeros(n ** 3)
    for call in range(2):
        rho = rng.standard_normal(n ** 3) * 1e-5
        ref, st = sim.solve_poisson(rho, phi0=phi_prev)
        d_b = torch.tensor((rho / cases.EPS0) * V, device=dev)
        d_x.copy_(torch.tensor(phi_prev, device=dev))
        iters = C.c_int(-1)
        res = C.c_double(-1.0)
        status = lib.picgpu_solve_ldu_noalloc(n ** 3, d_diag.data_ptr(), d_off.data_ptr(), d_nbr.data_ptr(),
                                              d_b.data_ptr(), d_x.data_ptr(), tol, 20000, C.byref(iters),
                                              C.byref(res), None)
        assert status == abi.OK, abi.STATUS_NAMES.get(status)
        torch.cuda.synchronize()
        x = d_x.cpu().numpy()
        assert 0 < iters.value <= 20000 and res.value <= tol
        scale = np.abs(ref).max()
        np.testing.assert_allclose(x, ref, rtol=0, atol=1e-10 * scale, err_msg=f"call {call}")
        phi_prev = ref
    # beyond the fixed scratch: rejected before any GPU work
    status = lib.picgpu_solve_ldu_noalloc(65537, d_diag.data_ptr(), d_off.data_ptr(), d_nbr.data_ptr(),
                                          d_x.data_ptr(), d_x.data_ptr(), tol, 10, None, None, None)
    assert status == abi.CAPACITY
    sim.close()
