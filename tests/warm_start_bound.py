"""How many Jacobi-PCG iterations a better start potential can save, measured
on a model problem (TEST INFRASTRUCTURE; CPU only, numpy + scipy).

    python tests/warm_start_bound.py [n]

The cell-centred 7-point Laplacian on an n^3 box with Dirichlet walls (the
operator of the electrostatic solve on a uniform block mesh), a smooth
charge density plus cell noise, and a step-to-step change of the right-hand
side of 10 % of its norm as white noise (the shot-noise increment a PIC step
makes; the previous-step potential then starts at a relative residual of
about 0.1, as on the electrode case).  Printed, as one JSON document:

  previous          iterations to 1e-8 from the previous potential
  coarse_head       from the previous potential plus a Galerkin coarse-grid
                    correction of its residual (aggregates of a^3 cells)
  smoothed          from the previous potential plus ten weighted-Jacobi
                    sweeps on the error equation (a local predictor that
                    removes the high-frequency residual, as the U-Net does)
  exact_plus_error  from the exact solution plus an error whose residual is
                    white noise of relative size eps: the iterations as a
                    function of the start residual alone

The iteration count falls by a fixed amount per decade of start residual,
so halving it needs a start guess about 1e-4.5 accurate in the relative
residual: a predictor as accurate as several multigrid cycles.
"""
import json
import sys

import numpy as np
import scipy.sparse as sp


def laplacian(n):
    t = sp.diags([-np.ones(n - 1), 2 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1])
    i = sp.identity(n)
    return (sp.kron(sp.kron(t, i), i) + sp.kron(sp.kron(i, t), i) + sp.kron(sp.kron(i, i), t)).tocsr()


def pcg(A, D, b, x0, tol, maxit=20000):
    """Jacobi-preconditioned CG until ||b - Ax|| <= tol ||b||."""
    x = x0.copy()
    r = b - A @ x
    z = r / D
    p = z.copy()
    rz = r @ z
    nb = np.linalg.norm(b)
    for k in range(maxit):
        if np.linalg.norm(r) <= tol * nb:
            return x, k
        q = A @ p
        a = rz / (p @ q)
        x += a * p
        r -= a * q
        z = r / D
        rz, rz_old = r @ z, rz
        p = z + (rz / rz_old) * p
    return x, maxit


def aggregation(n, a):
    m = n // a
    c = np.arange(n) // a
    idx = (c[:, None, None] * m * m + c[None, :, None] * m + c[None, None, :]).ravel()
    return sp.csr_matrix((np.ones(n ** 3), (np.arange(n ** 3), idx)), shape=(n ** 3, m ** 3))


def main(n=64, seed=1):
    A = laplacian(n)
    D = A.diagonal()
    N = n ** 3
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    b_prev = (np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(np.pi * Z)).ravel() + 0.2 * rng.standard_normal(N)
    phi_prev, _ = pcg(A, D, b_prev, np.zeros(N), 1e-13)
    delta = rng.standard_normal(N)
    b = b_prev + delta * 0.1 * np.linalg.norm(b_prev) / np.linalg.norm(delta)
    r0 = b - A @ phi_prev
    rel = lambda v: float(np.linalg.norm(b - A @ v) / np.linalg.norm(b))  # noqa: E731
    out = {"n": n, "start_residual": rel(phi_prev), "previous": pcg(A, D, b, phi_prev, 1e-8)[1], "coarse_head": {}}
    for a in (16, 8, 4):
        P = aggregation(n, a)
        x0 = phi_prev + P @ np.linalg.solve((P.T @ A @ P).toarray(), P.T @ r0)
        out["coarse_head"][f"{a}^3"] = {"iterations": pcg(A, D, b, x0, 1e-8)[1], "start_residual": rel(x0)}
    e = np.zeros(N)
    for _ in range(10):
        e += 0.67 * (r0 - A @ e) / D
    out["smoothed"] = {"iterations": pcg(A, D, b, phi_prev + e, 1e-8)[1], "start_residual": rel(phi_prev + e)}
    xs, _ = pcg(A, D, b, phi_prev, 1e-14)
    out["exact_plus_error"] = {}
    for eps in (1e-1, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6):
        w = rng.standard_normal(N)
        w *= eps * np.linalg.norm(b) / np.linalg.norm(w)
        err, _ = pcg(A, D, w, np.zeros(N), 1e-12)
        out["exact_plus_error"][f"{eps:g}"] = pcg(A, D, b, xs + err, 1e-8)[1]
    return out


if __name__ == "__main__":
    print(json.dumps(main(int(sys.argv[1]) if len(sys.argv) > 1 else 64), indent=1))
