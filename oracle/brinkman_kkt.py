"""Direct solve of the Brinkman fixed point.  TEST INFRASTRUCTURE ONLY.

The reference iteration (src/brinkman/FluidBrinkman.cpp:282-507) is at rest
exactly where

    (alpha + 6 mu) u - mu sum_nbr u + grad_c p = f      (momentum, :313-369, u* = u)
    div_c u = 0                                           (projection, :371-466, phi = 0)

with, per voxel, alpha = solid_penalty on solid and 0 on fluid, mu =
fluid_mu on fluid and 1 on solid (buildCoefficientFields, :152-191),
sum_nbr the six periodic face neighbours, and grad_c / div_c the periodic
central difference 0.5 (a[+1] - a[-1]) (:335-337, :380-383).  This module
assembles that saddle-point system as a sparse matrix and solves it with
scipy's direct solver.  The pressure is fixed only up to the null space of
grad_c (constants and the checkerboards at k_i = n_i/2); a -eps I block on
the pressure (eps = 1e-12) selects one representative and perturbs u by
O(eps).

Used by the tests to check fp_brinkman_fft_solve, and pinned by a test that
runs the reference scheme itself for many iterations toward the same point.
"""
from __future__ import annotations

import numpy as np


def solve(ids: np.ndarray, fluid_id: int = 1, fluid_mu: float = 1.0, solid_penalty: float = 1e4,
          force=(1.0, 0.0, 0.0), eps: float = 1e-12):
    """Returns dict(ux, uy, uz, p, U) for material ids of shape (nz, ny, nx)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    ids = np.asarray(ids)
    nz, ny, nx = ids.shape
    n = ids.size
    fluid = (ids == fluid_id).ravel()
    alpha = np.where(fluid, 0.0, float(solid_penalty))
    mu = np.where(fluid, float(fluid_mu), 1.0)
    idx = np.arange(n).reshape(nz, ny, nx)

    def shift(axis, s):
        # row i picks the neighbour at +s along axis (x-fastest flat index)
        cols = np.roll(idx, -s, axis=axis).ravel()
        return sp.csr_matrix((np.ones(n), (np.arange(n), cols)), shape=(n, n))

    nbr = sum(shift(a, s) for a in (0, 1, 2) for s in (1, -1))
    gx = 0.5 * (shift(2, 1) - shift(2, -1))
    gy = 0.5 * (shift(1, 1) - shift(1, -1))
    gz = 0.5 * (shift(0, 1) - shift(0, -1))
    A = sp.diags(alpha + 6.0 * mu) - sp.diags(mu) @ nbr
    Z = sp.csr_matrix((n, n))
    K = sp.bmat([[A, Z, Z, gx], [Z, A, Z, gy], [Z, Z, A, gz], [gx, gy, gz, -eps * sp.identity(n)]],
                format="csc")
    f = np.asarray(force, dtype=np.float64)
    rhs = np.concatenate([np.full(n, f[0]), np.full(n, f[1]), np.full(n, f[2]), np.zeros(n)])
    sol = spl.spsolve(K, rhs)
    ux, uy, uz, p = (sol[i * n:(i + 1) * n].reshape(nz, ny, nx) for i in range(4))
    return dict(ux=ux, uy=uy, uz=uz, p=p, U=np.array([ux.mean(), uy.mean(), uz.mean()]))


def residuals(ids, u, p, fluid_id=1, fluid_mu=1.0, solid_penalty=1e4, force=(1.0, 0.0, 0.0)):
    """Max-norm momentum and divergence residuals of (u, p) in the discrete
    equations above (u: (3, nz, ny, nx))."""
    ids = np.asarray(ids)
    fluid = ids == fluid_id
    alpha = np.where(fluid, 0.0, float(solid_penalty))
    mu = np.where(fluid, float(fluid_mu), 1.0)
    axes = (2, 1, 0)  # x, y, z components differentiate along these array axes

    def grad(a, ax):
        return 0.5 * (np.roll(a, -1, ax) - np.roll(a, 1, ax))

    mom = 0.0
    for c in range(3):
        s = sum(np.roll(u[c], sh, ax) for ax in (0, 1, 2) for sh in (1, -1))
        r = (alpha + 6 * mu) * u[c] - mu * s + grad(p, axes[c]) - force[c]
        mom = max(mom, float(np.abs(r).max()))
    div = sum(grad(u[c], axes[c]) for c in range(3))
    return mom, float(np.abs(div).max())
