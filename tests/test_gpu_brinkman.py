"""GPU parity of the Brinkman iteration (src/brinkman/FluidBrinkman.cpp:282-553).

The kernels follow the reference expression by expression and are compiled
without FMA contraction, so the FP64 fields after k iterations equal the
reference's (tolerance 1e-14 relative, the order of the L2 sum differs only in
the residual)."""
import os

import numpy as np
import pytest

from conftest import ROOT, rel_err
from fft_method_test_gb300 import geometry as G

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def brinkman(*a, **k):
    from fft_method_test_gb300.permeability import solveBrinkman

    return solveBrinkman(*a, **k)


def test_brinkman_16_matches_reference_golden(gpu_lib):
    g = np.load(GOLDEN)
    ids = g["br16_ids"].astype(np.uint32)
    r = brinkman(ids, (1.0, 0.0, 0.0), solid_penalty=1e4, relaxation=0.9, tolerance=1e-8,
                 max_iterations=40, want_fields=True)
    assert r["iterations"] == 40 and not r["converged"]
    assert rel_err(r["ux"].ravel(), g["br16_ux"]) < 1e-14
    assert rel_err(r["superficialVelocity"], g["br16_U"]) < 1e-14
    assert abs(r["residual"] - g["br16_residual"][0]) <= 1e-12 * g["br16_residual"][0]


def test_brinkman_c2_128_matches_reference_golden(gpu_lib):
    g = np.load(GOLDEN)
    bits = g["c2_mask_bits"]
    mask = np.unpackbits(bits)[: 128 ** 3].reshape(128, 128, 128).astype(np.uint8)
    r = brinkman(G.to_ids(mask), (1.0, 0.0, 0.0), solid_penalty=1e4, max_iterations=10)
    assert rel_err(r["superficialVelocity"], g["c2_br10_U"]) < 1e-13
    assert abs(r["residual"] - g["c2_br10_residual"][0]) <= 1e-12 * g["c2_br10_residual"][0]
    assert abs(r["porosity"] - G.porosity(mask)) < 1e-15


@pytest.mark.parametrize("shape,seed", [((12, 12, 12), 3), ((5, 9, 7), 4)])
def test_brinkman_matches_oracle(gpu_lib, restatement, shape, seed):
    mask = (np.random.default_rng(seed).random(shape) >= 0.4).astype(np.uint8)
    ids = G.to_ids(mask)
    ro = restatement.brinkman(ids, 1, 1.3, 1e4, 0.9, 1e-8, 25, (0.2, -1.0, 0.5), want_fields=True)
    r = brinkman(ids, (0.2, -1.0, 0.5), fluid_mu=1.3, solid_penalty=1e4, max_iterations=25,
                 want_fields=True)
    for f in ("ux", "uy", "uz", "p"):
        assert rel_err(r[f].ravel(), ro[f]) < 1e-14, f
    assert r["iterations"] == ro["iterations"]


def test_brinkman_permeability_and_convergence(gpu_lib, restatement):
    from fft_method_test_gb300.permeability import computePermeabilityTensor

    mask = G.spheres(10, 2.0, 0.6, seed=8)
    ids = G.to_ids(mask)
    K, st = computePermeabilityTensor(ids, solid_penalty=1e4, tolerance=1e-30, max_iterations=30)
    for j in range(3):
        f = [0.0, 0.0, 0.0]
        f[j] = 1.0
        ro = restatement.brinkman(ids, 1, 1.0, 1e4, 0.9, 1e-30, 30, f)
        assert rel_err(K[:, j], ro["viscosity"] * ro["U"]) < 1e-13
    # a loose tolerance stops early exactly where the reference stops
    r = brinkman(ids, (1, 0, 0), solid_penalty=1e4, tolerance=1e-2, max_iterations=500)
    ro = restatement.brinkman(ids, 1, 1.0, 1e4, 0.9, 1e-2, 500, (1, 0, 0))
    assert r["converged"] and r["iterations"] == ro["iterations"]


def test_brinkman_errors(gpu_lib):
    from fft_method_test_gb300._capi import FpError

    with pytest.raises(FpError):  # no solid id
        brinkman(np.ones((4, 4, 4), np.uint32), (1, 0, 0))
    with pytest.raises(FpError):  # no fluid id
        brinkman(np.full((4, 4, 4), 2, np.uint32), (1, 0, 0))
    # over-relaxation diverges: the reference throws on a non-finite residual
    ids = G.to_ids(G.spheres(8, 2.0, 0.6, seed=2))
    with pytest.raises(FpError) as ei:
        brinkman(ids, (1, 0, 0), solid_penalty=1e4, relaxation=3.5, max_iterations=20000)
    assert "unstable" in str(ei.value)


# ---- the fixed point of the same equations (fp_brinkman_fft_solve) ----------

def fixed_point(*a, **k):
    from fft_method_test_gb300.permeability import solveBrinkmanFixedPoint

    return solveBrinkmanFixedPoint(*a, **k)


@pytest.mark.parametrize("shape,seed,force", [((12, 12, 12), 5, (1.0, 0.0, 0.0)),
                                              ((16, 16, 16), 6, (0.3, -1.0, 0.5)),
                                              ((10, 12, 8), 7, (0.0, 0.0, 2.0))])
def test_fixed_point_matches_direct_kkt_solve(gpu_lib, shape, seed, force):
    """Velocity equal to the direct sparse solve of the reference's discrete
    equations (oracle/brinkman_kkt.py) within 1e-8 relative; the pressure
    satisfies the momentum equation with it."""
    import brinkman_kkt as BK

    rng = np.random.default_rng(seed)
    mask = (rng.random(shape) >= 0.45).astype(np.uint8)
    ids = G.to_ids(mask)
    k = BK.solve(ids, solid_penalty=1e4, force=force)
    r = fixed_point(ids, force, solid_penalty=1e4, tolerance=1e-12, max_iterations=20000,
                    want_fields=True)
    assert r["converged"] and r["residual"] <= 1e-12
    for c in ("ux", "uy", "uz"):
        assert rel_err(r[c], k[c]) < 1e-8, c
    assert rel_err(r["superficialVelocity"], k["U"]) < 1e-9
    u = np.array([r["ux"], r["uy"], r["uz"]])
    mom, div = BK.residuals(ids, u, r["p"], solid_penalty=1e4, force=force)
    assert mom < 1e-7 * max(1.0, np.abs(force).max()) and div < 1e-10


def test_fixed_point_is_where_the_gpu_reference_scheme_goes(gpu_lib):
    """The reference scheme (kernels_brinkman.cu) run longer approaches the
    fixed point monotonically."""
    mask = G.spheres(16, 2.5, 0.6, seed=11)
    ids = G.to_ids(mask)
    fp_ = fixed_point(ids, (1.0, 0.0, 0.0), solid_penalty=1e4, tolerance=1e-11, want_fields=True)
    errs = []
    for its in (200, 2000, 8000):
        r = brinkman(ids, (1.0, 0.0, 0.0), solid_penalty=1e4, tolerance=1e-30, max_iterations=its,
                     want_fields=True)
        errs.append(rel_err(r["ux"], fp_["ux"]))
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 1e-2


def test_fixed_point_c2_128(gpu_lib):
    """C2: 128^3 spheres r=8 at porosity 0.45, penalty 1e4, tol 1e-8 (the
    tolerance the reference scheme cannot reach): converged, discretely
    divergence-free, and K symmetric to the solve tolerance."""
    from fft_method_test_gb300.permeability import computePermeabilityTensorFixedPoint

    g = np.load(GOLDEN)
    mask = np.unpackbits(g["c2_mask_bits"])[: 128 ** 3].reshape(128, 128, 128).astype(np.uint8)
    ids = G.to_ids(mask)
    r = fixed_point(ids, (1.0, 0.0, 0.0), solid_penalty=1e4, tolerance=1e-8, want_fields=True)
    assert r["converged"] and r["residual"] <= 1e-8
    div = sum(0.5 * (np.roll(r[c], -1, ax) - np.roll(r[c], 1, ax))
              for c, ax in (("ux", 2), ("uy", 1), ("uz", 0)))
    assert np.abs(div).max() < 1e-10 * np.abs(r["ux"]).max()
    K, st = computePermeabilityTensorFixedPoint(ids, solid_penalty=1e4, tolerance=1e-8)
    assert all(s["converged"] for s in st)
    assert np.abs(K - K.T).max() < 1e-6 * np.abs(K).max()
    assert abs(K[0, 0] - r["superficialVelocity"][0]) < 1e-7 * abs(K[0, 0])


def test_fixed_point_errors(gpu_lib):
    from fft_method_test_gb300 import _capi

    ids = G.to_ids((np.random.default_rng(1).random((8, 8, 8)) > 0.5).astype(np.uint8))
    with pytest.raises(_capi.FpError) as e:
        fixed_point(ids, (1.0, 0.0, 0.0), fluid_mu=1.3)
    assert e.value.code == _capi.FP_ERR_UNSUPPORTED
    with pytest.raises(_capi.FpError):
        fixed_point(np.ones((8, 8, 8), np.uint32), (1.0, 0.0, 0.0))
    with pytest.raises(ValueError):
        fixed_point(ids, (1.0, 0.0, 0.0), tolerance=0.0)
