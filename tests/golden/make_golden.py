"""Generate tests/golden/golden.npz from the reference's OWN code.

Run where the reference sources are available (they are compiled unmodified
into oracle/_ref by ``make -C oracle ref``):

    python tests/golden/make_golden.py

Every value stored here is produced by the reference's classes
(oracle/ref_capi.cpp drives them) on seeded synthetic geometries; the tests
compare the C restatement of the oracle and the GPU path against them.
"""
from __future__ import annotations

import os
import sys

# The reference's MINRES dot products are OpenMP reductions whose summation
# order depends on the thread count; one thread makes its output
# deterministic (and bit-identical to the C restatement).
os.environ["OMP_NUM_THREADS"] = "1"

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as orc  # noqa: E402
from fft_method_test_gb300 import geometry as G  # noqa: E402


def main():
    ref = orc.Reference()
    out = {}

    # C1: 32^3 spheres r=4 porosity 0.60 seed 1001, tol 1e-10 (maxit 2000)
    m1 = G.spheres(32, 4.0, 0.60, seed=1001)
    out["c1_mask_bits"] = np.packbits(m1.ravel())
    out["c1_support"] = ref.support(m1).astype(np.int32)
    ctx = ref.context(m1, threads=1)
    K, it = ctx.solve_permeability(1e-10, 2000)
    out["c1_K"] = K
    out["c1_iters"] = it
    b = ctx.build_rhs([1.0, 0.0, 0.0])
    r = ctx.minres(b, 1e-10, 60)
    out["c1_hist60_x"] = r["residual_history"]
    ctx.close()

    # 16^3 operator apply on a seeded vector
    m2 = G.spheres(16, 3.0, 0.6, seed=7)
    out["op16_mask_bits"] = np.packbits(m2.ravel())
    ctx = ref.context(m2)
    x = np.random.default_rng(42).uniform(-1.0, 1.0, 3 * ctx.nb)
    out["op16_x"] = x
    out["op16_y"] = ctx.operator_apply(x)
    out["op16_rhs_y"] = ctx.build_rhs([0.0, 1.0, 0.0])
    avg, _ = ctx.recover([1.0, 0.0, 0.0], 0.1 * x)
    out["op16_recover_avg"] = avg
    ctx.close()

    # Green tensor of a non-cubic grid (full C2C spectrum)
    out["green_3x5x6"] = ref.green_tensor((3, 5, 6))

    # Brinkman: 16^3, alpha = 1e4, 40 iterations from rest
    ids16 = G.to_ids(G.spheres(16, 3.0, 0.6, seed=21))
    out["br16_ids"] = ids16.astype(np.uint8)
    rb = ref.brinkman(ids16, 1, 1.0, 1e4, 0.9, 1e-8, 40, (1.0, 0.0, 0.0), want_fields=True)
    out["br16_U"] = rb["U"]
    out["br16_residual"] = np.array([rb["residual"]])
    out["br16_ux"] = rb["ux"]

    # C2 geometry (128^3 spheres r=8 porosity 0.45 seed 1002): 10 Brinkman iterations
    m3 = G.spheres(128, 8.0, 0.45, seed=1002)
    out["c2_mask_bits"] = np.packbits(m3.ravel())
    rb = ref.brinkman(G.to_ids(m3), 1, 1.0, 1e4, 0.9, 1e-8, 10, (1.0, 0.0, 0.0))
    out["c2_br10_U"] = rb["U"]
    out["c2_br10_residual"] = np.array([rb["residual"]])

    path = os.path.join(HERE, "golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
