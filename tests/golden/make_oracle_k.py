"""Generate tests/golden/oracle_k.npz: CPU-oracle permeability tensors of
cells at the configurations' scale.  TEST INFRASTRUCTURE ONLY.

The checker is the plain-C restatement (oracle/fftperm_oracle.c), which is
pinned bit for bit to the reference build at one thread
(tests/test_oracle_cpu.py); here it runs on all host threads (K then agrees
with the one-thread result to round-off, far below the solve tolerance).

    python tests/golden/make_oracle_k.py [case ...]     # default: every case

Each case stores its grid, generator parameters, the sha256 of the mask
bytes (so a consumer can check that the regenerated mask is this one), the
mask itself as packed bits for grids up to 160^3, the tolerance, K and the
iteration counts.  Results are merged into the existing file, so cases can
be generated one at a time.

Cases:
  grf64        64^3 Gaussian random field (l 6, porosity 0.35, seed 3064), tol 1e-10
  grf128       128^3 Gaussian random field (l 6, porosity 0.35, seed 3128), tol 1e-10
  c4_96_grf    batch cell seed 2027: 96^3 Gaussian field, porosity 0.493, tol 1e-10
  c4_160_sph   batch cell seed 2012: 160^3 spheres r 3-10, porosity 0.337, tol 1e-10
  c2_128_sph   the Brinkman cell (128^3 spheres r 8, porosity 0.45, seed 1002), tol 1e-10
  grf256       the benchmark cell (256^3, l 6, porosity 0.35, seed 1003), tol 1e-7 (the
               benchmark's own stopping tolerance: its iteration counts are the
               CPU reference's at that tolerance)
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from fft_method_test_gb300 import geometry as G  # noqa: E402

PATH = os.path.join(HERE, "oracle_k.npz")
MAXIT = 20000

CASES = {
    "grf64": (lambda: G.gaussian_field(64, 6.0, 0.35, seed=3064), 1e-10),
    "grf128": (lambda: G.gaussian_field(128, 6.0, 0.35, seed=3128), 1e-10),
    "c4_96_grf": (lambda: G.batch_cell(2027), 1e-10),
    "c4_160_sph": (lambda: G.batch_cell(2012), 1e-10),
    "c2_128_sph": (lambda: G.spheres(128, 8.0, 0.45, seed=1002), 1e-10),
    "grf256": (lambda: G.gaussian_field(256, 6.0, 0.35, seed=1003), 1e-7),
}


def mask_sha(mask: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(mask, dtype=np.uint8).tobytes()).hexdigest()


def load() -> dict:
    if not os.path.exists(PATH):
        return {}
    with np.load(PATH) as z:
        return {k: z[k] for k in z.files}


def main(names):
    import oracle as orc

    R = orc.Restatement()
    for name in names:
        gen, tol = CASES[name]
        mask = gen()
        t0 = time.perf_counter()
        ctx = R.context(mask, threads=0)
        K, it = ctx.solve_permeability(tol, MAXIT)
        nb = ctx.nb
        ctx.close()
        dt = time.perf_counter() - t0
        out = load()
        out[name + "_shape"] = np.array(mask.shape, dtype=np.int64)
        out[name + "_sha256"] = np.array(mask_sha(mask))
        if mask.size <= 160 ** 3:
            out[name + "_mask_bits"] = np.packbits(mask.ravel())
        out[name + "_tol"] = np.array(tol)
        out[name + "_K"] = K
        out[name + "_iters"] = np.asarray(it, dtype=np.int64)
        out[name + "_nb"] = np.array(nb, dtype=np.int64)
        out[name + "_seconds"] = np.array(dt)
        np.savez_compressed(PATH, **out)
        print("%s: nb=%d iterations=%s %.1f s K=%s" % (name, nb, list(it), dt, K.ravel()),
              flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or list(CASES))
