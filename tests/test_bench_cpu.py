"""Host-side pieces of bench.py (no GPU): the roofline byte model, the
synthetic workloads and the CPU-baseline extrapolation."""
import os
import sys

import numpy as np

from conftest import ROOT

sys.path.insert(0, ROOT)


def test_apply_byte_model():
    """216 B per half-spectrum point + 56 B per support voxel in mixed mode
    (FP32 spectrum and Green table, FP64 compact vectors); 432 + 56 in FP64."""
    import bench

    nh, nb = 1000, 37
    assert bench.apply_bytes(nh, nb, "mixed") == 216 * nh + 56 * nb
    assert bench.apply_bytes(nh, nb, "fp64") == 432 * nh + 56 * nb
    # the 256^3 figure quoted with the bench line
    nh256 = (256 // 2 + 1) * 256 * 256
    assert abs(bench.apply_bytes(nh256, 1823496, "mixed") - 1928210880) < 1


def test_headline_workload_is_deterministic():
    import bench

    a = bench.workload_mask(32, 1003)
    b = bench.workload_mask(32, 1003)
    assert np.array_equal(a, b)
    assert abs(a.mean() - 0.35) < 1e-3


def test_batch_workload_matches_its_specification():
    """Edges from {48, 64, 80, 96, 128, 160}, porosity in [0.3, 0.8], seeds
    2000.. (spheres on even seeds, Gaussian fields on odd)."""
    import bench

    masks = bench.batch_workload(6)
    assert len(masks) == 6
    for i, m in enumerate(masks):
        assert m.ndim == 3 and m.shape[0] == m.shape[1] == m.shape[2]
        assert m.shape[0] in (48, 64, 80, 96, 128, 160)
        rng = np.random.default_rng(2000 + i)
        edge = int(rng.choice([48, 64, 80, 96, 128, 160]))
        phi = float(rng.uniform(0.3, 0.8))
        assert m.shape[0] == edge
        assert abs(m.mean() - phi) < 0.02, (i, m.mean(), phi)


def test_cpu_model_units_and_prediction(restatement):
    """The CPU baseline times the oracle's set-up, one apply and one MINRES
    iteration on the cell; seconds to K = set-ups + per load case two applies
    (RHS, recovery) + iterations x iteration time."""
    import bench
    from fft_method_test_gb300 import geometry as G

    mask = G.spheres(16, 3.0, 0.6, seed=7)
    u = bench.cpu_units(mask, threads=1)
    assert u["setup_s"] > 0 and u["apply_s"] > 0 and u["iter_s"] > 0
    its = [100, 120, 80]
    want = 3 * u["setup_s"] + sum(2 * u["apply_s"] + i * u["iter_s"] for i in its)
    assert abs(bench.cpu_predict(u, its, setups=3) - want) <= 1e-12 * want


def test_cpu_model_check_reports_a_full_solve(restatement):
    import bench
    from fft_method_test_gb300 import geometry as G

    chk = bench.cpu_model_check(G.spheres(16, 3.0, 0.6, seed=7), 1e-6, threads=1)
    assert chk["measured_s"] > 0 and chk["predicted_s"] > 0
    assert len(chk["iterations"]) == 3 and all(i > 0 for i in chk["iterations"])
    assert abs(chk["rel_err"]) < 1.0


def test_oracle_fixture_requires_the_same_mask():
    """The committed oracle K is used only for the very cell it was computed on."""
    import bench

    from fft_method_test_gb300 import geometry as G

    m = G.gaussian_field(64, 6.0, 0.35, seed=3064)
    fx = bench.oracle_fixture("grf64", m)
    assert fx is not None and fx["K"].shape == (3, 3) and len(fx["iterations"]) == 3
    m2 = m.copy()
    m2.flat[0] ^= 1
    assert bench.oracle_fixture("grf64", m2) is None
    assert bench.oracle_fixture("no_such_cell", m) is None
