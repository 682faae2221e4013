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


def test_cpu_baseline_extrapolation(restatement):
    """The CPU baseline times the oracle's set-up and applies on the given
    cell and extrapolates to 3 x (Green precompute + (iterations/3 + 2)
    applies), the reference's per-load-case structure."""
    import bench
    from fft_method_test_gb300 import geometry as G

    mask = G.spheres(16, 3.0, 0.6, seed=7)
    total, cores, info = bench.cpu_sample(mask, 300, threads=1, sample_applies=2)
    assert cores == 1 and info["sample_applies"] == 2
    expect = 3 * (info["setup_s"] + (300 / 3.0 + 2) * info["apply_s"])
    assert abs(total - expect) <= 1e-12 * expect
    assert info["setup_s"] > 0 and info["apply_s"] > 0
