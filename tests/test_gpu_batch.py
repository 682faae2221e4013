"""Batched solves of uneven microstructures, graph-replayed MINRES chunks and
the tile autotuner (no reference counterpart: the reference solves one
geometry per run).  Every batched K must equal the single-problem solve of
the same mask, and the FP64 ones the oracle's."""
import os

import numpy as np
import pytest

from conftest import rel_err
from fft_method_test_gb300 import geometry as G

pytestmark = pytest.mark.gpu


def _masks():
    return [G.spheres(24, 3.0, 0.6, seed=31),
            G.gaussian_field((20, 24, 30), 3.0, 0.5, seed=32),
            G.spheres(16, 2.0, 0.55, seed=33),
            G.gaussian_field(32, 4.0, 0.45, seed=34),
            G.spheres((18, 20, 16), 2.5, 0.65, seed=35)]


def _single(mask, precision, tol, maxit=6000):
    from fft_method_test_gb300.permeability import PermeabilityProblem

    with PermeabilityProblem(mask.shape, precision=precision) as p:
        p.set_geometry(mask)
        K, st = p.solve_permeability(tol, maxit)
    return K, st


def test_graph_replay_matches_plain_launches(gpu_lib):
    """MINRES chunks replayed as CUDA graphs give the same iterates as
    launching each kernel: bit-identical K and iteration counts."""
    mask = G.spheres(20, 2.5, 0.6, seed=41)
    K1, st1 = _single(mask, "fp64", 1e-10)
    os.environ["FFTPERM_NO_GRAPHS"] = "1"
    try:
        K0, st0 = _single(mask, "fp64", 1e-10)
    finally:
        del os.environ["FFTPERM_NO_GRAPHS"]
    assert np.array_equal(K1, K0)
    assert [s["iterations"] for s in st1] == [s["iterations"] for s in st0]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_batch_matches_single_solves(gpu_lib, precision, tol):
    from fft_method_test_gb300.permeability import batch_solve_permeability

    masks = _masks()
    K, stats, status = batch_solve_permeability(masks, precision=precision, tol=tol, maxit=6000,
                                                concurrency=3, autotune=True)
    assert status == [0] * len(masks)
    for i, m in enumerate(masks):
        Ks, sts = _single(m, precision, tol)
        # the tuned tiling regroups the partial sums of the x pass: equal to
        # rounding, amplified by the Krylov recurrence
        assert rel_err(K[i], Ks) < (1e-10 if precision == "fp64" else 1e-6), i
        assert all(s["converged"] for s in stats[i])


def test_batch_fp64_matches_oracle(gpu_lib, restatement):
    from fft_method_test_gb300.permeability import batch_solve_permeability

    masks = _masks()[:3]
    K, _, status = batch_solve_permeability(masks, precision="fp64", tol=1e-10, maxit=6000,
                                            concurrency=2, autotune=False)
    for i, m in enumerate(masks):
        K_ref, _ = restatement.context(m).solve_permeability(1e-10, 6000)
        assert rel_err(K[i], K_ref) < 1e-9, i


def test_autotune_keeps_the_apply(gpu_lib):
    """Tuning changes the schedule and the grouping of partial sums only."""
    from fft_method_test_gb300.permeability import PermeabilityProblem

    mask = G.gaussian_field(48, 4.0, 0.4, seed=43)
    with PermeabilityProblem(mask.shape, precision="mixed") as p:
        nb = p.set_geometry(mask)
        x = np.random.default_rng(0).uniform(-1, 1, 3 * nb)
        y0 = p.operator_apply(x)
        t = p.autotune()
        y1 = p.operator_apply(x)
        t2 = p.autotune()  # cached
    assert t["tile"] in (4, 8, 16, 32) and t["apply_ms"] > 0
    assert t2["tile"] == t["tile"] and t2["tma"] == t["tma"]
    assert rel_err(y1, y0) < 1e-12


def test_batch_errors(gpu_lib):
    from fft_method_test_gb300.permeability import batch_solve_permeability

    with pytest.raises(ValueError):
        batch_solve_permeability([G.spheres(8, 1.5, 0.6, seed=1)], concurrency=0)
    K, _, status = batch_solve_permeability([], concurrency=2)
    assert K.shape == (0, 3, 3) and status == []


def test_set_tiling_reproduces_the_tuned_apply(gpu_lib):
    """fp_set_tiling with the tuner's report gives the tuned schedule's result."""
    from fft_method_test_gb300.permeability import PermeabilityProblem

    mask = G.gaussian_field(40, 4.0, 0.4, seed=44)
    x = None
    with PermeabilityProblem(mask.shape, precision="mixed") as p:
        nb = p.set_geometry(mask)
        x = np.random.default_rng(1).uniform(-1, 1, 3 * nb)
        t = p.autotune()
        y0 = p.operator_apply(x)
    with PermeabilityProblem(mask.shape, precision="mixed") as q:
        q.set_geometry(mask)
        q.set_tiling(t["tile"], t["tma"], t["x_bulk"], t["x_rows"], t["lowreg"])
        y1 = q.operator_apply(x)
        with pytest.raises(Exception):
            q.set_tiling(7, True, True)
    assert np.array_equal(y0, y1)
