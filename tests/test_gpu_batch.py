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
    # mixed precision: the inverse x pass accumulates the output's component
    # sums (its mean removal) in FP32 per thread, so another row count per
    # tile moves the removed mean by FP32 rounding of the mean (~1e-10 of y)
    assert rel_err(y1, y0) < 1e-9


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


# ---- groups: one launch per pass for several problems of one grid ----------

def _group_masks(n):
    return [G.gaussian_field(n, 4.0, 0.4, seed=60 + n),
            G.spheres(n, 3.0, 0.55, seed=61 + n),
            G.gaussian_field(n, 3.0, 0.5, seed=62 + n),
            G.spheres(n, 2.5, 0.7, seed=63 + n)]


def _problems(masks, precision, tiling=None):
    from fft_method_test_gb300.permeability import PermeabilityProblem

    ps = []
    for m in masks:
        p = PermeabilityProblem(m.shape, precision=precision)
        p.set_geometry(m)
        if tiling is not None:
            p.set_tiling(**tiling)
        ps.append(p)
    return ps


@pytest.mark.parametrize("n", [32, 48])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-7)])
def test_group_equals_single_solves(gpu_lib, n, precision, tol):
    """A lockstep group (one launch per pass for all members, members
    converging at different iterations) computes for every member exactly what
    fp_solve_permeability computes for it alone: identical K and iteration
    counts."""
    from fft_method_test_gb300.permeability import group_solve_permeability

    masks = _group_masks(n)
    ps = _problems(masks, precision)
    try:
        Kg, stg = group_solve_permeability(ps, tol, 20000)
    finally:
        for p in ps:
            p.close()
    its = []
    for i, m in enumerate(masks):
        Ks, sts = _single(m, precision, tol, 20000)
        assert np.array_equal(Kg[i], Ks), (i, rel_err(Kg[i], Ks))
        assert [s["iterations"] for s in stg[i]] == [s["iterations"] for s in sts], i
        assert all(s["converged"] for s in stg[i])
        its.append(sum(s["iterations"] for s in sts))
    assert len(set(its)) > 1  # the members did stop at different iterations


def test_group_of_unspecialised_grid_solves_one_by_one(gpu_lib):
    """A grid without specialised passes (40^3) is solved member by member,
    with the same K as the single solves."""
    from fft_method_test_gb300.permeability import group_solve_permeability

    masks = _group_masks(40)[:2]
    ps = _problems(masks, "fp64")
    try:
        Kg, _ = group_solve_permeability(ps, 1e-10)
    finally:
        for p in ps:
            p.close()
    for i, m in enumerate(masks):
        Ks, _ = _single(m, "fp64", 1e-10)
        assert np.array_equal(Kg[i], Ks), i


def test_group_rejects_mixed_grids(gpu_lib):
    from fft_method_test_gb300.permeability import group_solve_permeability

    ps = _problems([_group_masks(32)[0], _group_masks(48)[0]], "fp64")
    try:
        with pytest.raises(ValueError):
            group_solve_permeability(ps, 1e-8)
    finally:
        for p in ps:
            p.close()


def test_group_rejects_different_tilings(gpu_lib):
    from fft_method_test_gb300.permeability import group_solve_permeability

    ps = _problems(_group_masks(32)[:2], "mixed")
    try:
        ps[1].set_tiling(8, True, True, 2, False)
        with pytest.raises(ValueError, match="tiling"):
            group_solve_permeability(ps, 1e-7)
    finally:
        for p in ps:
            p.close()


def test_grouped_batch_equals_ungrouped(gpu_lib):
    """fp_batch_solve_grouped (groups of up to 3 per grid) against the
    ungrouped batch: identical K and iterations; uneven group sizes."""
    from fft_method_test_gb300.permeability import batch_solve_permeability

    masks = _group_masks(32) + _group_masks(48)[:3] + [G.spheres(24, 3.0, 0.6, seed=31)]
    K1, st1, s1 = batch_solve_permeability(masks, precision="mixed", tol=1e-7, concurrency=3,
                                           autotune=True, max_group=1)
    K3, st3, s3 = batch_solve_permeability(masks, precision="mixed", tol=1e-7, concurrency=3,
                                           autotune=True, max_group=3)
    assert s1 == s3 == [0] * len(masks)
    assert np.array_equal(K1, K3)
    assert [[s["iterations"] for s in st] for st in st1] == [[s["iterations"] for s in st] for st in st3]


def test_grouped_batch_fp64_matches_oracle(gpu_lib, restatement):
    from fft_method_test_gb300.permeability import batch_solve_permeability

    masks = _group_masks(32)[:3]
    K, _, status = batch_solve_permeability(masks, precision="fp64", tol=1e-10, maxit=6000,
                                            concurrency=1, autotune=False, max_group=3)
    assert status == [0, 0, 0]
    for i, m in enumerate(masks):
        K_ref, _ = restatement.context(m).solve_permeability(1e-10, 6000)
        assert rel_err(K[i], K_ref) < 1e-9, i


@pytest.mark.parametrize("n,precision,tol", [(32, "fp64", 1e-10), (48, "mixed", 1e-7),
                                             (64, "mixed", 1e-7)])
def test_block_solve_equals_load_cases_one_by_one(gpu_lib, n, precision, tol):
    """fp_solve_permeability_block (three load cases in lockstep, one Green
    table for the three) gives the K and iteration counts of
    fp_solve_permeability exactly."""
    from fft_method_test_gb300.permeability import PermeabilityProblem

    mask = G.gaussian_field(n, 4.0, 0.4, seed=70 + n)
    with PermeabilityProblem(mask.shape, precision=precision) as p:
        p.set_geometry(mask)
        K0, st0 = p.solve_permeability(tol, 20000)
        K1, st1 = p.solve_permeability(tol, 20000, block=True)
        K2, _ = p.solve_permeability(tol, 20000)  # the handle is unchanged after a block solve
    assert np.array_equal(K0, K1), rel_err(K0, K1)
    assert np.array_equal(K0, K2)
    assert [s["iterations"] for s in st0] == [s["iterations"] for s in st1]


def test_block_solve_on_unspecialised_grid(gpu_lib):
    from fft_method_test_gb300.permeability import PermeabilityProblem

    mask = G.gaussian_field(40, 4.0, 0.4, seed=77)
    with PermeabilityProblem(mask.shape, precision="fp64") as p:
        p.set_geometry(mask)
        K0, _ = p.solve_permeability(1e-10, 20000)
        K1, _ = p.solve_permeability(1e-10, 20000, block=True)
    assert np.array_equal(K0, K1)
