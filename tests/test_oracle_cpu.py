"""CPU tests of the oracle itself (no GPU).

1. The oracle's CPU FFT against numpy.fft (the contract FFTW gives the reference).
2. The reference's own unit-test assertions (tests/*.cpp of the reference)
   replayed on the C restatement.
3. The C restatement against the reference's own code (oracle/_ref, where it
   was built) and against the committed golden fixtures made from it.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import ROOT, rel_err
from fft_method_test_gb300 import geometry as G

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def unpack(bits, shape):
    return np.unpackbits(bits)[: int(np.prod(shape))].reshape(shape).astype(np.uint8)


# ---------------------------------------------------------------------------
# 1. FFT
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("shape", [(1, 1, 1), (4, 4, 4), (3, 5, 6), (8, 16, 12), (7, 11, 13),
                                   (2, 2, 1), (5, 9, 32)])
@pytest.mark.parametrize("sign", [-1, 1])
def test_cpu_fft_matches_numpy(restatement, shape, sign):
    lib = restatement.lib
    lib.cfft_exec_3d.argtypes = [C.c_int, C.c_int, C.c_int,
                                 np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS"),
                                 C.c_int, C.c_int]
    rng = np.random.default_rng(0)
    z = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    buf = np.ascontiguousarray(np.stack([z.real, z.imag], axis=-1)).ravel()
    lib.cfft_exec_3d(shape[0], shape[1], shape[2], buf, sign, 2)
    got = buf[0::2] + 1j * buf[1::2]
    want = (np.fft.fftn(z) if sign < 0 else np.fft.ifftn(z) * z.size).ravel()
    assert np.abs(got - want).max() <= 1e-13 * max(1.0, np.abs(want).max())


def test_fft_roundtrip(restatement):
    # reference tests/test_fft_roundtrip.cpp: forward + inverse / N = identity (< 1e-9)
    lib = restatement.lib
    n = 64
    data = np.zeros(2 * n)
    data[0::2] = np.arange(n, dtype=np.float64)
    ref = data.copy()
    lib.cfft_exec_3d(4, 4, 4, data, -1, 1)
    lib.cfft_exec_3d(4, 4, 4, data, +1, 1)
    assert np.abs(data / n - ref).max() < 1e-9


# ---------------------------------------------------------------------------
# 2. the reference's unit-test assertions on the restatement
# ---------------------------------------------------------------------------

def test_interface_voxels_kat(restatement):
    # tests/test_interface_voxels.cpp:9-26
    m = np.ones((4, 4, 4), np.uint8)
    m[1:3, 1:3, 1:3] = 0
    s = restatement.support(m)
    assert len(s) == 8 and np.all(np.diff(s) > 0)


def test_support_mapping_kat(restatement):
    # tests/test_support_mapping.cpp:10-40 (FullSolid support of two voxels)
    m = np.ones((4, 4, 4), np.uint8)
    m[1, 1, 1] = 0
    m[2, 2, 2] = 0
    s = restatement.support(m, mode=1)
    assert list(s) == [1 * 16 + 1 * 4 + 1, 2 * 16 + 2 * 4 + 2]


def test_background_force_kat(restatement):
    # tests/test_background_force.cpp:11-39
    m = np.ones((1, 2, 2), np.uint8)
    m[0, 0, 0] = 0
    m[0, 1, 1] = 0
    f0 = restatement.background_force(m, [1.0, 0.0, 0.0], mode=1)
    assert np.allclose(f0[0], -1.0, atol=1e-12, rtol=0)
    assert np.abs(f0[1:]).max() < 1e-12


def test_projector_green_kat(restatement):
    # tests/test_projector_green.cpp:10-48: finite, G(0) = 0
    g = restatement.green_tensor((4, 4, 4))
    assert np.all(np.isfinite(g))
    assert np.abs(g[:, 0, 0, 0]).max() < 1e-15


def test_operator_symmetry(restatement):
    # tests/test_variational_operator_symmetry.cpp:16-61 (bar tightened to FP64)
    m = np.ones((4, 4, 4), np.uint8)
    m[1, 1, 1] = 0
    m[2, 2, 2] = 0
    m[2, 2, 1] = 0
    ctx = restatement.context(m)
    rng = np.random.default_rng(42)
    x = rng.uniform(-1, 1, 3 * ctx.nb)
    y = rng.uniform(-1, 1, 3 * ctx.nb)
    ax, ay = ctx.operator_apply(x), ctx.operator_apply(y)
    gap = abs(x @ ay - ax @ y) / max(1.0, abs(x @ ay), abs(ax @ y), np.sqrt((x @ x) * (y @ y)))
    assert gap < 1e-12


def test_rhs_mean_and_recovery_mean(restatement):
    # tests/test_variational_rhs.cpp:14-46 and tests/test_velocity_recovery.cpp:15-43
    m = np.ones((3, 3, 3), np.uint8)
    m[1, 1, 1] = 0
    m[1, 1, 2] = 0
    ctx = restatement.context(m)
    b1, b2 = ctx.build_rhs([1, 0, 0]), ctx.build_rhs([1, 0, 0])
    assert np.array_equal(b1, b2)
    assert np.abs(b1.reshape(-1, 3).mean(axis=0)).max() < 1e-12
    m = np.ones((4, 4, 4), np.uint8)
    m[1, 1, 1] = 0
    m[2, 2, 2] = 0
    m[2, 1, 2] = 0
    ctx = restatement.context(m)
    n = ctx.nb
    x = np.zeros(3 * n)
    x[0::3] = 0.1 * np.arange(1, n + 1)
    x[1::3] = -0.05 * np.arange(2, n + 2)
    x[2::3] = 0.03 * np.arange(3, n + 3)
    _, v = ctx.recover([1, 0, 0], x, want_field=True)
    sup = restatement.support(m)
    assert np.abs(v.reshape(3, -1)[:, sup].mean(axis=1)).max() < 1e-12
    assert np.all(np.isfinite(v))


def test_small_pipeline(restatement):
    # tests/test_small_permeability_pipeline.cpp:18-56
    m = np.ones((4, 4, 4), np.uint8)
    for k, j, i in [(1, 1, 1), (1, 2, 1), (2, 1, 2), (2, 2, 2)]:
        m[k, j, i] = 0
    ctx = restatement.context(m)
    r = ctx.minres(ctx.build_rhs([1, 0, 0]), 1e-8, 60)
    assert np.isfinite(r["final_rel_residual"]) and len(r["residual_history"]) > 0
    avg, _ = ctx.recover([1, 0, 0], r["solution"])
    assert np.all(np.isfinite(avg))


# ---------------------------------------------------------------------------
# 3. pinning the restatement to the reference
# ---------------------------------------------------------------------------

def test_restatement_matches_golden(restatement, golden):
    m1 = unpack(golden["c1_mask_bits"], (32, 32, 32))
    assert np.array_equal(restatement.support(m1), golden["c1_support"].astype(np.int64))
    m2 = unpack(golden["op16_mask_bits"], (16, 16, 16))
    ctx = restatement.context(m2)
    assert rel_err(ctx.operator_apply(golden["op16_x"]), golden["op16_y"]) < 1e-13
    assert rel_err(ctx.build_rhs([0, 1, 0]), golden["op16_rhs_y"]) < 1e-13
    avg, _ = ctx.recover([1, 0, 0], 0.1 * golden["op16_x"])
    assert rel_err(avg, golden["op16_recover_avg"]) < 1e-11
    g = restatement.green_tensor((3, 5, 6))
    assert rel_err(g, golden["green_3x5x6"]) < 1e-14


def test_restatement_c1_permeability_matches_golden(restatement, golden):
    m1 = unpack(golden["c1_mask_bits"], (32, 32, 32))
    ctx = restatement.context(m1)
    b = ctx.build_rhs([1, 0, 0])
    r = ctx.minres(b, 1e-10, 60)
    h = golden["c1_hist60_x"]
    # single-threaded reference and restatement agree bit for bit
    assert np.max(np.abs(r["residual_history"] - h) / h) < 1e-13
    K, it = ctx.solve_permeability(1e-10, 2000)
    assert rel_err(K, golden["c1_K"]) < 1e-10
    assert np.all(np.abs(it - golden["c1_iters"]) <= 5)


def test_restatement_brinkman_matches_golden(restatement, golden):
    ids = golden["br16_ids"].astype(np.uint32)
    r = restatement.brinkman(ids, 1, 1.0, 1e4, 0.9, 1e-8, 40, (1.0, 0.0, 0.0), want_fields=True)
    assert rel_err(r["U"], golden["br16_U"]) < 1e-12
    assert rel_err(r["ux"], golden["br16_ux"]) < 1e-12
    assert abs(r["residual"] - golden["br16_residual"][0]) <= 1e-12 * golden["br16_residual"][0]


def test_restatement_vs_reference_live(restatement, reference):
    """Where oracle/_ref exists: the restatement equals the reference's code."""
    for shape, seed in [((8, 12, 10), 5), ((16, 16, 16), 7)]:
        m = (np.random.default_rng(seed).random(shape) >= 0.35).astype(np.uint8)
        assert np.array_equal(restatement.support(m), reference.support(m))
        assert np.array_equal(restatement.support(m, 1), reference.support(m, 1))
        a, b = restatement.context(m), reference.context(m)
        x = np.random.default_rng(1).uniform(-1, 1, 3 * a.nb)
        assert rel_err(a.operator_apply(x), b.operator_apply(x)) < 1e-14
        assert np.array_equal(restatement.green_tensor(shape), reference.green_tensor(shape))
        ra, rb = a.minres(a.build_rhs([0, 0, 1]), 1e-10, 50), b.minres(b.build_rhs([0, 0, 1]), 1e-10, 50)
        # the reference's OpenMP dot products reorder sums with the thread
        # count; Lanczos amplifies that round-off after a few dozen steps
        d = np.abs(ra["residual_history"] - rb["residual_history"]) / rb["residual_history"]
        assert np.max(d[:25]) < 1e-9
    ids = G.to_ids(G.spheres(12, 2.5, 0.6, seed=3))
    ra = restatement.brinkman(ids, max_iterations=25, want_fields=True)
    rb = reference.brinkman(ids, max_iterations=25, want_fields=True)
    assert rel_err(ra["ux"], rb["ux"]) < 1e-13 and ra["iterations"] == rb["iterations"]


# ---------------------------------------------------------------------------
# host-side helpers
# ---------------------------------------------------------------------------

def test_geometry_generators_deterministic():
    a = G.spheres(24, 4.0, 0.6, seed=5)
    b = G.spheres(24, 4.0, 0.6, seed=5)
    assert np.array_equal(a, b)
    assert 0.55 < G.porosity(a) <= 0.6
    g = G.gaussian_field(32, 6.0, 0.35, seed=3)
    assert abs(G.porosity(g) - 0.35) < 1e-3


def test_fgeo_roundtrip(tmp_path):
    m = G.spheres(8, 2.0, 0.5, seed=1)
    p = str(tmp_path / "g.fgeo")
    G.write_fgeo(p, m)
    ids = G.read_fgeo(p)
    assert np.array_equal(ids == G.FLUID_ID, m.astype(bool))
    with open(p, "rb") as f:
        raw = f.read()
    assert raw[:4] == b"FGEO" and raw[4] == 1 and raw[5] == 2 and len(raw) == 32 + 2 * m.size


def test_brinkman_fixed_point_oracle_is_where_the_reference_scheme_goes(restatement):
    """The direct KKT solve (oracle/brinkman_kkt.py) satisfies the discrete
    equations, and the reference's own iteration, run longer and longer,
    approaches it (error falls with the iteration count)."""
    import brinkman_kkt as BK

    mask = G.spheres(8, 1.5, 0.6, seed=5)
    ids = G.to_ids(mask)
    k = BK.solve(ids)
    uk = np.array([k["ux"], k["uy"], k["uz"]])
    mom, div = BK.residuals(ids, uk, k["p"])
    assert mom < 1e-10 and div < 1e-9
    import oracle as orc

    checker = orc.Reference() if orc.reference_available() else restatement
    errs = []
    for its in (1000, 5000, 20000):
        o = checker.brinkman(ids, tolerance=1e-30, max_iterations=its, want_fields=True)
        u = np.array([o["ux"], o["uy"], o["uz"]]).reshape(uk.shape)
        errs.append(float(np.abs(u - uk).max()))
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 2e-4


def test_network_restatement_gradients():
    """The CPU restatement of the warm-start network (oracle/nn_ref.py) used
    to check the GPU kernels: its data gradient is the adjoint of its
    convolution, its weight gradient and loss gradient match finite
    differences."""
    import nn_ref as R

    rng = np.random.default_rng(0)
    x = rng.standard_normal((1, 4, 5, 6, 3))
    w = rng.standard_normal((27, 2, 3))
    y = rng.standard_normal((1, 4, 5, 6, 2))
    for dil in (1, 2):
        lhs = np.sum(R.conv(x, w, dil) * y)
        assert abs(lhs - np.sum(x * R.conv_data_grad(y, w, dil))) < 1e-10 * abs(lhs) + 1e-10
        gw = R.conv_weight_grad(y, x, dil)
        for t, o, i in ((0, 0, 0), (13, 1, 2), (26, 1, 1)):
            e = np.zeros_like(w)
            e[t, o, i] = 1e-6
            fd = (np.sum(R.conv(x, w + e, dil) * y) - np.sum(R.conv(x, w - e, dil) * y)) / 2e-6
            assert abs(fd - gw[t, o, i]) < 1e-6 * max(1.0, abs(fd))
    pred = rng.standard_normal((2, 10, 4))
    sup = rng.random((2, 10)) > 0.3
    tgt = rng.standard_normal((2, 10, 3)) * sup[..., None]
    for b in range(2):
        tgt[b, sup[b]] -= tgt[b, sup[b]].mean(axis=0)
    loss, d = R.loss_grad(pred, tgt, sup)
    e = np.zeros_like(pred)
    e[1, np.flatnonzero(sup[1])[0], 2] = 1e-6
    fd = (R.loss_grad(pred + e, tgt, sup)[0][1] - R.loss_grad(pred - e, tgt, sup)[0][1]) / 2e-6
    assert abs(fd - d[1, np.flatnonzero(sup[1])[0], 2]) < 1e-6
    assert R.bf16(np.array([1.0, 1.0 + 2 ** -9, 3.0])).tolist() == [1.0, 1.0, 3.0]
