"""GPU parity at the configurations' scale, and against the reference-built
golden fixtures directly.

* Permeability tensors of cells of 64^3 to 160^3 (Gaussian random fields of
  the benchmark's kind, batch cells of edges 96 and 160, the Brinkman cell)
  against the CPU oracle's K, stored in tests/golden/oracle_k.npz by
  tests/golden/make_oracle_k.py (the oracle is pinned bit for bit to the
  reference build).  Both solves stop at a relative MINRES residual of 1e-10;
  K agrees to 1e-9 relative (the solves' own residual level), and to 1e-6 for
  mixed precision at tol 1e-7.
* Operator applies on the specialised passes (edges 32 to 256 with factors
  2, 3, 5) against the oracle (1e-12 FP64, 5e-6 mixed) and against the
  generic passes (FFTPERM_NO_FAST).
* The reference-built fixtures of tests/golden/golden.npz (C1 K, the 16^3
  apply and RHS, the non-cubic Green table) read straight into GPU checks.
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import rel_err
from fft_method_test_gb300 import geometry as G

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_K = os.path.join(HERE, "golden", "oracle_k.npz")
GOLDEN = os.path.join(HERE, "golden", "golden.npz")


def problem(shape, **kw):
    from fft_method_test_gb300.permeability import PermeabilityProblem

    return PermeabilityProblem(shape, **kw)


def fixture_case(name):
    with np.load(ORACLE_K) as z:
        if name + "_K" not in z.files:
            pytest.fail("oracle fixture %s missing from %s" % (name, ORACLE_K))
        shape = tuple(int(v) for v in z[name + "_shape"])
        bits = z[name + "_mask_bits"]
        mask = np.unpackbits(bits)[: int(np.prod(shape))].reshape(shape).astype(np.uint8)
        sha = str(z[name + "_sha256"])
        assert hashlib.sha256(mask.tobytes()).hexdigest() == sha
        return mask, z[name + "_K"].copy(), float(z[name + "_tol"]), int(z[name + "_nb"])


@pytest.mark.parametrize("name", ["grf64", "grf128", "c4_96_grf", "c4_160_sph", "c2_128_sph"])
def test_permeability_at_scale_matches_oracle(gpu_lib, name):
    mask, K_ref, tol, nb_ref = fixture_case(name)
    with problem(mask.shape, precision="fp64") as p:
        assert p.set_geometry(mask) == nb_ref
        K, st = p.solve_permeability(tol, 20000)
    assert all(s["converged"] for s in st), st
    assert rel_err(K, K_ref) < 1e-9, (name, rel_err(K, K_ref))


@pytest.mark.parametrize("name", ["grf128", "c4_160_sph"])
def test_mixed_permeability_at_scale_within_1e6(gpu_lib, name):
    mask, K_ref, _, _ = fixture_case(name)
    with problem(mask.shape, precision="mixed") as p:
        p.set_geometry(mask)
        p.autotune()
        K, st = p.solve_permeability(1e-7, 20000)
    assert all(s["converged"] for s in st), st
    assert rel_err(K, K_ref) < 1e-6, (name, rel_err(K, K_ref))


@pytest.mark.parametrize("shape", [(32, 32, 32), (64, 64, 64), (128, 128, 128), (64, 32, 128),
                                   (256, 128, 64), (48, 48, 48), (80, 80, 80), (96, 80, 160),
                                   (160, 96, 48)])
def test_specialised_apply_matches_oracle(gpu_lib, restatement, shape):
    """Edges 32, 48, 64, 80, 96, 128, 160 and 256 run the specialised passes
    (radix-12 and radix-20 four-step lines for the edges with a factor 3 or
    5): FP64 apply to 1e-12 and mixed to FP32 accuracy against the oracle."""
    mask = G.gaussian_field(shape, 4.0, 0.4, seed=sum(shape))
    ctx = restatement.context(mask)
    x = np.random.default_rng(5).uniform(-1, 1, 3 * ctx.nb)
    y_ref = ctx.operator_apply(x)
    ctx.close()
    with problem(shape, precision="fp64") as p:
        p.set_geometry(mask)
        y = p.operator_apply(x)
        assert rel_err(y, y_ref) < 1e-12
        p.set_precision("mixed")
        y32 = p.operator_apply(x)
    assert rel_err(y32, y_ref) < 5e-6


@pytest.mark.parametrize("shape", [(64, 128, 64), (160, 48, 96)])
@pytest.mark.parametrize("precision,bar", [("fp64", 1e-13), ("mixed", 2e-6)])
def test_specialised_passes_match_generic(gpu_lib, precision, bar, shape):
    mask = G.gaussian_field(shape, 5.0, 0.35, seed=9)
    x = None
    out = []
    for off in ("0", "1"):
        os.environ["FFTPERM_NO_FAST"] = off
        try:
            with problem(shape, precision=precision) as p:
                nb = p.set_geometry(mask)
                if x is None:
                    x = np.random.default_rng(2).uniform(-1, 1, 3 * nb)
                out.append(p.operator_apply(x))
        finally:
            os.environ.pop("FFTPERM_NO_FAST", None)
    assert rel_err(out[0], out[1]) < bar


def _golden():
    return np.load(GOLDEN)


def _mask_from_bits(bits, n):
    return np.unpackbits(bits)[: n ** 3].reshape(n, n, n).astype(np.uint8)


def test_golden_c1_K_direct(gpu_lib):
    """C1 (32^3 spheres r 4, porosity 0.60, seed 1001, tol 1e-10): the GPU K
    against the K the reference build computed."""
    g = _golden()
    mask = _mask_from_bits(g["c1_mask_bits"], 32)
    with problem(mask.shape) as p:
        p.set_geometry(mask)
        assert np.array_equal(p.support(), g["c1_support"])
        K, st = p.solve_permeability(1e-10, 2000)
    assert rel_err(K, g["c1_K"]) < 1e-10, rel_err(K, g["c1_K"])


def test_golden_op16_apply_and_rhs_direct(gpu_lib):
    g = _golden()
    mask = _mask_from_bits(g["op16_mask_bits"], 16)
    with problem(mask.shape) as p:
        p.set_geometry(mask)
        y = p.operator_apply(g["op16_x"])
        b = p.build_rhs((0.0, 1.0, 0.0))
        avg, _ = p.recover((1.0, 0.0, 0.0), 0.1 * g["op16_x"])
    assert rel_err(y, g["op16_y"]) < 1e-12
    assert rel_err(b, g["op16_rhs_y"]) < 1e-12
    assert rel_err(avg, g["op16_recover_avg"]) < 1e-12


def test_golden_green_3x5x6_direct(gpu_lib):
    g = _golden()
    full = g["green_3x5x6"]  # (6, nz, ny, nx) from the reference, unsymmetrised
    nz, ny, nx = full.shape[1:]
    neg = full[:, (-np.arange(nz)) % nz][:, :, (-np.arange(ny)) % ny][:, :, :, (-np.arange(nx)) % nx]
    want = 0.5 * (full + neg)[:, :, :, : nx // 2 + 1]
    with problem((nz, ny, nx)) as p:
        got = p.green_tensor()
    assert rel_err(got, want) < 1e-13


def test_fgeo_ingested_on_device_matches_host_mask(gpu_lib, tmp_path):
    """fp_load_fgeo (the reference's .fgeo read, the mask formed on the device
    from u16 and u32 ids) gives the support set of fp_set_geometry on the
    same mask, and a wrong size or magic is an argument error."""
    from fft_method_test_gb300._capi import FpError

    mask = G.gaussian_field((24, 20, 16), 3.0, 0.4, seed=77)
    ids16 = np.where(mask != 0, 1, 2).astype(np.uint16)
    f16 = tmp_path / "g16.fgeo"
    G.write_fgeo(str(f16), ids16, ids=True)
    f32 = tmp_path / "g32.fgeo"
    nz, ny, nx = mask.shape
    with open(f32, "wb") as fh:
        fh.write(b"FGEO" + bytes([1, 1, 0, 0]))
        fh.write(np.array([nx, ny, nz], "<u8").tobytes())
        fh.write(np.where(mask != 0, 7, 3).astype("<u4").tobytes())
    with problem(mask.shape) as p:
        nb = p.set_geometry(mask)
        want = p.support()
        assert p.load_fgeo(str(f16), fluid_id=1) == nb
        assert np.array_equal(p.support(), want)
        assert p.load_fgeo(str(f32), fluid_id=7) == nb
        assert np.array_equal(p.support(), want)
    bad = tmp_path / "bad.fgeo"
    bad.write_bytes(b"NOPE" + bytes(28))
    with problem((8, 8, 8)) as p:
        with pytest.raises((ValueError, FpError)):
            p.load_fgeo(str(f16))  # dimensions differ from the grid
        with pytest.raises((ValueError, FpError)):
            p.load_fgeo(str(bad))


def test_velocity_file_written_from_device(gpu_lib, tmp_path):
    """fp_recover_fvel writes the recovered field in the reference's .fvel
    layout, equal to fp_recover's field."""
    from fft_method_test_gb300.permeability import read_fvel

    mask = G.spheres(16, 3.0, 0.6, seed=7)
    with problem(mask.shape) as p:
        nb = p.set_geometry(mask)
        x = np.random.default_rng(1).uniform(-1, 1, 3 * nb)
        _, v = p.recover((1.0, 0.0, 0.0), x, want_field=True)
        path = tmp_path / "v.fvel"
        p.recover_fvel(str(path), (1.0, 0.0, 0.0), x, porosity=0.6, viscosity=1.0)
    d = read_fvel(str(path))
    assert d["velocity"].shape == v.shape
    assert np.array_equal(d["velocity"], v)
    assert d["porosity"] == 0.6 and np.array_equal(d["driving"], [1.0, 0.0, 0.0])
