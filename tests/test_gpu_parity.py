"""GPU parity of the variational hot path against the CPU oracle (FP64).

Every call goes through the C ABI (include/fftperm.h) via the reference-named
Python mirror.  Tolerances: support sets bit-exact; Green table 1e-13
relative; single operator applies 1e-12 relative; K 1e-10 relative
(Frobenius-max), the parity bar of the FP64 path.
"""
import numpy as np
import pytest

from conftest import rel_err
from fft_method_test_gb300 import geometry as G

pytestmark = pytest.mark.gpu


def problem(shape, **kw):
    from fft_method_test_gb300.permeability import PermeabilityProblem

    return PermeabilityProblem(shape, **kw)


def random_mask(shape, frac_solid, seed):
    rng = np.random.default_rng(seed)
    return (rng.random(shape) >= frac_solid).astype(np.uint8)


GEOMS = [
    ("block4", None),
    ("rand3x5x6", None),
    ("sph16", None),
    ("rand8x12x10", None),
]


def make_geom(name):
    if name == "block4":
        m = np.ones((4, 4, 4), np.uint8)
        m[1:3, 1:3, 1:3] = 0
        return m
    if name == "rand3x5x6":
        return random_mask((3, 5, 6), 0.4, 3)
    if name == "rand8x12x10":
        return random_mask((8, 12, 10), 0.35, 5)
    if name == "sph16":
        return G.spheres(16, 3.0, 0.6, seed=7)
    raise KeyError(name)


@pytest.mark.parametrize("name", [g[0] for g in GEOMS])
@pytest.mark.parametrize("mode", ["interface", "fullsolid"])
def test_support_bit_exact(gpu_lib, restatement, name, mode):
    mask = make_geom(name)
    with problem(mask.shape) as p:
        nb = p.set_geometry(mask, mode)
        sup = p.support()
    ref = restatement.support(mask, 0 if mode == "interface" else 1)
    assert nb == len(ref)
    assert np.array_equal(sup, ref)
    assert np.all(np.diff(sup) > 0)


def test_interface_voxels_kat(gpu_lib):
    # tests/test_interface_voxels.cpp: 2x2x2 solid block in 4^3 -> 8 interface voxels, sorted
    mask = make_geom("block4")
    with problem(mask.shape) as p:
        assert p.set_geometry(mask) == 8
        s = p.support()
    assert len(s) == 8 and np.all(np.diff(s) > 0)


def test_support_c1_bit_exact(gpu_lib, restatement):
    mask = G.spheres(32, 4.0, 0.60, seed=1001)
    with problem(mask.shape) as p:
        p.set_geometry(mask)
        sup = p.support()
    assert np.array_equal(sup, restatement.support(mask))


@pytest.mark.parametrize("shape", [(4, 4, 4), (3, 5, 6), (8, 6, 10), (16, 16, 16), (5, 4, 3)])
def test_green_table_matches_symmetrised_oracle(gpu_lib, restatement, shape):
    nz, ny, nx = shape
    g_full = restatement.green_tensor(shape)  # (6, nz, ny, nx), unsymmetrised
    neg = g_full[:, (-np.arange(nz)) % nz][:, :, (-np.arange(ny)) % ny][:, :, :, (-np.arange(nx)) % nx]
    gs = 0.5 * (g_full + neg)[:, :, :, : nx // 2 + 1]
    with problem(shape) as p:
        gt = p.green_tensor()
    assert rel_err(gt, gs) < 1e-13


@pytest.mark.parametrize("shape", [(4, 4, 4), (3, 5, 6), (16, 16, 16), (2, 2, 1), (1, 1, 8)])
def test_green_apply_matches_oracle(gpu_lib, restatement, shape):
    rng = np.random.default_rng(1)
    f = rng.uniform(-1, 1, (3,) + shape)
    mask = np.ones(shape, np.uint8)
    ctx = restatement.context(mask)
    # Green apply through the oracle's context on a dense field
    import oracle as orc  # noqa: F401
    u_ref = _oracle_green_apply(restatement, f)
    with problem(shape) as p:
        u = p.green_apply(f)
    assert rel_err(u, u_ref) < 1e-12
    del ctx


def _oracle_green_apply(restatement, f):
    import ctypes as C

    lib = restatement.lib
    shape = f.shape[1:]
    nz, ny, nx = shape
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    lib.orc_green_apply.argtypes = [C.c_void_p, dp, dp]
    ctx = restatement.context(np.ones(shape, np.uint8))
    u = np.zeros(f.size)
    lib.orc_green_apply(ctx.ptr, np.ascontiguousarray(f).ravel(), u)
    return u.reshape(f.shape)


@pytest.mark.parametrize("name", ["block4", "rand3x5x6", "sph16", "rand8x12x10"])
def test_operator_apply_matches_oracle(gpu_lib, restatement, name):
    mask = make_geom(name)
    ctx = restatement.context(mask)
    rng = np.random.default_rng(42)
    x = rng.uniform(-1, 1, 3 * ctx.nb)
    y_ref = ctx.operator_apply(x)
    with problem(mask.shape) as p:
        p.set_geometry(mask)
        y = p.operator_apply(x)
    assert rel_err(y, y_ref) < 1e-12


def test_operator_symmetry(gpu_lib):
    # tests/test_variational_operator_symmetry.cpp (seeded vectors), FP64 bar 1e-12
    mask = np.ones((4, 4, 4), np.uint8)
    mask[1, 1, 1] = 0
    mask[2, 2, 2] = 0
    mask[2, 2, 1] = 0
    with problem(mask.shape) as p:
        nb = p.set_geometry(mask)
        rng = np.random.default_rng(42)
        x = rng.uniform(-1, 1, 3 * nb)
        y = rng.uniform(-1, 1, 3 * nb)
        ax, ay = p.operator_apply(x), p.operator_apply(y)
    gap = abs(x @ ay - ax @ y) / max(1.0, abs(x @ ay), abs(ax @ y), np.sqrt((x @ x) * (y @ y)))
    assert gap < 1e-12


def test_background_force_kat(gpu_lib):
    # tests/test_background_force.cpp: 2x2x1 checkerboard, FullSolid: f0_x = -1 everywhere
    mask = np.ones((1, 2, 2), np.uint8)
    mask[0, 0, 0] = 0
    mask[0, 1, 1] = 0
    with problem(mask.shape) as p:
        p.set_geometry(mask, "fullsolid")
        f0 = p.background_force([1.0, 0.0, 0.0])
    assert np.allclose(f0[0], -1.0, atol=1e-12, rtol=0)
    assert np.allclose(f0[1:], 0.0, atol=1e-12, rtol=0)


@pytest.mark.parametrize("name", ["rand3x5x6", "sph16"])
def test_background_force_matches_oracle(gpu_lib, restatement, name):
    mask = make_geom(name)
    with problem(mask.shape) as p:
        p.set_geometry(mask)
        f0 = p.background_force([0.3, -1.0, 2.0])
    ref = restatement.background_force(mask, [0.3, -1.0, 2.0])
    assert rel_err(f0, ref) < 1e-15


@pytest.mark.parametrize("name", ["rand3x5x6", "sph16"])
def test_rhs_matches_oracle(gpu_lib, restatement, name):
    mask = make_geom(name)
    ctx = restatement.context(mask)
    with problem(mask.shape) as p:
        p.set_geometry(mask)
        for g in ([1, 0, 0], [0, 1, 0], [0.2, -0.5, 1.0]):
            b = p.build_rhs(g)
            assert rel_err(b, ctx.build_rhs(g)) < 1e-12
            # tests/test_variational_rhs.cpp: per-component support mean ~ 0
            assert np.abs(b.reshape(-1, 3).mean(axis=0)).max() < 1e-12 * np.abs(b).max()


def test_recovery_matches_oracle(gpu_lib, restatement):
    mask = make_geom("sph16")
    ctx = restatement.context(mask)
    rng = np.random.default_rng(9)
    x = rng.uniform(-0.1, 0.1, 3 * ctx.nb)
    avg_ref, v_ref = ctx.recover([1, 0, 0], x, want_field=True)
    with problem(mask.shape) as p:
        p.set_geometry(mask)
        avg, v = p.recover([1, 0, 0], x, want_field=True)
        sup = p.support()
    assert rel_err(v.ravel(), v_ref) < 1e-12
    assert rel_err(avg, avg_ref) < 1e-10
    # tests/test_velocity_recovery.cpp: zero support mean
    assert np.abs(v.reshape(3, -1)[:, sup].mean(axis=1)).max() < 1e-12 * np.abs(v).max()


def test_minres_history_matches_oracle(gpu_lib, restatement):
    mask = make_geom("sph16")
    ctx = restatement.context(mask)
    b = ctx.build_rhs([1, 0, 0])
    r_ref = ctx.minres(b, 1e-10, 60)
    with problem(mask.shape) as p:
        p.set_geometry(mask)
        r = p.minres(b, 1e-10, 60)
    h, hr = r.residual_history, r_ref["residual_history"]
    assert len(h) == len(hr) == 61
    # Lanczos amplifies round-off differences (summation order) after a few
    # dozen steps, exactly as the reference does between thread counts
    assert np.max(np.abs(h[:25] - hr[:25]) / hr[:25]) < 1e-9
    r25 = p_solution_after(mask, b, 25)
    assert rel_err(r25, ctx.minres(b, 1e-10, 25)["solution"]) < 1e-9


def p_solution_after(mask, b, iters):
    with problem(mask.shape) as p:
        p.set_geometry(mask)
        return p.minres(b, 1e-10, iters).solution


def test_minres_warm_start_and_edge_cases(gpu_lib, restatement):
    mask = make_geom("sph16")
    ctx = restatement.context(mask)
    b = ctx.build_rhs([0, 0, 1])
    with problem(mask.shape) as p:
        p.set_geometry(mask)
        # zero rhs -> converged at once with history [0] (MinresSolver.cpp:76-82)
        r0 = p.minres(np.zeros_like(b), 1e-10, 10)
        assert r0.converged and r0.iterations == 0 and np.all(r0.solution == 0)
        # maxit = 0 -> no iteration
        rz = p.minres(b, 1e-10, 0)
        assert rz.iterations == 0 and not rz.converged
        # warm start from a partial solution matches the oracle's warm start
        xw = ctx.minres(b, 1e-10, 20)["solution"]
        r = p.minres(b, 1e-10, 20, x0=xw)
        rr = ctx.minres(b, 1e-10, 20, x0=xw)
        assert np.max(np.abs(r.residual_history - rr["residual_history"]) / rr["residual_history"]) < 1e-8
        with pytest.raises(ValueError):
            p.minres(b, -1.0, 10)
        with pytest.raises(ValueError):
            p.minres(b[:-3], 1e-10, 10)


def test_permeability_c1_matches_oracle(gpu_lib, restatement):
    """32^3 spheres r=4, porosity 0.60, seed 1001, tol 1e-10: K to 1e-10."""
    mask = G.spheres(32, 4.0, 0.60, seed=1001)
    ctx = restatement.context(mask)
    K_ref, it_ref = ctx.solve_permeability(1e-10, 2000)
    with problem(mask.shape) as p:
        p.set_geometry(mask)
        K, stats = p.solve_permeability(1e-10, 2000)
    assert all(s["converged"] for s in stats)
    assert rel_err(K, K_ref) < 1e-10, (K, K_ref)
    # iteration counts move with summation order (the reference's own count
    # shifts with its OpenMP thread count); K is the parity quantity
    for s, ir in zip(stats, it_ref):
        assert abs(s["iterations"] - ir) <= max(5, 0.05 * ir)


def test_errors(gpu_lib):
    from fft_method_test_gb300._capi import FpError

    with pytest.raises(ValueError):
        problem((4, 4, 4), mu=0.0)
    with pytest.raises(ValueError):
        problem((0, 4, 4))
    with pytest.raises(FpError):
        problem((7, 4, 4))  # edge 7 is not a product of 2, 3, 5
    with problem((4, 4, 4)) as p:
        with pytest.raises(FpError):
            p.operator_apply(np.zeros(0))  # no geometry yet: state error from the C ABI
        with pytest.raises(ValueError):
            p.set_geometry(np.ones((4, 4, 5), np.uint8))
        # all-fluid medium -> empty support -> state error on the solve paths
        assert p.set_geometry(np.ones((4, 4, 4), np.uint8)) == 0
        with pytest.raises(FpError):
            p.build_rhs([1, 0, 0])


@pytest.mark.parametrize("shape", [(4, 4, 4), (3, 5, 6), (16, 16, 16), (2, 2, 1), (1, 1, 8), (6, 10, 9)])
def test_fft_forward_inverse_match_numpy(gpu_lib, shape):
    """IFFTBackend-level entry points: unnormalised forward R2C and the
    1/N-scaled real inverse, against numpy's FFT (the FFTW contract)."""
    rng = np.random.default_rng(4)
    f = rng.uniform(-1, 1, (3,) + shape)
    with problem(shape) as p:
        hs = p.fft_forward(f)
        want = np.fft.rfftn(f, axes=(1, 2, 3))
        assert np.abs(hs - want).max() < 1e-13 * np.abs(want).max()
        back = p.fft_inverse(hs)
        assert rel_err(back, f) < 1e-13
        # inverse keeps Re(IFFT) of a non-Hermitian spectrum: use its Hermitian part
        z = rng.standard_normal((3,) + shape) + 1j * rng.standard_normal((3,) + shape)
        neg = np.conj(z[:, (-np.arange(shape[0])) % shape[0]][:, :, (-np.arange(shape[1])) % shape[1]]
                      [:, :, :, (-np.arange(shape[2])) % shape[2]])
        herm = 0.5 * (z + neg)[:, :, :, : shape[2] // 2 + 1]
        re = np.fft.ifftn(z, axes=(1, 2, 3)).real
        assert rel_err(p.fft_inverse(herm), re) < 1e-12


def test_mixed_precision_apply_accuracy(gpu_lib, restatement):
    """FP32 FFT / Green / scatter-gather: a single apply within FP32 accuracy."""
    mask = make_geom("sph16")
    ctx = restatement.context(mask)
    x = np.random.default_rng(3).uniform(-1, 1, 3 * ctx.nb)
    with problem(mask.shape, precision="mixed") as p:
        p.set_geometry(mask)
        y = p.operator_apply(x)
    assert rel_err(y, ctx.operator_apply(x)) < 5e-6


def test_mixed_precision_permeability_within_1e6(gpu_lib, restatement):
    """Mixed precision (FP32 operator inside FP64 iterative refinement): K
    within 1e-6 of the FP64 oracle's K (tol 1e-10), and every load case
    converged on its FP64 residual."""
    mask = G.spheres(32, 4.0, 0.60, seed=1001)
    K_ref, _ = restatement.context(mask).solve_permeability(1e-10, 2000)
    with problem(mask.shape, precision="mixed") as p:
        p.set_geometry(mask)
        K, stats = p.solve_permeability(1e-7, 4000)
    assert rel_err(K, K_ref) < 1e-6, rel_err(K, K_ref)
    for s in stats:
        assert s["converged"] and s["final_rel_residual"] <= 1e-7, stats


def test_mixed_precision_minres_reaches_fp64_tolerance(gpu_lib, restatement):
    """Mixed mode reaches a tolerance far below the FP32 operator's accuracy:
    the returned iterate's residual, recomputed by the FP64 oracle, is below
    tol and equals the reported one."""
    mask = make_geom("sph16")
    ctx = restatement.context(mask)
    tol = 1e-10
    with problem(mask.shape, precision="mixed") as p:
        p.set_geometry(mask)
        b = p.build_rhs((1.0, 0.0, 0.0))
        r = p.minres(b, tol, 4000)
    assert r.converged, r.final_rel_residual
    true_rel = np.linalg.norm(b - ctx.operator_apply(r.solution)) / np.linalg.norm(b)
    assert true_rel <= 1.05 * tol, true_rel
    assert abs(true_rel - r.final_rel_residual) <= 0.05 * tol


def test_largest_grid_512_apply_properties(gpu_lib):
    """At 512^3 (134 M voxels, beyond any oracle run): the FP64 operator is
    symmetric to round-off, the mixed (FP32) apply agrees with it to FP32
    accuracy, and the RHS has zero mean per component."""
    from fft_method_test_gb300.permeability import PermeabilityProblem

    n = 512
    z, y, x = np.ogrid[:n, :n, :n]
    field = (np.sin(2 * np.pi * x / 64) * np.sin(2 * np.pi * y / 128 + 0.3)
             + np.sin(2 * np.pi * z / 80) * np.cos(2 * np.pi * x / 128))
    mask = (field < 0.4).astype(np.uint8)
    del field
    rng = np.random.default_rng(7)
    with PermeabilityProblem(mask.shape, precision="fp64") as p:
        nb = p.set_geometry(mask)
        a = rng.uniform(-1, 1, 3 * nb)
        b = rng.uniform(-1, 1, 3 * nb)
        Aa = p.operator_apply(a)
        Ab = p.operator_apply(b)
        assert abs(a @ Ab - b @ Aa) < 1e-11 * np.abs(a) @ np.abs(Ab)
        rhs = p.build_rhs((0.0, 0.0, 1.0)).reshape(-1, 3)
        assert np.abs(rhs.mean(axis=0)).max() < 1e-12 * np.abs(rhs).max()
        p.set_precision("mixed")
        Aa32 = p.operator_apply(a)
    assert rel_err(Aa32, Aa) < 5e-6


@pytest.mark.parametrize("p_radius,h,mu,support", [(0, 1.0, 1.0, "interface"),
                                                   (1, 0.5, 2.0, "interface"),
                                                   (3, 1.0, 1.0, "interface"),
                                                   (2, 1.0, 1.0, "fullsolid")])
def test_permeability_variants_match_oracle(gpu_lib, restatement, p_radius, h, mu, support):
    """The reference's other choices (alias radius p_radius of the Green sum,
    voxel size, viscosity, FullSolid support): K within 1e-10 of the oracle."""
    mask = G.spheres((12, 15, 16), 2.5, 0.6, seed=21)
    mode = 0 if support == "interface" else 1
    K_ref, _ = restatement.context(mask, h=h, mu=mu, p_radius=p_radius,
                                   mode=mode).solve_permeability(1e-11, 4000)
    with problem(mask.shape, voxel_size=h, mu=mu, p_radius=p_radius) as p:
        p.set_geometry(mask, support)
        K, st = p.solve_permeability(1e-11, 4000)
    assert all(s["converged"] for s in st)
    assert rel_err(K, K_ref) < 1e-9, rel_err(K, K_ref)
