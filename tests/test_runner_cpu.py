"""Host logic of the runner mirror (fft_method_test_gb300/runner.py): the .cfg
reader, the geometry readers, the output paths and the text/.fvel files of
both fluid modes and both solvers.  The solves are stood in for by fakes with
a known answer, so nothing here needs a GPU; the same runs on the GPU are in
tests/test_gpu_runner.py."""
import os

import numpy as np
import pytest

from fft_method_test_gb300 import geometry as G
from fft_method_test_gb300 import runner as R
from fft_method_test_gb300.permeability import PermeabilityTensor, read_fvel

# the fakes' permeability: <v> = M grad / mu, so K[row][col] = M[row][col]
M = np.array([[0.5, 0.01, 0.0], [0.01, 0.4, 0.02], [0.0, 0.02, 0.3]])


class FakeProblem:
    """Stands in for PermeabilityProblem with the same call signatures."""

    def __init__(self, shape, mu):
        self.shape, self.mu, self.calls = shape, mu, []

    def solve_load_case(self, grad, tol, maxit, x0=None, want_solution=False):
        self.calls.append(("solve", tuple(grad), tol, maxit, want_solution))
        st = dict(iterations=17, converged=True, final_rel_residual=3.25e-11, seconds=0.0,
                  refinements=0)
        return M @ np.asarray(grad, float) / self.mu, st, (np.ones(6) if want_solution else None)

    def recover(self, grad, x, want_field=False):
        self.calls.append(("recover", tuple(grad), want_field))
        avg = M @ np.asarray(grad, float) / self.mu
        field = np.broadcast_to(avg[:, None, None, None], (3,) + self.shape).copy()
        return avg, (field if want_field else None)

    def autotune(self):
        self.calls.append(("autotune",))
        return {}


def _mask():
    return G.spheres(8, 1.5, 0.6, seed=3)


def test_config_sections_precedence_and_gpu_keys(tmp_path):
    p = tmp_path / "run.cfg"
    p.write_text(
        "# legacy keys\n"
        "geometry_file = data/cell.fgeo   ; trailing comment\n"
        "output_file = out/result.txt\n"
        "max_iterations = 250\n"
        "voxel_size = 2.5e-6\n"
        "[Bignonnet]\n"
        "tolerance = 1e-8\n"
        "p_radius = 1\n"
        "[fluid]\n"
        "mode = Pressure_Gradient\n"
        "pressure_gradient = 0.5, -1 ,2\n"
        "mu = 1.8e-5\n"
        "tolerance = 1e-9\n"
        "write_velocity_fields = yes\n"
        "[fluid.bignonnet]\n"
        "support = FullSolid\n"
        "gradient = y\n"
        "[brinkman]\n"
        "solid_penalty = 1e6\n"
        "relaxation = 0.8\n"
        "[gpu]\n"
        "precision = mixed\n"
        "autotune = on\n"
        "brinkman_method = fixed_point\n"
        "unknown_key = ignored\n")
    c = R.SimulationConfig.from_file(str(p))
    assert c.geometry_file == "data/cell.fgeo" and c.output_file == "out/result.txt"
    assert c.max_iterations == 250 and c.voxel_size == 2.5e-6 and c.p_radius == 1
    assert c.fluid_mode == "pressure_gradient" and c.pressure_gradient == (0.5, -1.0, 2.0)
    assert c.mu == 1.8e-5 and c.mu_explicit
    # [fluid] tolerance overrides the legacy [bignonnet] one and sets Brinkman's too
    assert c.tolerance == 1e-9 and c.brinkman_tolerance == 1e-9
    assert c.support_mode == "fullsolid" and c.gradient_mode == "y"
    assert c.write_velocity_fields and c.brinkman_write_velocity_fields
    assert c.brinkman_solid_penalty == 1e6 and c.brinkman_relaxation == 0.8
    assert c.precision == "mixed" and c.autotune and c.brinkman_method == "fixed_point"
    d = R.SimulationConfig()
    assert (d.tolerance, d.max_iterations, d.p_radius, d.mu) == (1e-10, 400, 2, 1.0)


@pytest.mark.parametrize("text, msg", [
    ("[fluid\nmu = 1\n", "missing closing"),
    ("mu 1\n", "expected key = value"),
    ("mu =\n", "empty key or value"),
    ("[fluid]\ncompute_backend = tpu\n", "Invalid compute backend"),
    ("[fluid]\npressure_gradient = 1 2\n", "Expected three numbers"),
    ("[fluid]\npressure_gradient = 1 2 3 4\n", "exactly three numbers"),
    ("[fluid]\nmode = stress\n", "Invalid fluid analysis mode"),
    ("[bignonnet]\nsupport = all\n", "Invalid support value"),
    ("[bignonnet]\ngradient = w\n", "Use x|y|z|all"),
    ("[gpu]\nprecision = fp16\n", "gpu.precision"),
])
def test_config_errors(tmp_path, text, msg):
    p = tmp_path / "bad.cfg"
    p.write_text(text)
    with pytest.raises((RuntimeError, ValueError), match=msg):
        R.SimulationConfig.from_file(str(p))


def test_config_numbers_parse_like_stod_and_stoi(tmp_path):
    p = tmp_path / "n.cfg"
    p.write_text("max_iterations = 12abc\nvoxel_size = 1.5e-3x\n[bignonnet]\np_radius = 3.7\n")
    c = R.SimulationConfig.from_file(str(p))
    assert (c.max_iterations, c.voxel_size, c.p_radius) == (12, 1.5e-3, 3)
    with pytest.raises(RuntimeError, match="Cannot open config file"):
        R.SimulationConfig.from_file(str(tmp_path / "missing.cfg"))


def test_output_paths_follow_the_reference():
    assert R.text_output_path("out/result.txt", "permeability") == os.path.join(
        "out", "result_permeability.txt")
    assert R.text_output_path("result", "velocity") == "result_velocity.txt"
    assert R.text_output_path("", "velocity") == "output_velocity.txt"
    assert R.text_output_path("a.b.txt", "x") == "a.b_x.txt"
    assert R.text_output_path("out/", "x") == os.path.join("out", "output_x.txt")
    assert R.velocity_field_output_path("/tmp/r.txt") == "/tmp/r.fvel"
    assert R.velocity_field_output_path_axis("r.txt", 0) == "r_axis1.fvel"
    assert R.velocity_field_output_path_axis("r.txt", 2) == "r_axis3.fvel"


def test_tensor_text_is_scientific_six_digits():
    t = PermeabilityTensor()
    for col in range(3):
        t.set_column(col, -M[:, col] * (col + 1))
    s = t.to_string("  ")
    assert s.split("\n")[0] == "5.000000e-01  2.000000e-02  0.000000e+00"
    assert s.split("\n")[1] == "  1.000000e-02  8.000000e-01  6.000000e-02"


def test_geometry_text_reader_and_loader(tmp_path):
    p = tmp_path / "cell.geom"
    p.write_text("# a 3 x 2 x 2 cell\n\n; ids follow\n3 2 2 extra\n"
                 "1 2 1 2 # comment 9 9\n1\n2 2 2 1 1 1 2 7 7\n")
    ids = G.read_geom_text(str(p))
    assert ids.shape == (2, 2, 3)
    assert ids.ravel().tolist() == [1, 2, 1, 2, 1, 2, 2, 2, 1, 1, 1, 2]
    assert G.load_mask(str(p), 2).ravel().tolist() == [0, 1, 0, 1, 0, 1, 1, 1, 0, 0, 0, 1]
    p.write_text("2 2 2\n1 1 1\n")
    with pytest.raises(ValueError, match="insufficient voxel values"):
        G.read_geom_text(str(p))
    p.write_text("# only a comment\n")
    with pytest.raises(ValueError, match="nx ny nz"):
        G.read_geom_text(str(p))
    m = _mask()
    f = tmp_path / "cell.fgeo"
    G.write_fgeo(str(f), m)
    assert np.array_equal(G.load_mask(str(f)), m)


def test_bignonnet_permeability_run_writes_the_reference_files(tmp_path):
    m = _mask()
    cfg = R.SimulationConfig(geometry_file="cell.fgeo", output_file=str(tmp_path / "res.txt"),
                             mu=2.0, tolerance=1e-9, max_iterations=77,
                             write_velocity_fields=True, autotune=True)
    fake = FakeProblem(m.shape, cfg.mu)
    out = R.run_bignonnet(cfg, mask=m, problem=fake)
    # K[row][col] = mu <v_row> for grad e_col
    assert np.allclose(out.permeability, M)
    assert fake.calls[0] == ("autotune",)
    assert ("solve", (1.0, 0.0, 0.0), 1e-9, 77, True) in fake.calls
    por = G.porosity(m)
    txt = open(tmp_path / "res_permeability.txt").read().split("\n")
    assert txt[:8] == ["# FFT_Method permeability result",
                       "# geometry_file = cell.fgeo",
                       "# grid = 8 x 8 x 8",
                       "# voxel_size = 1",
                       "# porosity = %g" % por,
                       "# mu = 2",
                       "#",
                       "# Permeability tensor K (Darcy sign, K > 0):"]
    assert txt[8] == "5.000000e-01  1.000000e-02  0.000000e+00"
    assert txt[10] == "0.000000e+00  2.000000e-02  3.000000e-01" and txt[11] == ""
    for axis in range(3):
        f = read_fvel(str(tmp_path / ("res_axis%d.fvel" % (axis + 1))))
        assert f["porosity"] == por and f["viscosity"] == 2.0
        assert f["driving"].tolist() == [float(axis == c) for c in range(3)]
        assert np.allclose(f["velocity"][:, 0, 0, 0], M[:, axis] / 2.0)
    assert len(out.files) == 4


def test_bignonnet_single_gradient_and_pressure_gradient_modes(tmp_path):
    m = _mask()
    cfg = R.SimulationConfig(gradient_mode="z", output_file="")
    fake = FakeProblem(m.shape, 1.0)
    out = R.run_bignonnet(cfg, mask=m, problem=fake)
    assert [r.col for r in out.directions] == [2] and out.files == []
    assert np.allclose(out.permeability[:, 2], M[:, 2]) and not out.permeability[:, :2].any()
    assert all(c[0] == "solve" and c[4] is False for c in fake.calls)

    cfg = R.SimulationConfig(fluid_mode="pressure_gradient", pressure_gradient=(0.0, 2.0, -1.0),
                             output_file=str(tmp_path / "pg.txt"), write_velocity_fields=True)
    out = R.run_bignonnet(cfg, mask=m, problem=FakeProblem(m.shape, 1.0))
    u = M @ np.array([0.0, 2.0, -1.0])
    assert np.allclose(out.velocity, u) and out.permeability is None
    txt = open(tmp_path / "pg_velocity.txt").read().split("\n")
    assert txt[:2] == ["# FFT_Method fluid pressure-gradient response", "# solver = bignonnet"]
    assert txt[6:12] == ["# mu = 1",
                         "# pressure_gradient = 0 2 -1",
                         "# macroscopic_velocity = %g %g %g" % tuple(u),
                         "# iterations = 17",
                         "# final_rel_residual = 3.25e-11",
                         "# converged = true"]
    f = read_fvel(str(tmp_path / "pg.fvel"))
    assert f["driving"].tolist() == [0.0, 2.0, -1.0]


def test_brinkman_runs_write_the_reference_files(tmp_path, monkeypatch):
    from fft_method_test_gb300 import permeability as Pm

    ids = G.to_ids(_mask())
    seen = {}

    def fake_solve(ids_, force, want_fields=False, **kw):
        seen.setdefault("solve", []).append((tuple(force), want_fields, kw))
        U = M @ np.asarray(force, float)
        out = dict(superficialVelocity=U, iterations=400, converged=False, residual=2.5e-4,
                   porosity=0.6, viscosity=1.5, seconds=0.0)
        if want_fields:
            for c, name in enumerate(("ux", "uy", "uz")):
                out[name] = np.full(ids_.shape, U[c])
            out["p"] = np.zeros(ids_.shape)
        return out

    def fake_tensor(ids_, forcing=1.0, voxel_size=1.0, **kw):
        seen["tensor"] = (forcing, voxel_size, kw)
        st = dict(iterations=400, converged=False, residual=1e-4, porosity=0.6, viscosity=1.5,
                  seconds=0.0)
        return M * voxel_size ** 2, [st] * 3

    monkeypatch.setattr(Pm, "solveBrinkman", fake_solve)
    monkeypatch.setattr(Pm, "computePermeabilityTensor", fake_tensor)
    cfg = R.SimulationConfig(solver="brinkman", fluid_mode="pressure_gradient",
                             pressure_gradient=(1.0, 0.0, 0.0), mu=1.5,
                             output_file=str(tmp_path / "b.txt"), write_velocity_fields=True)
    out = R.run_brinkman(cfg, ids=ids)
    force, want, kw = seen["solve"][0]
    assert force == (-1.0, -0.0, -0.0) and want
    assert kw == dict(fluid_id=1, fluid_mu=1.5, solid_penalty=1e8, tolerance=1e-8,
                      max_iterations=400, relaxation=0.9)
    txt = open(tmp_path / "b_velocity.txt").read().split("\n")
    assert txt[1] == "# solver = brinkman" and txt[5:7] == ["# porosity = 0.6", "# viscosity = 1.5"]
    assert txt[9:12] == ["# iterations = 400", "# residual = 0.00025", "# converged = false"]
    assert read_fvel(str(tmp_path / "b.fvel"))["driving"].tolist() == [-1.0, 0.0, 0.0]

    cfg = R.SimulationConfig(solver="brinkman", voxel_size=2.0, mu=1.5,
                             output_file=str(tmp_path / "k.txt"), write_velocity_fields=True)
    out = R.run_brinkman(cfg, ids=ids)
    assert np.allclose(out.permeability, 4 * M) and seen["tensor"][:2] == (1.0, 2.0)
    txt = open(tmp_path / "k_permeability.txt").read().split("\n")
    assert txt[:3] == ["# FFT_Method permeability result", "# solver = brinkman",
                       "# geometry_file = data/sample_geometry.geom"]
    assert txt[6] == "# viscosity = 1.5" and txt[9] == "2.000000e+00  4.000000e-02  0.000000e+00"
    assert [os.path.basename(f) for f in out.files] == [
        "k_axis1.fvel", "k_axis2.fvel", "k_axis3.fvel", "k_permeability.txt"]


def test_run_dispatch_errors():
    with pytest.raises(RuntimeError, match="Only fluid analysis"):
        R.run(R.SimulationConfig(analysis="elastic"))
    with pytest.raises(ValueError, match="material files"):
        R.run(R.SimulationConfig(material_file="mats.txt"))
    with pytest.raises(ValueError, match="Unknown solver"):
        R.run(R.SimulationConfig(solver="lbm"))


def test_reference_config_test_cases(tmp_path):
    """The assertions of the reference's tests/test_simulation_config.cpp,
    command-line flags given as overrides."""
    legacy = tmp_path / "legacy.cfg"
    legacy.write_text("solver = brinkman\nthreads = 4\nmax_iterations = 321\n"
                      "geometry_file = examples/sample_inputs/geometry.geom\n\n"
                      "[bignonnet]\nfft_threads = 0\n\n[brinkman]\ntolerance = 1e-6\n")
    c = R.SimulationConfig.from_file(str(legacy))
    assert c.solver == "brinkman" and c.threads == 4 and c.fft_threads == 4
    assert c.max_iterations == 321 and c.brinkman_tolerance == 1e-6
    c = R.SimulationConfig.from_file(str(legacy), threads=6, fft_threads=2)
    assert c.threads == 6 and c.fft_threads == 2

    schema = tmp_path / "schema.cfg"
    schema.write_text("solver = bignonnet\n\n[analysis]\ntype = fluid\n\n[fluid]\n"
                      "mode = pressure_gradient\nsolver = brinkman\ncompute_backend = gpu\n"
                      "pressure_gradient = 0.0, 2.5, -1.0\nthreads = 3\nfft_threads = 0\n"
                      "write_velocity_fields = true\nmax_iterations = 120\ntolerance = 2e-7\n\n"
                      "[fluid.brinkman]\ntolerance = 3e-7\nforcing_magnitude = 4.0\n")
    c = R.SimulationConfig.from_file(str(schema))
    assert c.analysis == "fluid" and c.fluid_mode == "pressure_gradient"
    assert c.solver == "brinkman" and c.compute_backend == "gpu"
    assert c.threads == 3 and c.fft_threads == 3 and c.write_velocity_fields
    assert c.max_iterations == 120 and c.tolerance == 2e-7
    assert c.brinkman_tolerance == 3e-7 and c.brinkman_forcing_magnitude == 4.0
    assert c.pressure_gradient == (0.0, 2.5, -1.0)
    c = R.SimulationConfig.from_file(str(schema), fluid_mode="permeability", solver="bignonnet",
                                     compute_backend="cpu")
    assert (c.fluid_mode, c.solver, c.compute_backend) == ("permeability", "bignonnet", "cpu")

    bad = tmp_path / "bad.cfg"
    bad.write_text("[analysis]\ntype = fluid\n\n[fluid]\nmode = pressure_gradient\n"
                   "pressure_gradient = 0, 0, 0\n")
    with pytest.raises(ValueError, match="non-zero"):
        R.SimulationConfig.from_file(str(bad))
    bad.write_text("[analysis]\ntype = elastic\n")
    with pytest.raises(ValueError, match="analysis must be 'fluid'"):
        R.SimulationConfig.from_file(str(bad))


@pytest.mark.parametrize("body, msg", [
    ("solver = lbm\n", "solver must be"),
    ("[fluid]\nmu = 0\n", "mu must be positive"),
    ("voxel_size = -1\n", "voxel_size must be > 0"),
    ("[fluid]\ntolerance = 0\n", "tolerance must be positive"),
    ("max_iterations = 0\n", "max_iterations must be >= 1"),
    ("threads = -2\n", "fft_threads must be >= 1"),   # inherits threads first
    ("threads = -2\n[bignonnet]\nfft_threads = 2\n", "threads must be >= 0"),
    ("[bignonnet]\np_radius = -1\n", "p_radius must be >= 0"),
])
def test_config_validation(tmp_path, body, msg):
    p = tmp_path / "v.cfg"
    p.write_text(body)
    with pytest.raises(ValueError, match=msg):
        R.SimulationConfig.from_file(str(p))


def test_reference_voxelio_test_cases(tmp_path):
    """The assertions of the reference's tests/test_voxelio_load_geometry.cpp."""
    import struct

    t = tmp_path / "geometry.geom"
    t.write_text("# comment\n2 2 1\n0 5\n9 0\n")
    ids = G.load_ids(str(t))
    assert ids.shape == (1, 2, 2) and ids.ravel().tolist() == [0, 5, 9, 0]
    f = tmp_path / "geometry.fgeo"
    f.write_bytes(b"FGEO" + bytes([1, 2, 0, 0]) + struct.pack("<3Q", 2, 2, 1)
                  + struct.pack("<4H", 1, 7, 9, 1))
    ids = G.load_ids(str(f))
    assert ids.shape == (1, 2, 2) and ids.ravel().tolist() == [1, 7, 9, 1]
