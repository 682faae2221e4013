"""The runner mirror end to end on the GPU: a .cfg file and a .fgeo geometry
in, the reference's text and .fvel files out, with the numbers equal to the
ones the problem-level API gives for the same solves."""
import numpy as np
import pytest

from conftest import rel_err
from fft_method_test_gb300 import geometry as G
from fft_method_test_gb300 import runner as R
from fft_method_test_gb300.permeability import (PermeabilityProblem, computePermeabilityTensor,
                                                read_fvel)

pytestmark = pytest.mark.gpu


def _case(tmp_path, body):
    m = G.spheres(16, 2.5, 0.6, seed=11)
    geo = tmp_path / "cell.fgeo"
    G.write_fgeo(str(geo), m)
    cfg = tmp_path / "run.cfg"
    cfg.write_text("geometry_file = %s\noutput_file = %s\n" % (geo, tmp_path / "res.txt") + body)
    return m, R.SimulationConfig.from_file(str(cfg))


def test_permeability_run_matches_the_problem_api(gpu_lib, tmp_path):
    m, cfg = _case(tmp_path, "[bignonnet]\ntolerance = 1e-10\n[fluid]\nmax_iterations = 3000\n"
                             "write_velocity_fields = true\n")
    out = R.run(cfg)
    with PermeabilityProblem(m.shape) as p:
        p.set_geometry(m)
        K, stats = p.solve_permeability(1e-10, 3000)
    assert all(s["converged"] for s in stats)
    # both solves stop at a relative residual of 1e-10
    assert rel_err(out.permeability, K) < 1e-9
    txt = open(tmp_path / "res_permeability.txt").read().split("\n")
    Kr = out.permeability
    assert txt[8:11] == ["  ".join("%.6e" % Kr[r, c] for c in range(3)) for r in range(3)]
    for axis in range(3):
        f = read_fvel(str(tmp_path / ("res_axis%d.fvel" % (axis + 1))))
        # the field's domain average is the <v> that K came from (mu = 1)
        assert rel_err(f["velocity"].reshape(3, -1).mean(axis=1), Kr[:, axis]) < 1e-10


def test_pressure_gradient_run_matches_the_problem_api(gpu_lib, tmp_path):
    m, cfg = _case(tmp_path, "[fluid]\nmode = pressure_gradient\npressure_gradient = 0.3 -1 0.5\n"
                             "tolerance = 1e-10\nmax_iterations = 3000\n[gpu]\nprecision = mixed\n")
    out = R.run(cfg)
    with PermeabilityProblem(m.shape, precision="mixed") as p:
        p.set_geometry(m)
        avg, st, _ = p.solve_load_case((0.3, -1.0, 0.5), 1e-10, 3000)
    assert st["converged"] and out.directions[0].stats["converged"]
    assert rel_err(out.velocity, avg) < 1e-8
    txt = open(tmp_path / "res_velocity.txt").read().split("\n")
    assert txt[7] == "# pressure_gradient = 0.3 -1 0.5"
    assert txt[8] == "# macroscopic_velocity = %g %g %g" % tuple(out.velocity)


def test_brinkman_run_matches_the_tensor_call(gpu_lib, tmp_path):
    m, cfg = _case(tmp_path, "solver = brinkman\nmax_iterations = 40\n[brinkman]\n"
                             "solid_penalty = 1e4\n")
    out = R.run(cfg)
    K, stats = computePermeabilityTensor(G.to_ids(m), solid_penalty=1e4, max_iterations=40)
    # the same 40 Jacobi iterations per load case
    assert rel_err(out.permeability, K) < 1e-12
    txt = open(tmp_path / "res_permeability.txt").read().split("\n")
    assert txt[1] == "# solver = brinkman"
