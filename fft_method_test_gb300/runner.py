"""Host mirror of the reference's fluid runner over the GPU library.

The reference's ``fft_method`` executable reads a sectioned ``.cfg`` file
(src/app/SimulationConfig.cpp:104-330), loads the geometry
(src/io/VoxelIO.cpp), runs one of two fluid modes with one of two solvers and
writes text results and ``.fvel`` velocity fields
(src/app/PermeabilityRunner.cpp).  This module does the same on top of
:mod:`fft_method_test_gb300.permeability`, with every solve on the GPU:

========================================  ====================================
reference                                 here
========================================  ====================================
SimulationConfig / parseConfigFile        ``SimulationConfig`` /
                                          ``parse_config_file`` /
                                          ``SimulationConfig.from_file``
PermeabilityRunner::run (bignonnet)       ``run`` -> ``run_bignonnet``
run_brinkman                              ``run`` -> ``run_brinkman``
solve_one_direction                       ``solve_one_direction``
velocity_field_output_path(_axis),        same names
text_output_path
========================================  ====================================

Text files are written line for line in the reference's layout, numbers in
C++ stream formatting (default ``%g``; the tensor ``%.6e``).  Two keys have
no reference counterpart and live in a ``[gpu]`` section: ``precision``
(``fp64`` or ``mixed``) and ``autotune`` (pick the FFT tiling before the
solves); plus ``brinkman_method`` = ``jacobi`` (the reference's scheme) or
``fixed_point`` (the FFT-preconditioned solve to the scheme's fixed point).
The reference refuses ``compute_backend = gpu`` for the Brinkman solver
(PermeabilityRunner.cpp:464-468); here every solver runs on the GPU and the
key is read but not used.  Material files are not read: give ``mu`` and
``fluid_id`` in the configuration.
"""
from __future__ import annotations

import os
import re
import time
from dataclasses import dataclass, field

import numpy as np

from . import geometry as G

# ---------------------------------------------------------------------------
# Configuration (src/app/SimulationConfig.hpp, SimulationConfig.cpp)
# ---------------------------------------------------------------------------


@dataclass
class SimulationConfig:
    """Defaults of src/app/SimulationConfig.hpp:22-64, then the [gpu] keys."""
    geometry_file: str = "data/sample_geometry.geom"
    material_file: str = ""
    output_file: str = "output.txt"
    log_file: str = ""
    analysis: str = "fluid"
    fluid_mode: str = "permeability"          # | "pressure_gradient"
    compute_backend: str = "cpu"
    pressure_gradient: tuple = (1.0, 0.0, 0.0)
    support_mode: str = "interface"           # | "fullsolid"
    gradient_mode: str = "all"                # | "x" | "y" | "z"
    mu: float = 1.0
    mu_explicit: bool = False
    fluid_id: int = 1
    fluid_id_explicit: bool = False
    voxel_size: float = 1.0
    tolerance: float = 1e-10
    max_iterations: int = 400
    p_radius: int = 2
    progress_interval: int = 0
    threads: int = 0
    fft_threads: int = 0
    parallel_load_cases: bool = False
    write_velocity_fields: bool = False
    solver: str = "bignonnet"                 # | "brinkman"
    brinkman_solid_penalty: float = 1.0e8
    brinkman_relaxation: float = 0.9
    brinkman_tolerance: float = 1.0e-8
    brinkman_forcing_magnitude: float = 1.0
    brinkman_write_velocity_fields: bool = False
    brinkman_require_single_solid_id: bool = True
    # [gpu] section
    precision: str = "fp64"
    autotune: bool = False
    brinkman_method: str = "jacobi"           # | "fixed_point"

    @classmethod
    def from_file(cls, path: str, **overrides) -> "SimulationConfig":
        """SimulationConfig::from_cli (SimulationConfig.cpp:305-439): the
        --config file (legacy keys first, then the hierarchical sections
        override them), then ``overrides`` (field name -> value, in the place
        of the command-line flags), then ``validate``."""
        cfg = cls()
        m = parse_config_file(path)
        _apply_global(cfg, m)
        _apply_bignonnet(cfg, m, "bignonnet")
        _apply_brinkman(cfg, m, "brinkman")
        if (v := _lookup(m, "analysis", "type")) is not None:
            cfg.analysis = _choice(v, ("fluid", "elastic"), "Invalid analysis type: ")
        _apply_fluid(cfg, m)
        _apply_bignonnet(cfg, m, "fluid.bignonnet")
        _apply_brinkman(cfg, m, "fluid.brinkman")
        _apply_gpu(cfg, m)
        for key, val in overrides.items():
            if not hasattr(cfg, key):
                raise ValueError("Unknown option: " + key)
            setattr(cfg, key, val)
        cfg.validate()
        return cfg

    def validate(self) -> None:
        """The checks that end from_cli (SimulationConfig.cpp:407-436); an
        unset ``fft_threads`` inherits ``threads`` (at least 1)."""
        if self.fft_threads == 0:
            self.fft_threads = self.threads or 1
        if self.analysis != "fluid":
            raise ValueError("analysis must be 'fluid' (other analyses are not implemented yet)")
        if self.solver not in ("bignonnet", "brinkman"):
            raise ValueError("solver must be 'bignonnet' or 'brinkman'")
        if self.fluid_mode == "pressure_gradient" and not any(self.pressure_gradient):
            raise ValueError("pressure_gradient must be non-zero when fluid mode is "
                             "pressure_gradient")
        checks = ((self.mu_explicit and self.mu <= 0.0, "mu must be positive"),
                  (self.voxel_size <= 0.0, "voxel_size must be > 0"),
                  (self.tolerance <= 0.0, "tolerance must be positive"),
                  (self.max_iterations == 0, "max_iterations must be >= 1"),
                  (self.fft_threads <= 0, "fft_threads must be >= 1"),
                  (self.threads < 0, "threads must be >= 0"),
                  (self.p_radius < 0, "p_radius must be >= 0"))
        for bad, msg in checks:
            if bad:
                raise ValueError(msg)


def _trim(s: str) -> str:
    return s.strip(" \t\r\n")


def parse_config_file(path: str) -> dict:
    """parseConfigFile (SimulationConfig.cpp:104-146): '#' or ';' starts a
    comment; ``[section]`` headers (lower-cased); ``key = value`` lines (keys
    lower-cased).  Returns {section: {key: value}}, '' for the global section."""
    try:
        f = open(path)
    except OSError:
        raise RuntimeError("Cannot open config file: " + path) from None
    sections: dict = {}
    section = ""
    with f:
        for line_no, line in enumerate(f.read().split("\n"), start=1):
            line = _trim(G.strip_comment(line))
            if not line:
                continue
            if line[0] == "[":
                close = line.find("]")
                if close < 0:
                    raise RuntimeError("Config line %d: missing closing ']'" % line_no)
                section = _trim(line[1:close]).lower()
                continue
            eq = line.find("=")
            if eq < 0:
                raise RuntimeError("Config line %d: expected key = value" % line_no)
            key, val = _trim(line[:eq]).lower(), _trim(line[eq + 1:])
            if not key or not val:
                raise RuntimeError("Config line %d: empty key or value" % line_no)
            sections.setdefault(section, {})[key] = val
    return sections


def _lookup(m: dict, section: str, key: str):
    return m.get(section, {}).get(key)


_FLOAT = re.compile(r"\s*([+-]?(?:\d+\.?\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?"
                    r"|inf(?:inity)?|nan))", re.IGNORECASE)
_INT = re.compile(r"\s*([+-]?\d+)")


def _stod(v: str) -> float:
    """std::stod: the longest leading decimal number; invalid_argument if none."""
    m = _FLOAT.match(v)
    if not m:
        raise ValueError("stod: no conversion: " + v)
    return float(m.group(1))


def _stoi(v: str) -> int:
    m = _INT.match(v)
    if not m:
        raise ValueError("stoi: no conversion: " + v)
    return int(m.group(1))


def _bool(v: str) -> bool:
    """parseBool (SimulationConfig.cpp:31-34)."""
    return _trim(v).lower() in ("1", "true", "yes", "on")


def _choice(v: str, allowed, msg: str, suffix: str = "") -> str:
    lo = _trim(v).lower()
    if lo not in allowed:
        raise ValueError(msg + v + suffix)
    return lo


def _vector3(v: str, name: str) -> tuple:
    """parseVector3 (SimulationConfig.cpp:67-92): three numbers separated by
    blanks and/or commas, nothing after them."""
    toks = v.replace(",", " ").split()
    try:
        if len(toks) < 3:
            raise ValueError
        xyz = tuple(float(t) for t in toks[:3])
    except ValueError:
        raise ValueError("Invalid %s value: %s. Expected three numbers" % (name, v)) from None
    if len(toks) > 3:
        raise ValueError("Invalid %s value: %s. Expected exactly three numbers" % (name, v))
    return xyz


def _backend(v: str) -> str:
    return _choice(v, ("cpu", "gpu"), "Invalid compute backend: ", ". Use cpu|gpu")


def _apply_global(cfg: SimulationConfig, m: dict) -> None:
    """applyGlobal (SimulationConfig.cpp:160-172)."""
    g = m.get("", {})
    for key in ("geometry_file", "material_file", "output_file", "log_file", "solver"):
        if key in g:
            setattr(cfg, key, g[key])
    if "compute_backend" in g:
        cfg.compute_backend = _backend(g["compute_backend"])
    if "threads" in g:
        cfg.threads = _stoi(g["threads"])
    if "max_iterations" in g:
        cfg.max_iterations = _stoi(g["max_iterations"])
    if "progress_interval" in g:
        cfg.progress_interval = _stoi(g["progress_interval"])
    if "voxel_size" in g:
        cfg.voxel_size = _stod(g["voxel_size"])


def _apply_fluid(cfg: SimulationConfig, m: dict) -> None:
    """applyFluidCommon (SimulationConfig.cpp:181-230)."""
    s = m.get("fluid", {})
    if "mode" in s:
        cfg.fluid_mode = _choice(s["mode"], ("permeability", "pressure_gradient"),
                                 "Invalid fluid analysis mode: ")
    if "solver" in s:
        cfg.solver = s["solver"]
    if "compute_backend" in s:
        cfg.compute_backend = _backend(s["compute_backend"])
    if "pressure_gradient" in s:
        cfg.pressure_gradient = _vector3(s["pressure_gradient"], "fluid.pressure_gradient")
    if "mu" in s:
        cfg.mu, cfg.mu_explicit = _stod(s["mu"]), True
    if "fluid_id" in s:
        cfg.fluid_id, cfg.fluid_id_explicit = _stoi(s["fluid_id"]), True
    if "voxel_size" in s:
        cfg.voxel_size = _stod(s["voxel_size"])
    if "tolerance" in s:
        cfg.tolerance = _stod(s["tolerance"])
        cfg.brinkman_tolerance = cfg.tolerance
    for key in ("max_iterations", "progress_interval", "threads", "fft_threads"):
        if key in s:
            setattr(cfg, key, _stoi(s[key]))
    if "parallel_load_cases" in s:
        cfg.parallel_load_cases = _bool(s["parallel_load_cases"])
    if "write_velocity_fields" in s:
        cfg.write_velocity_fields = _bool(s["write_velocity_fields"])
        cfg.brinkman_write_velocity_fields = cfg.write_velocity_fields


def _apply_bignonnet(cfg: SimulationConfig, m: dict, sec: str) -> None:
    """applyBignonnetSection (SimulationConfig.cpp:232-262)."""
    s = m.get(sec, {})
    if "mu" in s:
        cfg.mu, cfg.mu_explicit = _stod(s["mu"]), True
    if "fluid_id" in s:
        cfg.fluid_id, cfg.fluid_id_explicit = _stoi(s["fluid_id"]), True
    if "tolerance" in s:
        cfg.tolerance = _stod(s["tolerance"])
    if "p_radius" in s:
        cfg.p_radius = _stoi(s["p_radius"])
    if "fft_threads" in s:
        cfg.fft_threads = _stoi(s["fft_threads"])
    if "parallel_load_cases" in s:
        cfg.parallel_load_cases = _bool(s["parallel_load_cases"])
    if "support" in s:
        cfg.support_mode = _choice(s["support"], ("interface", "fullsolid"),
                                   "Invalid support value: ")
    if "gradient" in s:
        cfg.gradient_mode = _choice(s["gradient"], ("x", "y", "z", "all"),
                                    "Invalid %s.gradient value: " % sec, ". Use x|y|z|all")


def _apply_brinkman(cfg: SimulationConfig, m: dict, sec: str) -> None:
    """applyBrinkmanSection (SimulationConfig.cpp:272-289)."""
    s = m.get(sec, {})
    for key, attr in (("solid_penalty", "brinkman_solid_penalty"),
                      ("relaxation", "brinkman_relaxation"),
                      ("tolerance", "brinkman_tolerance"),
                      ("forcing_magnitude", "brinkman_forcing_magnitude")):
        if key in s:
            setattr(cfg, attr, _stod(s[key]))
    if "write_velocity_fields" in s:
        cfg.brinkman_write_velocity_fields = _bool(s["write_velocity_fields"])
        cfg.write_velocity_fields = cfg.brinkman_write_velocity_fields
    if "require_single_solid_id" in s:
        cfg.brinkman_require_single_solid_id = _bool(s["require_single_solid_id"])


def _apply_gpu(cfg: SimulationConfig, m: dict) -> None:
    """The [gpu] section: keys of this library with no reference counterpart."""
    s = m.get("gpu", {})
    if "precision" in s:
        cfg.precision = _choice(s["precision"], ("fp64", "mixed"), "Invalid gpu.precision value: ")
    if "autotune" in s:
        cfg.autotune = _bool(s["autotune"])
    if "brinkman_method" in s:
        cfg.brinkman_method = _choice(s["brinkman_method"], ("jacobi", "fixed_point"),
                                      "Invalid gpu.brinkman_method value: ")


# ---------------------------------------------------------------------------
# Output files (src/app/PermeabilityRunner.cpp:79-160)
# ---------------------------------------------------------------------------


def _cpp_stem(name: str) -> str:
    """std::filesystem::path::stem of a file name."""
    if name in (".", ".."):
        return name
    dot = name.rfind(".")
    return name if dot <= 0 else name[:dot]


def base_output_stem(base_output: str):
    """(parent directory, stem) of the output base; "output.txt" when empty."""
    parent, name = os.path.split(base_output or "output.txt")
    stem = _cpp_stem(name)
    return parent, (stem or "output")


def velocity_field_output_path(base_output: str, suffix: str = "") -> str:
    parent, stem = base_output_stem(base_output)
    name = stem + ".fvel" if not suffix else stem + "_" + suffix + ".fvel"
    return os.path.join(parent, name) if parent else name


def velocity_field_output_path_axis(base_output: str, axis: int) -> str:
    return velocity_field_output_path(base_output, "axis%d" % (axis + 1))


def text_output_path(base_output: str, suffix: str) -> str:
    parent, stem = base_output_stem(base_output)
    name = stem + "_" + suffix + ".txt"
    return os.path.join(parent, name) if parent else name


def _g(x) -> str:
    """A number as a C++ ostream prints it by default (%g, 6 digits)."""
    return "%g" % float(x)


def _write_fvel(path: str, field_, porosity: float, viscosity: float, driving) -> None:
    from .permeability import write_fvel

    parent = os.path.dirname(path)
    if parent:
        os.makedirs(parent, exist_ok=True)
    write_fvel(path, field_, porosity, viscosity, driving)


def _open_text(path: str):
    try:
        return open(path, "w")
    except OSError:
        raise RuntimeError("Cannot open output file: " + path) from None


def _header(cfg: SimulationConfig, shape, title: str, solver: str | None) -> list:
    nz, ny, nx = shape
    lines = ["# FFT_Method " + title]
    if solver:
        lines.append("# solver = " + solver)
    lines += ["# geometry_file = " + cfg.geometry_file,
              "# grid = %d x %d x %d" % (nx, ny, nz),
              "# voxel_size = " + _g(cfg.voxel_size)]
    return lines


def permeability_text(cfg: SimulationConfig, shape, porosity: float, tensor,
                      solver: str | None = None, viscosity: float | None = None) -> str:
    """The ``<stem>_permeability.txt`` file: PermeabilityRunner.cpp:798-815
    (bignonnet: ``mu`` line, no solver line) or :427-442 (brinkman: solver
    and ``viscosity`` lines)."""
    lines = _header(cfg, shape, "permeability result", solver)
    lines.append("# porosity = " + _g(porosity))
    lines.append("# viscosity = " + _g(viscosity) if solver == "brinkman" else "# mu = " + _g(cfg.mu))
    lines += ["#", "# Permeability tensor K (Darcy sign, K > 0):", tensor.to_string()]
    return "\n".join(lines) + "\n"


def pressure_gradient_text(cfg: SimulationConfig, shape, porosity: float, velocity, stats: dict,
                           solver: str = "bignonnet", viscosity: float | None = None) -> str:
    """The ``<stem>_velocity.txt`` file: PermeabilityRunner.cpp:660-684
    (bignonnet) or :361-384 (brinkman)."""
    lines = _header(cfg, shape, "fluid pressure-gradient response", solver)
    lines.append("# porosity = " + _g(porosity))
    if solver == "brinkman":
        lines.append("# viscosity = " + _g(viscosity))
    else:
        lines.append("# mu = " + _g(cfg.mu))
    lines.append("# pressure_gradient = " + " ".join(_g(v) for v in cfg.pressure_gradient))
    lines.append("# macroscopic_velocity = " + " ".join(_g(v) for v in velocity))
    lines.append("# iterations = %d" % stats["iterations"])
    if solver == "brinkman":
        lines.append("# residual = " + _g(stats["residual"]))
    else:
        lines.append("# final_rel_residual = " + _g(stats["final_rel_residual"]))
    lines.append("# converged = " + ("true" if stats["converged"] else "false"))
    return "\n".join(lines) + "\n"


# ---------------------------------------------------------------------------
# Runs
# ---------------------------------------------------------------------------


@dataclass
class DirectionSolveResult:
    """PermeabilityRunner.cpp:65-71."""
    col: int
    stats: dict
    avg_velocity: np.ndarray
    velocity_field: np.ndarray | None = None
    elapsed_seconds: float = 0.0


@dataclass
class RunResult:
    mode: str
    solver: str
    porosity: float
    permeability: np.ndarray | None = None           # 3x3, K[row][col]
    directions: list = field(default_factory=list)   # DirectionSolveResult or Brinkman stats
    velocity: np.ndarray | None = None               # pressure-gradient mode: <v>
    files: list = field(default_factory=list)


def directions_from_mode(mode: str):
    """directions_from_mode (PermeabilityRunner.cpp:48-63): (column, unit gradient)."""
    units = {0: (1.0, 0.0, 0.0), 1: (0.0, 1.0, 0.0), 2: (0.0, 0.0, 1.0)}
    cols = {"x": [0], "y": [1], "z": [2], "all": [0, 1, 2]}[mode]
    return [(c, units[c]) for c in cols]


def solve_one_direction(problem, col: int, grad, tol: float, maxit: int,
                        want_field: bool) -> DirectionSolveResult:
    """solve_one_direction (PermeabilityRunner.cpp:173-242) on a problem whose
    geometry is set: RHS, MINRES from a zero guess, recovery, <v> over the
    domain; the velocity field only when asked (one more Green apply)."""
    t0 = time.perf_counter()
    if want_field:
        _, st, x = problem.solve_load_case(grad, tol, maxit, want_solution=True)
        avg, v = problem.recover(grad, x, want_field=True)
    else:
        avg, st, _ = problem.solve_load_case(grad, tol, maxit)
        v = None
    return DirectionSolveResult(col=col, stats=st, avg_velocity=np.asarray(avg, np.float64),
                                velocity_field=v, elapsed_seconds=time.perf_counter() - t0)


def run_bignonnet(cfg: SimulationConfig, mask: np.ndarray | None = None,
                  problem=None) -> RunResult:
    """PermeabilityRunner::run for solver = bignonnet (PermeabilityRunner.cpp:450-820).

    ``mask`` overrides reading ``cfg.geometry_file``; ``problem`` is a
    :class:`~fft_method_test_gb300.permeability.PermeabilityProblem` whose
    geometry is already set to ``mask`` (default: one is made from ``cfg``
    and closed afterwards)."""
    from .permeability import PermeabilityTensor

    if mask is None:
        mask = G.load_mask(cfg.geometry_file, cfg.fluid_id)
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    por = G.porosity(mask)
    own = problem is None
    if own:
        from .permeability import PermeabilityProblem

        problem = PermeabilityProblem(mask.shape, voxel_size=cfg.voxel_size, mu=cfg.mu,
                                      p_radius=cfg.p_radius, precision=cfg.precision)
    try:
        if own:
            problem.set_geometry(mask, cfg.support_mode)
        if cfg.autotune:
            problem.autotune()
        out = RunResult(mode=cfg.fluid_mode, solver="bignonnet", porosity=por)
        want = cfg.write_velocity_fields
        if cfg.fluid_mode == "pressure_gradient":
            grad = tuple(float(g) for g in cfg.pressure_gradient)
            r = solve_one_direction(problem, 0, grad, cfg.tolerance, cfg.max_iterations, want)
            out.directions.append(r)
            out.velocity = r.avg_velocity
            if want:
                path = velocity_field_output_path(cfg.output_file, "")
                _write_fvel(path, r.velocity_field, por, cfg.mu, grad)
                out.files.append(path)
            if cfg.output_file:
                path = text_output_path(cfg.output_file, "velocity")
                with _open_text(path) as f:
                    f.write(pressure_gradient_text(cfg, mask.shape, por, r.avg_velocity, r.stats))
                out.files.append(path)
            return out
        tensor = PermeabilityTensor()
        for col, grad in directions_from_mode(cfg.gradient_mode):
            r = solve_one_direction(problem, col, grad, cfg.tolerance, cfg.max_iterations, want)
            out.directions.append(r)
            # colK = -mu <v>; set_column stores -colK (PermeabilityRunner.cpp:772-777)
            tensor.set_column(col, -cfg.mu * r.avg_velocity)
            if want:
                path = velocity_field_output_path_axis(cfg.output_file, col)
                _write_fvel(path, r.velocity_field, por, cfg.mu, grad)
                out.files.append(path)
        out.permeability = tensor.data().reshape(3, 3).copy()
        if cfg.output_file:
            path = text_output_path(cfg.output_file, "permeability")
            with _open_text(path) as f:
                f.write(permeability_text(cfg, mask.shape, por, tensor))
            out.files.append(path)
        return out
    finally:
        if own:
            problem.close()


def run_brinkman(cfg: SimulationConfig, ids: np.ndarray | None = None) -> RunResult:
    """run_brinkman (PermeabilityRunner.cpp:250-446) on the GPU Brinkman
    solvers.  ``ids`` (material ids, (nz, ny, nx)) overrides reading
    ``cfg.geometry_file``.  In permeability mode with velocity fields the
    three load cases are solved once more with fields kept, K coming from
    the tensor call."""
    from . import permeability as Pm
    from .permeability import PermeabilityTensor

    if cfg.mu <= 0.0:
        raise RuntimeError("Brinkman solver requires mu > 0; provide --mu or a material_file "
                           "with viscosity")
    if ids is None:
        ids = G.load_ids(cfg.geometry_file)
    ids = np.ascontiguousarray(ids, dtype=np.uint32)
    fixed = cfg.brinkman_method == "fixed_point"
    common = dict(fluid_id=cfg.fluid_id, fluid_mu=cfg.mu, solid_penalty=cfg.brinkman_solid_penalty,
                  tolerance=cfg.brinkman_tolerance, max_iterations=cfg.max_iterations)
    if not fixed:
        common["relaxation"] = cfg.brinkman_relaxation
    solve = Pm.solveBrinkmanFixedPoint if fixed else Pm.solveBrinkman
    want = cfg.write_velocity_fields
    if cfg.fluid_mode == "pressure_gradient":
        force = tuple(-float(g) for g in cfg.pressure_gradient)
        res = solve(ids, force, want_fields=want, **common)
        out = RunResult(mode=cfg.fluid_mode, solver="brinkman", porosity=res["porosity"],
                        directions=[res], velocity=np.asarray(res["superficialVelocity"]))
        if want:
            path = velocity_field_output_path(cfg.output_file, "")
            _write_fvel(path, np.stack([res["ux"], res["uy"], res["uz"]]), res["porosity"],
                        res["viscosity"], force)
            out.files.append(path)
        if cfg.output_file:
            path = text_output_path(cfg.output_file, "velocity")
            with _open_text(path) as f:
                f.write(pressure_gradient_text(cfg, ids.shape, res["porosity"], out.velocity, res,
                                               solver="brinkman", viscosity=res["viscosity"]))
            out.files.append(path)
        return out
    tensor_fn = Pm.computePermeabilityTensorFixedPoint if fixed else Pm.computePermeabilityTensor
    K, stats = tensor_fn(ids, forcing=cfg.brinkman_forcing_magnitude,
                         voxel_size=cfg.voxel_size, **common)
    out = RunResult(mode=cfg.fluid_mode, solver="brinkman", porosity=stats[0]["porosity"],
                    permeability=np.asarray(K), directions=stats)
    if want:
        for axis in range(3):
            force = [0.0, 0.0, 0.0]
            force[axis] = cfg.brinkman_forcing_magnitude
            res = solve(ids, force, want_fields=True, **common)
            path = velocity_field_output_path_axis(cfg.output_file, axis)
            _write_fvel(path, np.stack([res["ux"], res["uy"], res["uz"]]), res["porosity"],
                        res["viscosity"], force)
            out.files.append(path)
    if cfg.output_file:
        tensor = PermeabilityTensor()
        tensor.k = np.asarray(K, np.float64).ravel().copy()
        path = text_output_path(cfg.output_file, "permeability")
        with _open_text(path) as f:
            f.write(permeability_text(cfg, ids.shape, stats[0]["porosity"], tensor,
                                      solver="brinkman", viscosity=stats[0]["viscosity"]))
        out.files.append(path)
    return out


def run(cfg: SimulationConfig) -> RunResult:
    """PermeabilityRunner::run: fluid analysis only, solver by name."""
    if cfg.analysis != "fluid":
        raise RuntimeError("Only fluid analysis is implemented in this version")
    if cfg.material_file:
        raise ValueError("material files are not read here: set mu and fluid_id in the "
                         "configuration")
    if cfg.solver == "brinkman":
        return run_brinkman(cfg)
    if cfg.solver != "bignonnet":
        raise ValueError("Unknown solver: " + cfg.solver)
    return run_bignonnet(cfg)
