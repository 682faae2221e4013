"""Python host mirror of the reference's operator/solver interfaces, over the
C ABI (include/fftperm.h).  Names, argument meaning and errors follow the
reference so that a test written against the reference reads the same here:

=====================================  ==========================================
reference (C++)                        here
=====================================  ==========================================
ForceSupport (ForceSupport.cpp:9-25)   ``PermeabilityProblem.set_geometry`` /
                                       ``ForceSupport``
BackgroundForce::build                 ``BackgroundForce.build``
GreenOperator::apply                   ``GreenOperator.apply``
VariationalOperator (ILinearOperator)  ``VariationalOperator.size`` / ``.apply``
VariationalRHS::build                  ``VariationalRHS.build``
MinresSolver::solve -> SolverResult    ``MinresSolver.solve`` -> ``SolverResult``
VelocityRecovery::recover              ``VelocityRecovery.recover`` /
                                       ``.average_over_domain``
solve_one_direction + K assembly       ``PermeabilityProblem.solve_load_case`` /
                                       ``.solve_permeability``
=====================================  ==========================================

Arrays: masks and fields are numpy arrays shaped (nz, ny, nx) (x fastest, the
reference's flat index); vector fields are (3, nz, ny, nx); compact support
vectors are flat [3*local + comp].
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _capi

PRECISIONS = {"fp64": _capi.FP_PREC_FP64, "mixed": _capi.FP_PREC_MIXED}
SUPPORT_MODES = {"interface": _capi.FP_SUPPORT_INTERFACE, "fullsolid": _capi.FP_SUPPORT_FULLSOLID}


@dataclass
class SolverResult:
    """src/solver/SolverResult.hpp:10-16"""
    solution: np.ndarray
    converged: bool = False
    iterations: int = 0
    final_rel_residual: float = 1.0
    residual_history: np.ndarray = field(default_factory=lambda: np.zeros(0))
    seconds: float = 0.0
    refinements: int = 0


class PermeabilityProblem:
    """One periodic grid with its device-resident solver state (an fp_handle)."""

    def __init__(self, shape, voxel_size: float = 1.0, mu: float = 1.0, p_radius: int = 2,
                 precision: str = "fp64"):
        self.lib = _capi.load()
        nz, ny, nx = (shape, shape, shape) if np.isscalar(shape) else tuple(shape)
        self.shape = (int(nz), int(ny), int(nx))
        self.mu = float(mu)
        self.voxel_size = float(voxel_size)
        self.p_radius = int(p_radius)
        h = C.c_void_p()
        rc = self.lib.fp_create(int(nx), int(ny), int(nz), float(voxel_size), float(mu),
                                int(p_radius), PRECISIONS[precision], C.byref(h))
        self._h = h
        if rc != _capi.FP_OK:
            try:
                _capi.check(self.lib, h, rc)
            finally:
                self.close()
        self.nb = 0
        self.n = int(nx) * int(ny) * int(nz)

    # -- lifetime ----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.fp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        _capi.check(self.lib, self._h, rc)

    @property
    def handle(self):
        return self._h

    # -- configuration -----------------------------------------------------
    def set_precision(self, precision: str):
        self._check(self.lib.fp_set_precision(self._h, PRECISIONS[precision]))

    def autotune(self) -> dict:
        """fp_autotune: picks the fastest FFT tiling for this grid."""
        tile, off, xb, xr, lo = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0)
        ms = C.c_double(0.0)
        self._check(self.lib.fp_autotune(self._h, C.byref(tile), C.byref(off), C.byref(xb),
                                         C.byref(xr), C.byref(lo), C.byref(ms)))
        return dict(tile=tile.value, tma=not off.value, x_bulk=bool(xb.value), x_rows=xr.value,
                    lowreg=bool(lo.value), apply_ms=ms.value)

    def set_tiling(self, tile: int = 0, tma: bool = True, x_bulk: bool = True, x_rows: int = 0,
                   lowreg: bool = False):
        """fp_set_tiling: a given FFT tiling (e.g. one autotune reported)."""
        self._check(self.lib.fp_set_tiling(self._h, int(tile), int(not tma), int(x_bulk),
                                           int(x_rows), int(lowreg)))

    def set_geometry(self, fluid_mask: np.ndarray, support: str = "interface") -> int:
        m = np.ascontiguousarray(fluid_mask, dtype=np.uint8)
        if m.shape != self.shape:
            raise ValueError("BinaryMedium mask size must match grid size")
        nb = C.c_int64(0)
        self._check(self.lib.fp_set_geometry(self._h, m.ravel(), SUPPORT_MODES[support],
                                             C.byref(nb)))
        self.nb = int(nb.value)
        self.mask = m
        return self.nb

    def load_fgeo(self, path: str, fluid_id: int = 1, support: str = "interface") -> int:
        """fp_load_fgeo: the geometry of a .fgeo file, the mask formed on the device."""
        if support not in SUPPORT_MODES:
            raise ValueError("unknown support mode " + repr(support))
        nb = C.c_int64(0)
        self._check(self.lib.fp_load_fgeo(self._h, path.encode(), int(fluid_id),
                                          SUPPORT_MODES[support], C.byref(nb)))
        self.nb = int(nb.value)
        self.mask = None
        return self.nb

    def recover_fvel(self, path: str, grad, x, porosity: float, viscosity: float = 1.0) -> None:
        """fp_recover_fvel: the recovered velocity field written to a .fvel file."""
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        if x.size != 3 * self.nb:
            raise ValueError("VelocityRecovery::recover compact solution size mismatch")
        self._check(self.lib.fp_recover_fvel(self._h, path.encode(), np.asarray(grad, np.float64), x,
                                             float(porosity), float(viscosity)))

    def support(self) -> np.ndarray:
        out = np.zeros(max(self.nb, 1), dtype=np.int64)
        self._check(self.lib.fp_get_support(self._h, out))
        return out[: self.nb]

    def green_tensor(self) -> np.ndarray:
        nz, ny, nx = self.shape
        g = np.zeros(6 * nz * ny * (nx // 2 + 1))
        self._check(self.lib.fp_get_green(self._h, g))
        return g.reshape(6, nz, ny, nx // 2 + 1)

    # -- operators -----------------------------------------------------------
    def green_apply(self, force: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(force, dtype=np.float64)
        if f.size != 3 * self.n:
            raise ValueError("GreenOperator::apply grid mismatch")
        u = np.zeros(3 * self.n)
        self._check(self.lib.fp_green_apply(self._h, f.ravel(), u))
        return u.reshape((3,) + self.shape)

    def fft_forward(self, real_field: np.ndarray) -> np.ndarray:
        """Half spectrum (3, nz, ny, nx//2+1) complex of a real (3, nz, ny, nx) field."""
        f = np.ascontiguousarray(real_field, dtype=np.float64)
        if f.size != 3 * self.n:
            raise ValueError("FFT backend forward grid size mismatch")
        nz, ny, nx = self.shape
        out = np.zeros(3 * nz * ny * (nx // 2 + 1) * 2)
        self._check(self.lib.fp_fft_forward(self._h, f.ravel(), out))
        return out.view(np.complex128).reshape(3, nz, ny, nx // 2 + 1)

    def fft_inverse(self, half_spectrum: np.ndarray) -> np.ndarray:
        """Real part of the inverse DFT (times 1/N) of a Hermitian half spectrum."""
        nz, ny, nx = self.shape
        h = np.ascontiguousarray(half_spectrum, dtype=np.complex128)
        if h.shape != (3, nz, ny, nx // 2 + 1):
            raise ValueError("FFT backend inverse grid size mismatch")
        out = np.zeros(3 * self.n)
        self._check(self.lib.fp_fft_inverse(self._h, h.view(np.float64).ravel(), out))
        return out.reshape((3,) + self.shape)

    def background_force(self, grad) -> np.ndarray:
        f0 = np.zeros(3 * self.n)
        self._check(self.lib.fp_background_force(self._h, np.asarray(grad, np.float64), f0))
        return f0.reshape((3,) + self.shape)

    def operator_apply(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        if x.size != 3 * self.nb:
            raise ValueError("VariationalOperator::apply input size mismatch")
        y = np.zeros(3 * self.nb)
        self._check(self.lib.fp_operator_apply(self._h, x, y))
        return y

    def build_rhs(self, grad) -> np.ndarray:
        b = np.zeros(3 * self.nb)
        self._check(self.lib.fp_build_rhs(self._h, np.asarray(grad, np.float64), b))
        return b

    def minres(self, b, tol: float, maxit: int, x0=None, history: bool = True) -> SolverResult:
        b = np.ascontiguousarray(b, dtype=np.float64).ravel()
        if b.size != 3 * self.nb:
            raise ValueError("MinresSolver::solve rhs size mismatch")
        x = np.zeros(3 * self.nb)
        hist = np.zeros(maxit + 1) if history else None
        st = _capi.SolverStats()
        x0p = None
        if x0 is not None:
            x0 = np.ascontiguousarray(x0, dtype=np.float64).ravel()
            if x0.size != 3 * self.nb:
                raise ValueError("MinresSolver::solve initial guess size mismatch")
            x0p = x0.ctypes.data
        self._check(self.lib.fp_minres(self._h, b, x0p, float(tol), int(maxit), x,
                                       hist.ctypes.data if history else None, C.byref(st)))
        d = st.as_dict()
        return SolverResult(solution=x, converged=d["converged"], iterations=d["iterations"],
                            final_rel_residual=d["final_rel_residual"],
                            residual_history=(hist[: d["iterations"] + 1] if history else np.zeros(0)),
                            seconds=d["seconds"], refinements=d["refinements"])

    def recover(self, grad, x, want_field: bool = False):
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        if x.size != 3 * self.nb:
            raise ValueError("VelocityRecovery::recover compact solution size mismatch")
        avg = np.zeros(3)
        v = np.zeros(3 * self.n) if want_field else None
        self._check(self.lib.fp_recover(self._h, np.asarray(grad, np.float64), x,
                                        v.ctypes.data if want_field else None, avg))
        return avg, (v.reshape((3,) + self.shape) if want_field else None)

    def solve_load_case(self, grad, tol: float, maxit: int, x0=None, want_solution: bool = False):
        avg = np.zeros(3)
        st = _capi.SolverStats()
        x0p = None
        if x0 is not None:
            x0 = np.ascontiguousarray(x0, dtype=np.float64).ravel()
            x0p = x0.ctypes.data
        xo = np.zeros(3 * self.nb) if want_solution else None
        self._check(self.lib.fp_solve_load_case(self._h, np.asarray(grad, np.float64), x0p,
                                                float(tol), int(maxit), avg,
                                                xo.ctypes.data if want_solution else None,
                                                C.byref(st)))
        return avg, st.as_dict(), xo

    def solve_permeability(self, tol: float, maxit: int, block: bool = False):
        """K from the three load cases (fp_solve_permeability), or with
        block=True the three as one lockstep block (fp_solve_permeability_block;
        the same K)."""
        K = np.zeros(9)
        stats = (_capi.SolverStats * 3)()
        fn = self.lib.fp_solve_permeability_block if block else self.lib.fp_solve_permeability
        self._check(fn(self._h, float(tol), int(maxit), K, stats))
        return K.reshape(3, 3), [s.as_dict() for s in stats]


# ---------------------------------------------------------------------------
# Reference-named facades
# ---------------------------------------------------------------------------

class ForceSupport:
    """src/bignonnet/ForceSupport.hpp:12-31 over a PermeabilityProblem."""

    def __init__(self, problem: PermeabilityProblem, fluid_mask, mode: str = "interface"):
        self.problem = problem
        problem.set_geometry(fluid_mask, mode)
        self._active = problem.support()
        self._local = {int(v): i for i, v in enumerate(self._active)}

    def size(self) -> int:
        return 3 * len(self._active)

    def num_active_voxels(self) -> int:
        return len(self._active)

    def active_voxels(self) -> np.ndarray:
        return self._active

    def contains_voxel(self, voxel: int) -> bool:
        return int(voxel) in self._local

    def local_index(self, voxel: int) -> int:
        if int(voxel) not in self._local:
            raise IndexError("Voxel is not in active support")
        return self._local[int(voxel)]

    def global_index(self, local: int) -> int:
        if not 0 <= local < len(self._active):
            raise IndexError("Support local index out of range")
        return int(self._active[local])


class GreenOperator:
    """src/bignonnet/GreenOperator.hpp:13-44: apply(force) -> velocity-like field."""

    def __init__(self, problem: PermeabilityProblem):
        self.problem = problem

    def apply(self, force: np.ndarray) -> np.ndarray:
        return self.problem.green_apply(force)


class BackgroundForce:
    """src/bignonnet/BackgroundForce.hpp:10-19."""

    def __init__(self, problem: PermeabilityProblem):
        self.problem = problem

    def build(self, grad) -> np.ndarray:
        return self.problem.background_force(grad)


class VariationalOperator:
    """The ILinearOperator of the method (src/bignonnet/VariationalOperator.hpp:10-26)."""

    def __init__(self, problem: PermeabilityProblem):
        self.problem = problem

    def size(self) -> int:
        return 3 * self.problem.nb

    def apply(self, x) -> np.ndarray:
        return self.problem.operator_apply(x)


class VariationalRHS:
    """src/bignonnet/VariationalRHS.hpp:11-26."""

    def __init__(self, problem: PermeabilityProblem):
        self.problem = problem

    def build(self, grad) -> np.ndarray:
        return self.problem.build_rhs(grad)


class MinresSolver:
    """src/solver/MinresSolver.hpp:11-30; the iteration runs on the GPU."""

    def __init__(self, tolerance: float, max_iterations: int):
        if not tolerance > 0:
            raise ValueError("MinresSolver tolerance must be positive")
        self.tolerance = float(tolerance)
        self.max_iterations = int(max_iterations)

    def solve(self, op: VariationalOperator, rhs, initial_guess=None) -> SolverResult:
        return op.problem.minres(rhs, self.tolerance, self.max_iterations, x0=initial_guess)


class VelocityRecovery:
    """src/bignonnet/VelocityRecovery.hpp:13-29."""

    def __init__(self, problem: PermeabilityProblem):
        self.problem = problem

    def recover(self, grad, compact_solution) -> np.ndarray:
        _, v = self.problem.recover(grad, compact_solution, want_field=True)
        return v

    def average_over_domain(self, velocity: np.ndarray) -> np.ndarray:
        return velocity.reshape(3, -1).mean(axis=1)

    def average_over_support(self, velocity: np.ndarray) -> np.ndarray:
        sup = self.problem.support()
        return velocity.reshape(3, -1)[:, sup].mean(axis=1)


class PermeabilityTensor:
    """src/post/PermeabilityTensor.cpp:11-18: set_column(col, avg_velocity)
    stores -avg_velocity in column col (row-major k[row*3 + col])."""

    def __init__(self):
        self.k = np.zeros(9)

    def set_column(self, column: int, avg_velocity):
        if not 0 <= column < 3:
            raise IndexError("PermeabilityTensor::set_column index out of range")
        for row in range(3):
            self.k[row * 3 + column] = -avg_velocity[row]

    def data(self) -> np.ndarray:
        return self.k

    def to_string(self, indent: str = "") -> str:
        """src/post/PermeabilityTensor.cpp:20-28: rows in scientific notation
        with 6 digits, two spaces between entries, rows joined by newline +
        indent."""
        rows = ["  ".join("%.6e" % self.k[3 * r + c] for c in range(3)) for r in range(3)]
        return ("\n" + indent).join(rows)


# ---------------------------------------------------------------------------
# Brinkman penalisation (include/brinkman/FluidBrinkman.hpp:45-55)
# ---------------------------------------------------------------------------

def _brinkman_check(lib, rc):
    if rc == _capi.FP_OK:
        return
    msg = lib.fp_brinkman_last_error().decode()
    if rc == _capi.FP_ERR_INVALID:
        raise ValueError(msg)
    raise _capi.FpError(rc, msg)


def solveBrinkman(ids: np.ndarray, force, fluid_id: int = 1, fluid_mu: float = 1.0,
                  solid_penalty: float = 1.0e8, relaxation: float = 0.9,
                  tolerance: float = 1.0e-8, max_iterations: int = 600,
                  want_fields: bool = False) -> dict:
    """common::fluid::solveBrinkman on the GPU.  ids: material ids (nz, ny, nx);
    defaults are the reference's FluidConfig defaults (Config.hpp:33-47)."""
    lib = _capi.load()
    ids = np.ascontiguousarray(ids, dtype=np.uint32)
    nz, ny, nx = ids.shape
    n = ids.size
    fields = [np.zeros(n) for _ in range(4)] if want_fields else None
    U = np.zeros(3)
    st = _capi.BrinkmanStats()
    ptrs = [f.ctypes.data for f in fields] if want_fields else [None] * 4
    rc = lib.fp_brinkman_solve(nx, ny, nz, ids.ravel(), int(fluid_id), float(fluid_mu),
                               float(solid_penalty), float(relaxation), float(tolerance),
                               int(max_iterations), np.asarray(force, np.float64), *ptrs, U,
                               C.byref(st))
    _brinkman_check(lib, rc)
    out = dict(superficialVelocity=U, **st.as_dict())
    if want_fields:
        out.update(ux=fields[0].reshape(ids.shape), uy=fields[1].reshape(ids.shape),
                   uz=fields[2].reshape(ids.shape), p=fields[3].reshape(ids.shape))
    return out


def computePermeabilityTensor(ids: np.ndarray, fluid_id: int = 1, fluid_mu: float = 1.0,
                              solid_penalty: float = 1.0e8, relaxation: float = 0.9,
                              tolerance: float = 1.0e-8, max_iterations: int = 600,
                              forcing: float = 1.0, voxel_size: float = 1.0):
    """common::fluid::computePermeabilityTensor on the GPU: (K 3x3, [stats] * 3)."""
    lib = _capi.load()
    ids = np.ascontiguousarray(ids, dtype=np.uint32)
    nz, ny, nx = ids.shape
    K = np.zeros(9)
    stats = (_capi.BrinkmanStats * 3)()
    rc = lib.fp_brinkman_permeability(nx, ny, nz, ids.ravel(), int(fluid_id), float(fluid_mu),
                                      float(solid_penalty), float(relaxation), float(tolerance),
                                      int(max_iterations), float(forcing), float(voxel_size), K,
                                      stats)
    _brinkman_check(lib, rc)
    return K.reshape(3, 3), [s.as_dict() for s in stats]


def solveBrinkmanFixedPoint(ids: np.ndarray, force, fluid_id: int = 1, fluid_mu: float = 1.0,
                            solid_penalty: float = 1.0e8, tolerance: float = 1.0e-8,
                            max_iterations: int = 20000, want_fields: bool = False) -> dict:
    """The Brinkman problem of solveBrinkman solved to the discrete fixed point
    of the reference's equations (fp_brinkman_fft_solve: FFT-preconditioned
    projected conjugate gradient, FP64).  residual = |P(f - A u)| / |P f|."""
    lib = _capi.load()
    ids = np.ascontiguousarray(ids, dtype=np.uint32)
    nz, ny, nx = ids.shape
    n = ids.size
    fields = [np.zeros(n) for _ in range(4)] if want_fields else None
    U = np.zeros(3)
    st = _capi.BrinkmanStats()
    ptrs = [f.ctypes.data for f in fields] if want_fields else [None] * 4
    rc = lib.fp_brinkman_fft_solve(nx, ny, nz, ids.ravel(), int(fluid_id), float(fluid_mu),
                                   float(solid_penalty), float(tolerance), int(max_iterations),
                                   np.asarray(force, np.float64), *ptrs, U, C.byref(st))
    _brinkman_check(lib, rc)
    out = dict(superficialVelocity=U, **st.as_dict())
    if want_fields:
        out.update(ux=fields[0].reshape(ids.shape), uy=fields[1].reshape(ids.shape),
                   uz=fields[2].reshape(ids.shape), p=fields[3].reshape(ids.shape))
    return out


def computePermeabilityTensorFixedPoint(ids: np.ndarray, fluid_id: int = 1, fluid_mu: float = 1.0,
                                        solid_penalty: float = 1.0e8, tolerance: float = 1.0e-8,
                                        max_iterations: int = 20000, forcing: float = 1.0,
                                        voxel_size: float = 1.0):
    """computePermeabilityTensor on the fixed-point solver: (K 3x3, [stats] * 3)."""
    lib = _capi.load()
    ids = np.ascontiguousarray(ids, dtype=np.uint32)
    nz, ny, nx = ids.shape
    K = np.zeros(9)
    stats = (_capi.BrinkmanStats * 3)()
    rc = lib.fp_brinkman_fft_permeability(nx, ny, nz, ids.ravel(), int(fluid_id), float(fluid_mu),
                                          float(solid_penalty), float(tolerance),
                                          int(max_iterations), float(forcing), float(voxel_size),
                                          K, stats)
    _brinkman_check(lib, rc)
    return K.reshape(3, 3), [s.as_dict() for s in stats]


def batch_solve_permeability(masks, precision: str = "mixed", tol: float = 1e-7,
                             maxit: int = 20000, concurrency: int = 4, autotune: bool = True,
                             voxel_sizes=None, mu: float = 1.0, p_radius: int = 2,
                             support_mode: int = 0, max_group: int = 1):
    """fp_batch_solve_grouped over a list of fluid masks (each (nz, ny, nx),
    sizes may differ): returns (K of shape (count, 3, 3), stats per problem
    [3 dicts each], status codes).  max_group = 1 solves each problem on its
    own (fp_batch_solve_permeability); larger values solve up to that many
    problems of one grid together, one launch per pass for the group."""
    lib = _capi.load()
    count = len(masks)
    arrs = [np.ascontiguousarray(m, dtype=np.uint8) for m in masks]
    dims = np.array([[a.shape[2], a.shape[1], a.shape[0]] for a in arrs], dtype=np.int32).ravel()
    ptrs = (C.c_void_p * max(count, 1))(*[a.ctypes.data for a in arrs])
    vs = None if voxel_sizes is None else np.ascontiguousarray(voxel_sizes, dtype=np.float64)
    K = np.zeros(9 * max(count, 1))
    stats = (_capi.SolverStats * (3 * max(count, 1)))()
    status = np.zeros(max(count, 1), dtype=np.int32)
    rc = lib.fp_batch_solve_grouped(count, dims.ctypes.data, ptrs,
                                    None if vs is None else vs.ctypes.data, float(mu),
                                    int(p_radius), PRECISIONS[precision], int(support_mode),
                                    float(tol), int(maxit), int(concurrency), int(autotune),
                                    int(max_group), K, stats, status.ctypes.data)
    if rc != _capi.FP_OK:
        msg = lib.fp_batch_last_error().decode()
        if rc == _capi.FP_ERR_INVALID:
            raise ValueError(msg)
        raise _capi.FpError(rc, msg)
    st = [[stats[3 * i + c].as_dict() for c in range(3)] for i in range(count)]
    return K[: 9 * count].reshape(count, 3, 3), st, status[:count].tolist()


def group_solve_permeability(problems, tol: float, maxit: int = 20000):
    """fp_group_solve_permeability: K of several PermeabilityProblem objects of
    one grid (geometry set) solved together, one launch per pass for all of
    them.  Returns (K of shape (count, 3, 3), stats per problem [3 dicts])."""
    lib = _capi.load()
    count = len(problems)
    hs = (C.c_void_p * max(count, 1))(*[p.handle.value for p in problems])
    K = np.zeros(9 * max(count, 1))
    stats = (_capi.SolverStats * (3 * max(count, 1)))()
    rc = lib.fp_group_solve_permeability(count, hs, float(tol), int(maxit), K, stats)
    if rc != _capi.FP_OK:
        msg = "; ".join(lib.fp_last_error(p.handle).decode() for p in problems)
        if rc == _capi.FP_ERR_INVALID:
            raise ValueError(msg)
        raise _capi.FpError(rc, msg)
    st = [[stats[3 * i + c].as_dict() for c in range(3)] for i in range(count)]
    return K[: 9 * count].reshape(count, 3, 3), st


def write_fvel(path: str, velocity, porosity: float, viscosity: float, driving) -> None:
    """The reference's .fvel file (fp_write_fvel) from a (3, nz, ny, nx) field."""
    lib = _capi.load()
    v = np.asarray(velocity, dtype=np.float64)
    if v.ndim != 4 or v.shape[0] != 3:
        raise ValueError("velocity must have shape (3, nz, ny, nx)")
    nz, ny, nx = v.shape[1:]
    comps = [np.ascontiguousarray(v[c]).ravel() for c in range(3)]
    rc = lib.fp_write_fvel(path.encode(), int(nx), int(ny), int(nz), float(porosity),
                           float(viscosity), np.asarray(driving, np.float64), *comps)
    if rc != _capi.FP_OK:
        raise OSError("cannot write velocity file: " + path)


def read_fvel(path: str) -> dict:
    """Reads a .fvel file: dict(velocity (3, nz, ny, nx), porosity, viscosity, driving)."""
    raw = open(path, "rb").read()
    if raw[:4] != b"FVEL" or raw[4] != 1:
        raise ValueError("not a version-1 .fvel file: " + path)
    nx, ny, nz = np.frombuffer(raw, "<u8", 3, 8)
    por, mu = np.frombuffer(raw, "<f8", 2, 32)
    drv = np.frombuffer(raw, "<f8", 3, 48)
    n = int(nx) * int(ny) * int(nz)
    rec = np.frombuffer(raw, "<f8", 3 * n, 72).reshape(n, 3)
    vel = rec.T.reshape(3, int(nz), int(ny), int(nx)).copy()
    return dict(velocity=vel, porosity=float(por), viscosity=float(mu), driving=drv.copy())

