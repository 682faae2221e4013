"""ctypes front end for the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Two checkers share one Python interface:

* ``Restatement`` -- the plain-C FP64 restatement of the reference algorithm
  (``oracle/fftperm_oracle.c``), built by ``make -C oracle restatement`` into
  ``oracle/_build``.  It builds on any host with gcc, so it is the checker on
  the GPU host too.
* ``Reference`` -- the reference's OWN classes compiled unmodified from its
  sources (``make -C oracle ref``) into ``oracle/_ref``, driven through
  ``oracle/ref_capi.cpp``.  Available only where the reference sources were
  present at build time; used to pin the restatement and to make golden
  fixtures.

Only tests, the smoke check and the CPU-baseline leg of bench.py import this
module; the product path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RESTATEMENT_SO = os.path.join(HERE, "_build", "libfftperm_oracle.so")
REFERENCE_SO = os.path.join(HERE, "_ref", "libfftperm_ref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_ll = C.c_longlong


def build_restatement(quiet: bool = True) -> str:
    """Compile the restatement with make (gcc); returns the .so path."""
    out = subprocess.run(["make", "-C", HERE, "restatement"], capture_output=quiet, text=True)
    if out.returncode != 0:
        raise RuntimeError("building the oracle restatement failed:\n" + (out.stderr or ""))
    return RESTATEMENT_SO


def reference_available() -> bool:
    return os.path.exists(REFERENCE_SO)


class _Base:
    """Shared shape of both checkers (names mirror the reference classes)."""

    prefix = ""

    def __init__(self, so_path: str):
        self.lib = C.CDLL(so_path)
        p = self.prefix
        L = self.lib
        self._support = getattr(L, p + "support")
        self._ctx_create = getattr(L, p + ("ctx_create" if p == "ref_" else "create"))
        self._ctx_create.restype = C.c_void_p
        self._ctx_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                     _u8p, C.c_int, C.c_int]
        self._ctx_destroy = getattr(L, p + ("ctx_destroy" if p == "ref_" else "destroy"))
        self._ctx_destroy.argtypes = [C.c_void_p]
        self._ctx_nb = getattr(L, p + ("ctx_nb" if p == "ref_" else "nb"))
        self._ctx_nb.restype = _ll
        self._ctx_nb.argtypes = [C.c_void_p]
        self._op = getattr(L, p + "operator_apply")
        self._op.argtypes = [C.c_void_p, _dp, _dp]
        self._rhs = getattr(L, p + "build_rhs")
        self._rhs.argtypes = [C.c_void_p, _dp, _dp]
        self._minres = getattr(L, p + "minres")
        self._minres.restype = C.c_int
        self._minres.argtypes = [C.c_void_p, _dp, C.c_void_p, C.c_double, _ll, _dp, _dp,
                                 C.POINTER(_ll), C.POINTER(C.c_double), C.POINTER(C.c_int)]
        self._recover = getattr(L, p + "recover")
        self._recover.argtypes = [C.c_void_p, _dp, _dp, C.c_void_p, _dp]
        self._perm = getattr(L, p + "solve_permeability")
        self._perm.restype = C.c_int
        self._perm.argtypes = ([C.c_void_p] + ([C.c_double] if p == "ref_" else []) +
                               [C.c_double, _ll, _dp, _i64p])
        self._brink = getattr(L, p + "brinkman_solve")

    # -- support / f0 ------------------------------------------------------
    def support(self, mask: np.ndarray, mode: int = 0) -> np.ndarray:
        nz, ny, nx = mask.shape
        m = np.ascontiguousarray(mask, dtype=np.uint8).ravel()
        self._support.restype = _ll
        self._support.argtypes = [C.c_int, C.c_int, C.c_int, _u8p, C.c_int, C.c_void_p]
        nb = self._support(nx, ny, nz, m, mode, None)
        out = np.zeros(max(nb, 1), dtype=np.int64)
        self._support(nx, ny, nz, m, mode, out.ctypes.data)
        return out[:nb]

    # -- context -----------------------------------------------------------
    def context(self, mask: np.ndarray, h: float = 1.0, mu: float = 1.0, p_radius: int = 2,
                mode: int = 0, threads: int = 0) -> "_Ctx":
        return _Ctx(self, mask, h, mu, p_radius, mode, threads)


class _Ctx:
    def __init__(self, owner: _Base, mask, h, mu, p_radius, mode, threads):
        self.o = owner
        self.shape = mask.shape
        nz, ny, nx = mask.shape
        self.mu = mu
        m = np.ascontiguousarray(mask, dtype=np.uint8).ravel()
        self.ptr = owner._ctx_create(nx, ny, nz, h, mu, p_radius, m, mode, threads)
        if not self.ptr:
            raise RuntimeError("oracle context creation failed")
        self.nb = int(owner._ctx_nb(self.ptr))

    def close(self):
        if self.ptr:
            self.o._ctx_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        self.close()

    def operator_apply(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(3 * self.nb)
        self.o._op(self.ptr, x, y)
        return y

    def build_rhs(self, grad) -> np.ndarray:
        b = np.zeros(3 * self.nb)
        self.o._rhs(self.ptr, np.asarray(grad, dtype=np.float64), b)
        return b

    def minres(self, b, tol: float, maxit: int, x0=None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(3 * self.nb)
        hist = np.zeros(maxit + 1)
        it, rel, conv = _ll(0), C.c_double(0), C.c_int(0)
        x0p = None
        if x0 is not None:
            x0 = np.ascontiguousarray(x0, dtype=np.float64)
            x0p = x0.ctypes.data
        nh = self.o._minres(self.ptr, b, x0p, tol, maxit, x, hist, C.byref(it), C.byref(rel),
                            C.byref(conv))
        return dict(solution=x, iterations=int(it.value), final_rel_residual=float(rel.value),
                    converged=bool(conv.value), residual_history=hist[:nh].copy())

    def recover(self, grad, x, want_field: bool = False):
        n = int(np.prod(self.shape))
        v = np.zeros(3 * n) if want_field else None
        avg = np.zeros(3)
        self.o._recover(self.ptr, np.asarray(grad, dtype=np.float64),
                        np.ascontiguousarray(x, dtype=np.float64),
                        v.ctypes.data if want_field else None, avg)
        return avg, v

    def solve_permeability(self, tol: float, maxit: int):
        K = np.zeros(9)
        it = np.zeros(3, dtype=np.int64)
        if self.o.prefix == "ref_":
            rc = self.o._perm(self.ptr, self.mu, tol, maxit, K, it)
        else:
            rc = self.o._perm(self.ptr, tol, maxit, K, it)
        if rc != 0:
            raise RuntimeError("oracle permeability solve failed")
        return K.reshape(3, 3), it


class Restatement(_Base):
    prefix = "orc_"

    def __init__(self, so_path: str | None = None):
        path = so_path or RESTATEMENT_SO
        if not os.path.exists(path):
            build_restatement()
        super().__init__(path)
        L = self.lib
        L.orc_green_tensor.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                       _dp, C.c_int]
        L.orc_background_force.argtypes = [C.c_int, C.c_int, C.c_int, _u8p, _i64p, _ll, _dp, _dp]
        self._brink.restype = C.c_int
        self._brink.argtypes = [C.c_int, C.c_int, C.c_int, _u32p, C.c_uint, C.c_double,
                                C.c_double, C.c_double, C.c_double, C.c_int, _dp, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_void_p, _dp, C.POINTER(C.c_int),
                                C.POINTER(C.c_double), C.POINTER(C.c_int),
                                C.POINTER(C.c_double), C.POINTER(C.c_double)]

    def green_tensor(self, shape, h=1.0, mu=1.0, p_radius=2, threads=0) -> np.ndarray:
        nz, ny, nx = shape
        g = np.zeros(6 * nx * ny * nz)
        self.lib.orc_green_tensor(nx, ny, nz, h, mu, p_radius, g, threads)
        return g.reshape(6, nz, ny, nx)

    def background_force(self, mask, grad, mode=0) -> np.ndarray:
        nz, ny, nx = mask.shape
        sup = self.support(mask, mode)
        f0 = np.zeros(3 * mask.size)
        self.lib.orc_background_force(nx, ny, nz, np.ascontiguousarray(mask, np.uint8).ravel(),
                                      np.ascontiguousarray(sup), len(sup),
                                      np.asarray(grad, np.float64), f0)
        return f0.reshape(3, nz, ny, nx)

    def brinkman(self, ids: np.ndarray, fluid_id: int = 1, fluid_mu: float = 1.0,
                 solid_penalty: float = 1e4, relaxation: float = 0.9, tolerance: float = 1e-8,
                 max_iterations: int = 100, force=(1.0, 0.0, 0.0), want_fields: bool = False):
        nz, ny, nx = ids.shape
        n = ids.size
        fields = [np.zeros(n) for _ in range(4)] if want_fields else None
        U = np.zeros(3)
        it, res, conv = C.c_int(0), C.c_double(0), C.c_int(0)
        por, mm = C.c_double(0), C.c_double(0)
        ptrs = [f.ctypes.data for f in fields] if want_fields else [None] * 4
        rc = self._brink(nx, ny, nz, np.ascontiguousarray(ids, np.uint32).ravel(), fluid_id,
                         fluid_mu, solid_penalty, relaxation, tolerance, max_iterations,
                         np.asarray(force, np.float64), *ptrs, U, C.byref(it), C.byref(res),
                         C.byref(conv), C.byref(por), C.byref(mm))
        if rc != 0:
            raise RuntimeError("Brinkman oracle failed (non-finite residual or invalid phases)")
        out = dict(U=U, iterations=it.value, residual=res.value, converged=bool(conv.value),
                   porosity=por.value, viscosity=mm.value)
        if want_fields:
            out.update(ux=fields[0], uy=fields[1], uz=fields[2], p=fields[3])
        return out


class Reference(_Base):
    prefix = "ref_"

    def __init__(self, so_path: str | None = None):
        path = so_path or REFERENCE_SO
        if not os.path.exists(path):
            raise FileNotFoundError("reference build missing: run make -C oracle ref")
        super().__init__(path)
        L = self.lib
        L.ref_green_tensor.restype = C.c_int
        L.ref_green_tensor.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                       C.c_int, _dp]
        L.ref_background_force.restype = C.c_int
        L.ref_background_force.argtypes = [C.c_int, C.c_int, C.c_int, _u8p, C.c_int, _dp, _dp]
        L.ref_green_apply.restype = C.c_int
        L.ref_green_apply.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                      C.c_int, _dp, _dp]
        self._brink.restype = C.c_int
        self._brink.argtypes = [C.c_int, C.c_int, C.c_int, _u32p, C.c_uint, C.c_double,
                                C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, _dp,
                                C.c_void_p, C.c_void_p, C.c_void_p, _dp, C.POINTER(C.c_int),
                                C.POINTER(C.c_double), C.POINTER(C.c_int)]

    def green_tensor(self, shape, h=1.0, mu=1.0, p_radius=2) -> np.ndarray:
        nz, ny, nx = shape
        g = np.zeros(6 * nx * ny * nz)
        if self.lib.ref_green_tensor(nx, ny, nz, h, mu, p_radius, g) != 0:
            raise RuntimeError("ref_green_tensor failed")
        return g.reshape(6, nz, ny, nx)

    def green_apply(self, f_soa: np.ndarray, h=1.0, mu=1.0, p_radius=2, threads=1) -> np.ndarray:
        _, nz, ny, nx = f_soa.shape
        u = np.zeros(f_soa.size)
        if self.lib.ref_green_apply(nx, ny, nz, h, mu, p_radius, threads,
                                    np.ascontiguousarray(f_soa, np.float64).ravel(), u) != 0:
            raise RuntimeError("ref_green_apply failed")
        return u.reshape(f_soa.shape)

    def background_force(self, mask, grad, mode=0) -> np.ndarray:
        nz, ny, nx = mask.shape
        f0 = np.zeros(3 * mask.size)
        if self.lib.ref_background_force(nx, ny, nz, np.ascontiguousarray(mask, np.uint8).ravel(),
                                         mode, np.asarray(grad, np.float64), f0) != 0:
            raise RuntimeError("ref_background_force failed")
        return f0.reshape(3, nz, ny, nx)

    def brinkman(self, ids: np.ndarray, fluid_id: int = 1, fluid_mu: float = 1.0,
                 solid_penalty: float = 1e4, relaxation: float = 0.9, tolerance: float = 1e-8,
                 max_iterations: int = 100, force=(1.0, 0.0, 0.0), want_fields: bool = False,
                 voxel_size: float = 1.0):
        nz, ny, nx = ids.shape
        n = ids.size
        fields = [np.zeros(n) for _ in range(3)] if want_fields else None
        U = np.zeros(3)
        it, res, conv = C.c_int(0), C.c_double(0), C.c_int(0)
        ptrs = [f.ctypes.data for f in fields] if want_fields else [None] * 3
        rc = self._brink(nx, ny, nz, np.ascontiguousarray(ids, np.uint32).ravel(), fluid_id,
                         fluid_mu, solid_penalty, relaxation, tolerance, max_iterations,
                         voxel_size, np.asarray(force, np.float64), *ptrs, U, C.byref(it),
                         C.byref(res), C.byref(conv))
        if rc != 0:
            raise RuntimeError("reference solveBrinkman threw")
        out = dict(U=U, iterations=it.value, residual=res.value, converged=bool(conv.value))
        if want_fields:
            out.update(ux=fields[0], uy=fields[1], uz=fields[2])
        return out
