"""ctypes binding of the C ABI (include/fftperm.h) in _build/libfftperm.so.

Loading fails loudly when the library has not been built: there is no CPU
fallback on the product path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfftperm.so")

FP_OK = 0
FP_ERR_INVALID = 1
FP_ERR_STATE = 2
FP_ERR_CUDA = 3
FP_ERR_UNSUPPORTED = 4
FP_ERR_NOMEM = 5
FP_ERR_NONFINITE = 6

FP_PREC_FP64 = 0
FP_PREC_MIXED = 1

FP_SUPPORT_INTERFACE = 0
FP_SUPPORT_FULLSOLID = 1

# Every symbol declared in include/fftperm.h (checked by the CPU tests).
EXPORTED = [
    "fp_create", "fp_destroy", "fp_last_error", "fp_stream", "fp_synchronize",
    "fp_set_precision", "fp_set_geometry",
    "fp_get_support", "fp_get_green", "fp_fft_forward", "fp_fft_inverse", "fp_green_apply",
    "fp_background_force",
    "fp_operator_apply", "fp_operator_apply_device", "fp_build_rhs", "fp_minres", "fp_recover",
    "fp_solve_load_case", "fp_solve_permeability", "fp_brinkman_solve",
    "fp_brinkman_permeability", "fp_brinkman_last_error", "fp_green_apply_noalloc",
    "fp_kernel_launch_count", "fp_brinkman_fft_solve", "fp_brinkman_fft_permeability",
    "fp_autotune", "fp_set_tiling", "fp_batch_solve_permeability", "fp_batch_solve_grouped",
    "fp_group_solve_permeability", "fp_solve_permeability_block", "fp_batch_last_error", "fp_write_fvel",
    "fp_nn_conv", "fp_nn_wgrad", "fp_nn_bias_grad", "fp_nn_relu_back", "fp_nn_adam", "fp_nn_loss",
    "fp_measure_fp64_rate", "fp_nn_conv_tc", "fp_nn_tc_error", "fp_nn_pool2", "fp_nn_pool2_back",
    "fp_nn_up2_add", "fp_nn_up2_add_back", "fp_nn_wgrad_cc", "fp_time_apply",
    "fp_load_fgeo", "fp_recover_fvel",
]


class SolverStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int64),
        ("final_rel_residual", C.c_double),
        ("converged", C.c_int32),
        ("refinements", C.c_int32),
        ("seconds", C.c_double),
    ]

    def as_dict(self) -> dict:
        return dict(iterations=int(self.iterations), final_rel_residual=float(self.final_rel_residual),
                    converged=bool(self.converged), refinements=int(self.refinements),
                    seconds=float(self.seconds))


class BrinkmanStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("converged", C.c_int32),
        ("residual", C.c_double),
        ("porosity", C.c_double),
        ("viscosity", C.c_double),
        ("seconds", C.c_double),
    ]

    def as_dict(self) -> dict:
        return dict(iterations=int(self.iterations), converged=bool(self.converged),
                    residual=float(self.residual), porosity=float(self.porosity),
                    viscosity=float(self.viscosity), seconds=float(self.seconds))


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_h = C.c_void_p

_SIGNATURES = {
    "fp_create": ([C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                   C.POINTER(C.c_void_p)], C.c_int),
    "fp_destroy": ([_h], C.c_int),
    "fp_last_error": ([_h], C.c_char_p),
    "fp_stream": ([_h], C.c_void_p),
    "fp_synchronize": ([_h], C.c_int),
    "fp_kernel_launch_count": ([], C.c_longlong),
    "fp_measure_fp64_rate": ([C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
    "fp_time_apply": ([C.c_void_p, C.c_int, C.POINTER(C.c_double)], C.c_int),
    "fp_load_fgeo": ([C.c_void_p, C.c_char_p, C.c_uint32, C.c_int, C.POINTER(C.c_int64)], C.c_int),
    "fp_recover_fvel": ([C.c_void_p, C.c_char_p, _dp, _dp, C.c_double, C.c_double], C.c_int),
    "fp_set_precision": ([_h, C.c_int], C.c_int),
    "fp_set_geometry": ([_h, _u8p, C.c_int, C.POINTER(C.c_int64)], C.c_int),
    "fp_get_support": ([_h, _i64p], C.c_int),
    "fp_get_green": ([_h, _dp], C.c_int),
    "fp_fft_forward": ([_h, _dp, _dp], C.c_int),
    "fp_fft_inverse": ([_h, _dp, _dp], C.c_int),
    "fp_green_apply": ([_h, _dp, _dp], C.c_int),
    "fp_background_force": ([_h, _dp, _dp], C.c_int),
    "fp_operator_apply": ([_h, _dp, _dp], C.c_int),
    "fp_operator_apply_device": ([_h, C.c_void_p, C.c_void_p], C.c_int),
    "fp_build_rhs": ([_h, _dp, _dp], C.c_int),
    "fp_minres": ([_h, _dp, C.c_void_p, C.c_double, C.c_int64, _dp, C.c_void_p,
                   C.POINTER(SolverStats)], C.c_int),
    "fp_recover": ([_h, _dp, _dp, C.c_void_p, _dp], C.c_int),
    "fp_solve_load_case": ([_h, _dp, C.c_void_p, C.c_double, C.c_int64, _dp, C.c_void_p,
                            C.POINTER(SolverStats)], C.c_int),
    "fp_solve_permeability": ([_h, C.c_double, C.c_int64, _dp, C.POINTER(SolverStats)], C.c_int),
    "fp_brinkman_solve": ([C.c_int, C.c_int, C.c_int, _u32p, C.c_uint32, C.c_double, C.c_double,
                           C.c_double, C.c_double, C.c_int, _dp, C.c_void_p, C.c_void_p,
                           C.c_void_p, C.c_void_p, _dp, C.POINTER(BrinkmanStats)], C.c_int),
    "fp_brinkman_permeability": ([C.c_int, C.c_int, C.c_int, _u32p, C.c_uint32, C.c_double,
                                  C.c_double, C.c_double, C.c_double, C.c_int, C.c_double,
                                  C.c_double, _dp, C.POINTER(BrinkmanStats)], C.c_int),
    "fp_brinkman_last_error": ([], C.c_char_p),
    "fp_autotune": ([_h, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
                    C.c_int),
    "fp_set_tiling": ([_h, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int], C.c_int),
    "fp_batch_solve_permeability": ([C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                     C.c_int, C.c_int, C.c_int, C.c_double, C.c_int64, C.c_int,
                                     C.c_int, _dp, C.c_void_p, C.c_void_p], C.c_int),
    "fp_batch_solve_grouped": ([C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                C.c_int, C.c_int, C.c_int, C.c_double, C.c_int64, C.c_int,
                                C.c_int, C.c_int, _dp, C.c_void_p, C.c_void_p], C.c_int),
    "fp_group_solve_permeability": ([C.c_int, C.c_void_p, C.c_double, C.c_int64, _dp, C.c_void_p],
                                     C.c_int),
    "fp_solve_permeability_block": ([_h, C.c_double, C.c_int64, _dp, C.POINTER(SolverStats)], C.c_int),
    "fp_batch_last_error": ([], C.c_char_p),
    "fp_nn_conv": ([C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_int,
                    C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p],
                   C.c_int),
    "fp_nn_conv_tc": ([C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_int,
                       C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p],
                      C.c_int),
    "fp_nn_tc_error": ([C.POINTER(C.c_int), C.c_int], C.c_int),
    "fp_nn_pool2": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p],
                    C.c_int),
    "fp_nn_pool2_back": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                          C.c_void_p], C.c_int),
    "fp_nn_up2_add": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                       C.c_void_p, C.c_void_p], C.c_int),
    "fp_nn_up2_add_back": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                            C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "fp_nn_wgrad_cc": ([C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                        C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "fp_nn_wgrad": ([C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                     C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "fp_nn_bias_grad": ([C.c_void_p, C.c_int64, C.c_int, C.c_void_p, C.c_void_p], C.c_int),
    "fp_nn_relu_back": ([C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_void_p],
                        C.c_int),
    "fp_nn_adam": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float, C.c_float,
                    C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, C.c_void_p,
                    C.c_void_p, C.c_void_p], C.c_int),
    "fp_nn_loss": ([C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_void_p,
                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "fp_write_fvel": ([C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _dp, _dp, _dp,
                       _dp], C.c_int),
    "fp_brinkman_fft_solve": ([C.c_int, C.c_int, C.c_int, _u32p, C.c_uint32, C.c_double,
                               C.c_double, C.c_double, C.c_int, _dp, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_void_p, _dp, C.POINTER(BrinkmanStats)], C.c_int),
    "fp_brinkman_fft_permeability": ([C.c_int, C.c_int, C.c_int, _u32p, C.c_uint32, C.c_double,
                                      C.c_double, C.c_double, C.c_int, C.c_double, C.c_double,
                                      _dp, C.POINTER(BrinkmanStats)], C.c_int),
    "fp_green_apply_noalloc": ([C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
}

_lib = None


def load(path: str | None = None):
    """Load libfftperm.so (build it first with fft_method_test_gb300.build.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(
            "libfftperm.so is not built (expected at %s); run "
            "`python -c 'import __graft_entry__ as g; g.build()'`" % p)
    lib = C.CDLL(p)
    for name, (args, res) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


class FpError(RuntimeError):
    """A non-OK status from the C ABI."""

    def __init__(self, code: int, msg: str):
        super().__init__("fftperm error %d: %s" % (code, msg))
        self.code = code


def check(lib, handle, code: int):
    if code == FP_OK:
        return
    msg = lib.fp_last_error(handle).decode() if handle else "invalid handle"
    if code == FP_ERR_INVALID:
        # the reference throws std::invalid_argument here
        raise ValueError(msg)
    raise FpError(code, msg)
