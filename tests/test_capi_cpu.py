"""The C ABI library builds, loads and exports every symbol of include/fftperm.h.
No compute call is made (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np

import pytest

from conftest import ROOT


def declared_symbols():
    with open(os.path.join(ROOT, "include", "fftperm.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fp_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from fft_method_test_gb300 import _capi, build

    path = build.build()
    lib = C.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 18
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(_capi.EXPORTED)


def test_python_mirror_loads_and_validates_without_gpu():
    from fft_method_test_gb300 import _capi
    from fft_method_test_gb300.permeability import MinresSolver, PermeabilityTensor

    _capi.load()
    with pytest.raises(ValueError):
        MinresSolver(0.0, 10)
    t = PermeabilityTensor()
    t.set_column(1, [1.0, 2.0, 3.0])
    assert list(t.data()[[1, 4, 7]]) == [-1.0, -2.0, -3.0]
    with pytest.raises(IndexError):
        t.set_column(3, [0, 0, 0])


def test_group_and_batch_entries_reject_bad_arguments_without_gpu():
    """The group, block and grouped-batch entries check their arguments before
    any CUDA call (status FP_ERR_INVALID)."""
    import ctypes as C

    from fft_method_test_gb300 import _capi
    from fft_method_test_gb300.permeability import batch_solve_permeability

    lib = _capi.load()
    K = np.zeros(9)
    assert lib.fp_group_solve_permeability(0, None, 1e-7, 100, K, None) == _capi.FP_ERR_INVALID
    hs = (C.c_void_p * 2)(None, None)
    assert lib.fp_group_solve_permeability(2, hs, 1e-7, 100, K, None) == _capi.FP_ERR_INVALID
    assert lib.fp_solve_permeability_block(None, 1e-7, 100, K, None) == _capi.FP_ERR_INVALID
    mask = np.ones((8, 8, 8), np.uint8)
    with pytest.raises(ValueError):
        batch_solve_permeability([mask], max_group=0)
    with pytest.raises(ValueError):
        batch_solve_permeability([mask], concurrency=0, max_group=4)


@pytest.mark.parametrize("precision", ["FFT_METHOD_PRECISION_DOUBLE", "FFT_METHOD_PRECISION_FLOAT"])
def test_cpp_adapters_compile_against_reference(precision):
    """The C++ drop-ins (CudaFFTBackend : IFFTBackend, CudaVariationalOperator :
    ILinearOperator, cuda_solve_one_direction) compile against the reference's
    own headers in both of its precisions."""
    import shutil
    import subprocess

    from __graft_entry__ import REFERENCE_DIR as ref

    if not os.path.isdir(os.path.join(ref, "src")):
        pytest.skip("reference sources not present on this host")
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    src = os.path.join(ROOT, "fft_method_test_gb300", "host", "CudaBackends.cpp")
    r = subprocess.run([gxx, "-std=c++20", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                        "-D%s=1" % precision, "-I" + os.path.join(ref, "src"),
                        "-I" + os.path.join(ref, "include"), "-I" + os.path.join(ROOT, "include"), src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_fvel_writer_matches_the_reference_layout(tmp_path):
    """fp_write_fvel writes the reference's .fvel layout
    (src/app/PermeabilityRunner.cpp:109-159): 72-byte header, AoS doubles.
    Host code only: no GPU needed."""
    import struct

    from fft_method_test_gb300.permeability import read_fvel, write_fvel

    rng = np.random.default_rng(5)
    v = rng.standard_normal((3, 4, 5, 6))
    path = str(tmp_path / "out_axis1.fvel")
    write_fvel(path, v, 0.35, 1.5, (1.0, 0.0, 0.0))
    raw = open(path, "rb").read()
    assert len(raw) == 72 + 3 * 8 * v[0].size
    assert raw[:4] == b"FVEL" and raw[4] == 1 and raw[5:8] == b"\0\0\0"
    assert struct.unpack("<3Q", raw[8:32]) == (6, 5, 4)
    assert struct.unpack("<5d", raw[32:72]) == (0.35, 1.5, 1.0, 0.0, 0.0)
    first = struct.unpack("<3d", raw[72:96])
    assert first == (v[0, 0, 0, 0], v[1, 0, 0, 0], v[2, 0, 0, 0])
    r = read_fvel(path)
    assert np.array_equal(r["velocity"], v) and r["porosity"] == 0.35
