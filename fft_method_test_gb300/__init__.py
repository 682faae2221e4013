"""GB300-native hot path of the FFT permeability solver (Bignonnet variational
method + MINRES, Brinkman iteration, velocity recovery).

The compute runs in hand-written CUDA kernels for sm_103a behind the C ABI of
include/fftperm.h (library: fft_method_test_gb300/_build/libfftperm.so, built
by ``fft_method_test_gb300.build.build()``).  ``permeability`` mirrors the
reference's C++ classes on top of that ABI; ``runner`` mirrors its .cfg-driven
runner and output files; ``geometry`` generates seeded
synthetic microstructures and reads the reference's .fgeo and text geometry
formats.
"""
from . import geometry  # noqa: F401

__all__ = ["geometry", "permeability", "runner", "build"]
