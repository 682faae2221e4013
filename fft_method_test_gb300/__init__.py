"""GB300-native hot path of the FFT permeability solver (Bignonnet variational
method + MINRES, Brinkman iteration, velocity recovery).

The compute runs in hand-written CUDA kernels for sm_103a behind the C ABI of
include/fftperm.h (library: fft_method_test_gb300/_build/libfftperm.so, built
by ``fft_method_test_gb300.build.build()``).  ``permeability`` mirrors the
reference's C++ classes on top of that ABI; ``geometry`` generates seeded
synthetic microstructures and reads/writes the reference's .fgeo format.
"""
from . import geometry  # noqa: F401

__all__ = ["geometry", "permeability", "build"]
