import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libfftperm.so")


@pytest.fixture(scope="session")
def restatement():
    import oracle as orc

    orc.build_restatement()
    return orc.Restatement()


@pytest.fixture(scope="session")
def reference():
    import oracle as orc

    if not orc.reference_available():
        pytest.skip("reference build (oracle/_ref) not present on this host")
    return orc.Reference()


@pytest.fixture(scope="session")
def gpu_lib():
    """Loads libfftperm.so (building it if needed) and checks a GPU is visible."""
    from fft_method_test_gb300 import _capi, build

    build.build()
    lib = _capi.load()
    return lib


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)
