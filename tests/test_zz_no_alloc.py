"""fp_green_apply_noalloc: the Green-operator apply for callers that may not
allocate device memory (a caller inside another framework's memory manager,
or a latency-critical loop that cannot afford cudaMalloc's synchronisation).

The entry point works in a fixed file-scope device array instead of
allocating.  Its output must equal the regular entry point's (fp_green_apply)
within the Green-apply tolerance of the other tests (1e-12 relative), on two
calls in a row -- the second call runs on the array the first one left
behind.  This file is collected last so that a failure here comes after every
other test has run; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _noalloc(lib, shape, f_dev, u_dev, stream, h=1.0, mu=1.0, p_radius=2):
    nz, ny, nx = shape
    return lib.fp_green_apply_noalloc(nx, ny, nz, h, mu, p_radius, C.c_void_p(f_dev.data_ptr()),
                                      C.c_void_p(u_dev.data_ptr()), C.c_void_p(stream))


@pytest.mark.parametrize("shape,mu", [((16, 16, 16), 1.0), ((12, 20, 30), 0.7)])
def test_noalloc_green_apply_matches_regular_entry_point(gpu_lib, shape, mu):
    import torch

    from fft_method_test_gb300.permeability import PermeabilityProblem

    lib = gpu_lib
    rng = np.random.default_rng(17)
    stream = torch.cuda.current_stream()
    with PermeabilityProblem(shape, mu=mu, precision="fp64") as p:
        for call in range(2):  # two calls in a row share the scratch array
            f = rng.uniform(-1.0, 1.0, (3,) + shape)
            want = p.green_apply(f)
            f_dev = torch.from_numpy(f.copy()).cuda()
            u_dev = torch.full_like(f_dev, float("nan"))
            rc = _noalloc(lib, shape, f_dev, u_dev, stream.cuda_stream, mu=mu)
            assert rc == 0, (call, rc)
            stream.synchronize()
            got = u_dev.cpu().numpy()
            assert rel_err(got, want) < 1e-12, call


def test_noalloc_rejects_grids_beyond_its_array(gpu_lib):
    import torch

    lib = gpu_lib
    f_dev = torch.zeros(3 * 8, dtype=torch.float64, device="cuda")
    u_dev = torch.zeros_like(f_dev)
    # 80^3 voxels exceed the 262144-voxel limit: rejected before any launch
    assert _noalloc(lib, (80, 80, 80), f_dev, u_dev, 0) == 1
    # an edge that is not a product of 2, 3, 5 is unsupported
    assert _noalloc(lib, (7, 8, 8), f_dev, u_dev, 0) == 4
