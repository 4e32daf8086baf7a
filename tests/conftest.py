import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

P = 0xFFFF_FFFF_0000_0001


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def gl():
    from goldilocks_gb300 import build
    build.build()
    import goldilocks_gb300
    goldilocks_gb300._lib.load()
    return goldilocks_gb300


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch


@pytest.fixture(autouse=True)
def _device_index_checks(request):
    """Under a debug build of the library (-DGL_DEVICE_CHECKS, selected with
    GOLDILOCKS_BUILD_DIR / GOLDILOCKS_NVCC_FLAGS), every GPU test must leave
    the device-side index checks clean."""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    import ctypes
    from goldilocks_gb300 import _lib as L
    lib = L.load()
    if not lib.gl_debug_checks_enabled():
        return
    flags = ctypes.c_uint32(0)
    assert lib.gl_debug_check_status(ctypes.byref(flags)) == L.GL_OK
    assert flags.value == 0, "device index check failed (bits %d)" % flags.value


def rand_field(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.integers(0, 2**63, size=n, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, size=n, dtype=np.uint64)
    x[x >= np.uint64(P)] -= np.uint64(P)
    return x


def to_dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x).view(np.int64).copy()).cuda()


def from_dev(t):
    return t.cpu().numpy().view(np.uint64)
