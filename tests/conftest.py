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


def rand_field(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.integers(0, 2**63, size=n, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, size=n, dtype=np.uint64)
    x[x >= np.uint64(P)] -= np.uint64(P)
    return x


def to_dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x).view(np.int64).copy()).cuda()


def from_dev(t):
    return t.cpu().numpy().view(np.uint64)
