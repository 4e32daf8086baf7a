"""GPU: the opt-in alternatives selected by environment variables give the
same results as the defaults (each in a fresh process, where the switches are
read once):
  GOLDILOCKS_PASS_TWIDDLE=full   full per-plan pass-twiddle tables
  GOLDILOCKS_PASS_LANES=4        four-lane pass kernels for every pass size
  GOLDILOCKS_HOST_STAGING=1      host buffers staged through device memory
                                 instead of read in place"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHECK = r"""
import numpy as np, torch
import goldilocks_gb300 as gl
import oracle
from conftest import rand_field, to_dev, from_dev
oracle.build()
torch.cuda.set_device(0)
for n in (1 << 12, 1 << 16, 1 << 20, 3 << 20, 17 << 16, 1 << 25):
    x = rand_field(n, n % 1000)
    want = oracle.ntt(x) if n <= (1 << 22) else None
    d = to_dev(torch, x)
    gl.ntt(d)
    y = from_dev(d)
    if want is not None:
        assert np.array_equal(y, want), ("device", n)
    gl.intt(d)
    assert np.array_equal(from_dev(d), x), ("roundtrip", n)
    pinned = torch.empty(n, dtype=torch.int64, pin_memory=True)
    h = pinned.numpy().view(np.uint64)
    h[:] = x
    gl.ntt(h)
    assert np.array_equal(h, y), ("host", n)
    gl.intt(h)
    assert np.array_equal(h, x), ("host roundtrip", n)
print("ok")
"""


@pytest.mark.parametrize("var,value", [("GOLDILOCKS_PASS_TWIDDLE", "full"), ("GOLDILOCKS_PASS_LANES", "4"),
                                       ("GOLDILOCKS_HOST_STAGING", "1")])
def test_environment_variant_matches_oracle(var, value):
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([ROOT, os.path.join(ROOT, "tests")]))
    env[var] = value
    out = subprocess.run([sys.executable, "-c", CHECK], env=env, capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stdout + out.stderr
