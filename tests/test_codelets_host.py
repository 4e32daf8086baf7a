"""CPU: the device field arithmetic and the generated GPU codelets, compiled for
the host from the same headers (gl_field.cuh, gl_codelets.cuh), against the
oracle.  The device-only inline-PTX addition is covered by the GPU tests."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import P, ROOT, rand_field

CSRC = os.path.join(ROOT, "goldilocks_gb300", "csrc")

HARNESS = r"""
#include "gl_codelets.cuh"
extern "C" {
uint64_t h_add(uint64_t a, uint64_t b) { return gl_add(a, b); }
uint64_t h_sub(uint64_t a, uint64_t b) { return gl_sub(a, b); }
uint64_t h_mul(uint64_t a, uint64_t b) { return gl_mul(a, b); }
uint64_t h_shl(uint64_t a, uint32_t k) { return gl_shl_rt(a, k); }
uint64_t h_reduce128(uint64_t lo, uint64_t hi) { return gl_reduce128(lo, hi); }
int h_dft(int r, int inv, uint64_t *x) {
  switch (r * 2 + inv) {
%CASES%
  default: return -1;
  }
  return 0;
}
}
"""


def codelet_sizes():
    text = open(os.path.join(CSRC, "gl_codelets.cuh")).read()
    return sorted({int(m) for m in re.findall(r"struct gl_dft_impl<(\d+), (?:true|false)>", text)})


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    d = tmp_path_factory.mktemp("hostcodelets")
    cases = "\n".join("  case %d: gl_dft<%d, %s>(x); break;" % (r * 2 + i, r, "true" if i else "false")
                      for r in codelet_sizes() for i in (0, 1))
    src = d / "h.cpp"
    src.write_text(HARNESS.replace("%CASES%", cases))
    so = d / "h.so"
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I" + CSRC, str(src), "-o", str(so)],
                   check=True)
    lib = ctypes.CDLL(str(so))
    u64 = ctypes.c_uint64
    for f in ("h_add", "h_sub", "h_mul", "h_reduce128"):
        getattr(lib, f).restype = u64
        getattr(lib, f).argtypes = [u64, u64]
    lib.h_shl.restype = u64
    lib.h_shl.argtypes = [u64, ctypes.c_uint32]
    lib.h_dft.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    return lib


def test_field_ops(host):
    rng = np.random.default_rng(11)
    vals = [0, 1, 2, P - 1, P - 2, 2**32 - 1, 2**32, 2**32 + 1, 2**63, P - 2**32, 2**64 - 2**33] + \
        [int(v) % P for v in rng.integers(0, 2**63, 200, dtype=np.uint64) * 2 + 1]
    vals = [v % P for v in vals]
    for a in vals:
        for b in vals[:60]:
            assert host.h_add(a, b) == (a + b) % P
            assert host.h_sub(a, b) == (a - b) % P
            assert host.h_mul(a, b) == a * b % P
        for k in list(range(0, 200)) + [384, 1000]:
            assert host.h_shl(a, k) == a * pow(2, k, P) % P, (a, k)
    for lo, hi in [(2**64 - 1, 2**64 - 1), (0, 2**64 - 1), (2**64 - 1, 0), (5, 2**32)]:
        assert host.h_reduce128(lo, hi) == (hi * 2**64 + lo) % P


def test_codelets_against_oracle(host, oracle):
    for r in codelet_sizes():
        for inv in (0, 1):
            for seed in range(3):
                x = rand_field(r, seed=100 * r + seed)
                if seed == 1:
                    x[:] = P - 1
                y = x.copy()
                assert host.h_dft(r, inv, y.ctypes.data) == 0
                if inv:
                    want = oracle.intt(x)  # scaled by 1/r
                    scale = r % P
                    want = np.array([int(v) * scale % P for v in want], dtype=np.uint64)
                else:
                    want = oracle.naive_ntt(x)
                assert np.array_equal(y, want), (r, inv)
