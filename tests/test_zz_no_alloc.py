"""GPU: the allocation-free transform entry point (gl_ntt_noalloc) against the
allocating one (gl_ntt / gl_intt), bit for bit, on consecutive calls.

gl_ntt_noalloc serves callers that cannot allocate device memory (a worker
held to a device-memory budget another framework reserved, or a thread that
may not call cudaMalloc); its scratch is a fixed array inside the library.
This file is collected last so that a run stopping at its first failure has
run every other test first.
"""
import numpy as np
import pytest

from conftest import from_dev, to_dev

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point(gl, cuda):
    L = gl._lib
    lib = L.load()
    stream = cuda.cuda.current_stream().cuda_stream
    # Consecutive calls share the fixed scratch: different sizes and directions
    # back to back, including the largest accepted length.
    for n, direction in [(1 << 16, L.GL_FORWARD), (1 << 20, L.GL_INVERSE), (1 << 13, L.GL_FORWARD),
                         (1 << 20, L.GL_FORWARD)]:
        x = gl.fill_uniform(n, seed=0xA110C + n + direction)
        got, want = to_dev(cuda, x), to_dev(cuda, x)
        assert lib.gl_ntt_noalloc(got.data_ptr(), n, direction, stream) == L.GL_OK
        (gl.intt if direction == L.GL_INVERSE else gl.ntt)(want)
        assert np.array_equal(from_dev(got), from_dev(want)), (n, direction)


def test_noalloc_rejects_lengths_beyond_its_scratch(gl, cuda):
    L = gl._lib
    lib = L.load()
    stream = cuda.cuda.current_stream().cuda_stream
    big = cuda.zeros(1 << 21, dtype=cuda.int64, device="cuda")
    assert lib.gl_ntt_noalloc(big.data_ptr(), 1 << 21, L.GL_FORWARD, stream) == L.GL_ERR_INVALID
    assert lib.gl_ntt_noalloc(big.data_ptr(), 7, L.GL_FORWARD, stream) == L.GL_ERR_UNSUPPORTED_SIZE
