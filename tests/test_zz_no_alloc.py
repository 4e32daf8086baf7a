"""GPU: the allocation-free transform entry point (gl_ntt_noalloc), bit for bit
against the oracle and against the allocating entry point (gl_ntt / gl_intt),
on calls made back to back.

gl_ntt_noalloc serves callers that cannot allocate device memory: a worker
held to a device-memory budget that another framework has already reserved,
or a latency-critical thread that may not call cudaMalloc (which can
synchronise the whole device).  Its scratch is a fixed array inside the
library.  This file is collected last, so that a run stopping at its first
failure has run every other test first.
"""
import numpy as np
import pytest

from conftest import from_dev, to_dev

pytestmark = pytest.mark.gpu

# Consecutive calls share the fixed scratch: different lengths and directions
# back to back, the shortest and the longest accepted lengths, and inverse
# transforms at odd log2 lengths (unequal column and row passes).
CASES = [(1 << 16, 0), (1 << 20, 1), (1 << 13, 0), (1 << 13, 1), (1 << 17, 1), (1 << 20, 0),
         (1 << 15, 1)]


def test_noalloc_matches_oracle_and_allocating_entry_point(gl, cuda, oracle):
    L = gl._lib
    lib = L.load()
    stream = cuda.cuda.current_stream().cuda_stream
    dirs = {0: L.GL_FORWARD, 1: L.GL_INVERSE}
    inputs = [gl.fill_uniform(n, seed=0xA110C + n + d) for n, d in CASES]
    got = [to_dev(cuda, x) for x in inputs]
    want = [to_dev(cuda, x) for x in inputs]
    # The first call on the device looks up the fixed arrays (and loads the
    # device code): warm up on a buffer of its own before measuring memory.
    warm = to_dev(cuda, gl.fill_uniform(1 << 13, seed=1))
    assert lib.gl_ntt_noalloc(warm.data_ptr(), 1 << 13, L.GL_FORWARD, stream) == L.GL_OK
    cuda.cuda.synchronize()
    free_before = cuda.cuda.mem_get_info()[0]
    torch_before = cuda.cuda.memory_allocated()
    # Every device allocation the library itself would make fails meanwhile.
    lib.gl_debug_inject_alloc_failures(1 << 20)
    try:
        for (n, d), g in zip(CASES, got):
            assert lib.gl_ntt_noalloc(g.data_ptr(), n, dirs[d], stream) == L.GL_OK, (n, d)
        cuda.cuda.synchronize()
    finally:
        lib.gl_debug_inject_alloc_failures(0)
    assert cuda.cuda.mem_get_info()[0] == free_before
    assert cuda.cuda.memory_allocated() == torch_before
    for (n, d), x, g, w in zip(CASES, inputs, got, want):
        (gl.intt if d else gl.ntt)(w)
        out = from_dev(g)
        assert np.array_equal(out, (oracle.intt if d else oracle.ntt)(x)), (n, d)
        assert np.array_equal(out, from_dev(w)), (n, d)


def test_noalloc_rejects_lengths_beyond_its_scratch(gl, cuda):
    L = gl._lib
    lib = L.load()
    stream = cuda.cuda.current_stream().cuda_stream
    big = cuda.zeros(1 << 21, dtype=cuda.int64, device="cuda")
    assert lib.gl_ntt_noalloc(big.data_ptr(), 1 << 21, L.GL_FORWARD, stream) == L.GL_ERR_INVALID
    assert lib.gl_ntt_noalloc(big.data_ptr(), 7, L.GL_FORWARD, stream) == L.GL_ERR_UNSUPPORTED_SIZE
