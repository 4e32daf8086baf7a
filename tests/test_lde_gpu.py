"""GPU parity of the column-batched transforms and the coset LDE against the
oracle's composition (intt, coset multiply, zero pad, ntt)."""
import ctypes

import numpy as np
import pytest

from conftest import P, from_dev, rand_field, to_dev

pytestmark = pytest.mark.gpu


def cols_call(gl, cuda, d, rows, cols, inverse=False):
    L = gl._lib
    rc = L.load().gl_ntt_columns(d.data_ptr(), rows, cols, L.GL_INVERSE if inverse else L.GL_FORWARD,
                                 L.GL_MEM_DEVICE, cuda.cuda.current_stream().cuda_stream)
    assert rc == 0, rc


def lde_call(gl, cuda, d, out, n, cols, blowup, shift):
    L = gl._lib
    rc = L.load().gl_coset_lde(d.data_ptr(), out.data_ptr(), n, cols, blowup, shift,
                               L.GL_MEM_DEVICE, cuda.cuda.current_stream().cuda_stream)
    assert rc == 0, rc


@pytest.mark.parametrize("rows,cols", [(8, 3), (64, 5), (1024, 4), (4096, 7), (1 << 13, 4),
                                       (1 << 14, 6), (1 << 16, 2), (1 << 12, 64), (1 << 16, 1),
                                       (2, 5)])
def test_columns_match_oracle(gl, oracle, cuda, rows, cols):
    x = rand_field(rows * cols, seed=rows + cols)
    d = to_dev(cuda, x)
    cols_call(gl, cuda, d, rows, cols)
    got = from_dev(d).reshape(rows, cols)
    xm = x.reshape(rows, cols)
    for c in range(cols):
        assert np.array_equal(got[:, c], oracle.ntt(xm[:, c].copy())), c
    cols_call(gl, cuda, d, rows, cols, inverse=True)
    assert np.array_equal(from_dev(d), x)


@pytest.mark.parametrize("n,cols,blowup", [(16, 3, 4), (64, 4, 2), (1024, 8, 4), (4096, 5, 4),
                                           (1 << 13, 4, 2), (1 << 14, 4, 4), (1 << 12, 16, 8),
                                           (1024, 3, 1), (1 << 16, 2, 1), (2, 3, 4), (1, 4, 8)])
def test_lde_matches_oracle(gl, oracle, cuda, n, cols, blowup):
    x = rand_field(n * cols, seed=n * cols + blowup)
    d = to_dev(cuda, x)
    out = cuda.empty(n * blowup * cols, dtype=cuda.int64, device="cuda")
    lde_call(gl, cuda, d, out, n, cols, blowup, 7)
    assert np.array_equal(from_dev(out), oracle.coset_lde(x, n, cols, blowup, 7))


# From 2^16 coefficients the LDE runs one length-n transform per coset of the
# n-th roots (rows b j + k of the output), reading the coefficients with the
# factor (g w^k)^i: two-pass and three-pass-free lengths, one and several
# columns, mixed radix, blowups 2 to 8.
@pytest.mark.parametrize("n,cols,blowup", [(1 << 16, 3, 4), (1 << 17, 1, 2), (3 << 16, 2, 4),
                                           (1 << 16, 1, 8), (17 << 12, 5, 2)])
def test_lde_per_coset_transforms(gl, oracle, cuda, n, cols, blowup):
    x = rand_field(n * cols, seed=n + cols + blowup)
    d = to_dev(cuda, x)
    out = cuda.empty(n * blowup * cols, dtype=cuda.int64, device="cuda")
    lde_call(gl, cuda, d, out, n, cols, blowup, 7)
    assert np.array_equal(from_dev(out), oracle.coset_lde(x, n, cols, blowup, 7))


def test_lde_host_memory_and_shift(gl, oracle):
    n, cols, blowup, shift = 1024, 3, 4, 2717
    x = rand_field(n * cols, seed=5)
    out = np.zeros(n * cols * blowup, dtype=np.uint64)
    L = gl._lib
    rc = L.load().gl_coset_lde(x.ctypes.data, out.ctypes.data, n, cols, blowup, shift, L.GL_MEM_HOST, None)
    assert rc == 0
    assert np.array_equal(out, oracle.coset_lde(x, n, cols, blowup, shift))


def test_lde_full_size_sampled_columns(gl, oracle, cuda):
    """2^20 x 256 -> 2^22 x 256 (the commit-matrix shape); 16 seeded columns
    (with the first and the last) checked against the oracle, and every column
    through the round trip below."""
    n, cols, blowup = 1 << 20, 256, 4
    x = gl.fill_uniform(n * cols, seed=0x1DE)
    d = to_dev(cuda, x)
    out = cuda.empty(n * blowup * cols, dtype=cuda.int64, device="cuda")
    lde_call(gl, cuda, d, out, n, cols, blowup, 7)
    res = out.view(n * blowup, cols)
    xm = x.reshape(n, cols)
    rng = np.random.default_rng(0x1DE)
    picked = sorted({0, cols - 1, *rng.choice(cols, 14, replace=False).tolist()})
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=8) as ex:
        wants = list(ex.map(lambda c: oracle.coset_lde(xm[:, c].copy(), n, 1, blowup, 7), picked))
    for c, want in zip(picked, wants):
        assert np.array_equal(from_dev(res[:, c].contiguous()), want), c
    # Round trip on all columns: intt(4n) of the LDE, unshifted, is the
    # zero-padded coefficient vector; its top 3n rows must vanish.
    cols_call(gl, cuda, out, n * blowup, cols, inverse=True)
    tail = res[n:]
    assert int(cuda.count_nonzero(tail)) == 0


def test_lde_three_pass_target(gl, oracle, cuda):
    """n = 2^23 with blowup 8 extends to 2^26: the forward transform has three
    passes, the coset factor and the zero padding apply to the first."""
    n, cols, blowup = 1 << 23, 1, 8
    x = gl.fill_uniform(n * cols, seed=0x3D)
    d = to_dev(cuda, x)
    out = cuda.empty(n * blowup * cols, dtype=cuda.int64, device="cuda")
    lde_call(gl, cuda, d, out, n, cols, blowup, 7)
    assert np.array_equal(from_dev(out), oracle.coset_lde(x, n, cols, blowup, 7))
