"""GPU parity of the lengths with a prime factor 257 or 65537 (the Rader step,
ntt/src/ntt/rader.rs:19-93, in front of the ordinary plans) against the
oracle's runtime Rader plans: single transforms both ways, batches, column
batches, the LDE, the convolution, the batch and server entry points."""
import numpy as np
import pytest

from conftest import from_dev, rand_field, to_dev

pytestmark = pytest.mark.gpu

SIZES = [257, 514, 771, 1285, 257 * 16, 257 * 17, 65535, 257 * 4096, 65537, 65537 * 2, 65537 * 3,
         65537 * 16, 257 * 65536, 65537 * 257]


@pytest.mark.parametrize("n", SIZES)
def test_forward_inverse_match_oracle(gl, oracle, cuda, n):
    x = gl.fill_uniform(n, seed=n, offset=0)
    d = to_dev(cuda, x)
    gl.ntt(d)
    y = from_dev(d)
    assert np.array_equal(y, oracle.ntt(x)), gl.strategy(n).describe()
    gl.intt(d)
    assert np.array_equal(from_dev(d), x)
    d = to_dev(cuda, y)
    gl.intt(d)
    assert np.array_equal(from_dev(d), oracle.intt(y))


@pytest.mark.parametrize("n,count", [(257, 9), (514, 5), (65537, 3)])
def test_batched(gl, oracle, cuda, n, count):
    x = rand_field(n * count, seed=count)
    d = to_dev(cuda, x)
    gl.strategy(n).ntt(d)
    assert np.array_equal(from_dev(d), oracle.ntt(x, size=n))
    y = x.copy()
    gl.strategy(n).ntt(y)           # host memory
    assert np.array_equal(y, oracle.ntt(x, size=n))


@pytest.mark.parametrize("rows,cols", [(257, 7), (514, 3), (65537, 2)])
def test_columns(gl, oracle, cuda, rows, cols):
    L = gl._lib
    x = rand_field(rows * cols, seed=rows + cols)
    d = to_dev(cuda, x)
    s = cuda.cuda.current_stream().cuda_stream
    assert L.load().gl_ntt_columns(d.data_ptr(), rows, cols, L.GL_FORWARD, L.GL_MEM_DEVICE, s) == 0
    got = from_dev(d).reshape(rows, cols)
    for c in range(cols):
        assert np.array_equal(got[:, c], oracle.ntt(x.reshape(rows, cols)[:, c].copy())), c
    assert L.load().gl_ntt_columns(d.data_ptr(), rows, cols, L.GL_INVERSE, L.GL_MEM_DEVICE, s) == 0
    assert np.array_equal(from_dev(d), x)


@pytest.mark.parametrize("n,cols,blowup", [(257, 3, 4), (16, 2, 257), (4, 1, 65537), (3, 2, 1 << 14)])
def test_lde(gl, oracle, cuda, n, cols, blowup):
    """Rader plans on either side of the LDE, and a two-pass target whose
    factor n2 does not divide n (the separate coset-and-padding pass)."""
    L = gl._lib
    x = rand_field(n * cols, seed=n * cols + blowup)
    d = to_dev(cuda, x)
    out = cuda.empty(n * blowup * cols, dtype=cuda.int64, device="cuda")
    s = cuda.cuda.current_stream().cuda_stream
    assert L.load().gl_coset_lde(d.data_ptr(), out.data_ptr(), n, cols, blowup, 7, L.GL_MEM_DEVICE, s) == 0
    assert np.array_equal(from_dev(out), oracle.coset_lde(x, n, cols, blowup, 7))


@pytest.mark.parametrize("n,count,shared", [(257, 3, True), (514, 2, False), (65537, 1, True)])
def test_convolve(gl, oracle, cuda, n, count, shared):
    a = rand_field(n * count, seed=n)
    b = rand_field(n * (1 if shared else count), seed=n + 1)
    d = to_dev(cuda, a)
    gl.convolve(d, to_dev(cuda, b), size=n)
    assert np.array_equal(from_dev(d), oracle.convolve(a, b, size=n))


def test_batch_and_server_entry_points(gl, oracle, cuda):
    from goldilocks_gb300 import batch as B
    from goldilocks_gb300 import server as S
    sizes = [257 * 4, 4096, 65537, 771]
    xs = [rand_field(n, seed=i) for i, n in enumerate(sizes)]
    ds = [to_dev(cuda, x) for x in xs]
    B.run([(d, 0) for d in ds], mode=B.PERSISTENT)
    for x, d in zip(xs, ds):
        assert np.array_equal(from_dev(d), oracle.ntt(x))
    n, cols = 257 * 16, 3
    x = rand_field(n * cols, seed=99)
    inp = to_dev(cuda, x)
    out = cuda.empty(4 * n * cols, dtype=cuda.int64, device="cuda")
    with S.Server(budget_bytes=1 << 30, slots=2, max_batch=4) as srv:
        rid = srv.submit(S.GL_OP_LDE, n, cols, inp, out, blowup=4, shift=7)
        assert srv.wait(rid) == gl._lib.GL_OK
    assert np.array_equal(from_dev(out), oracle.coset_lde(x, n, cols, 4, 7))
