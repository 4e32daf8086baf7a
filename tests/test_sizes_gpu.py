"""GPU parity over the size space: every divisor of p - 1 up to 2^17 (the
reference plans any divisor: ntt/src/ntt/mod.rs:48-78), larger mixed-radix
lengths, and batched / column / LDE calls at such lengths, against the
oracle.  Lengths with a factor 257 or 65537 take the Rader step; the others
the compiled or run-time-radix pass kernels."""
import numpy as np
import pytest

from conftest import from_dev, rand_field, to_dev

pytestmark = pytest.mark.gpu


def supported(gl, n):
    try:
        gl.strategy(n)
        return True
    except ValueError:
        return False


def test_every_divisor_up_to_2p17(gl, oracle, cuda):
    sizes = [n for n in gl.divisors() if 2 <= n <= 1 << 17]
    assert len(sizes) == 153  # 45 of them with a factor 257 or 65537
    for n in sizes:
        assert supported(gl, n), n
        x = rand_field(n * 3, seed=n)
        d = to_dev(cuda, x)
        gl.strategy(n).ntt(d)
        assert np.array_equal(from_dev(d), oracle.ntt(x, size=n)), n
        gl.strategy(n).intt(d)
        assert np.array_equal(from_dev(d), x), n


@pytest.mark.parametrize("n", [3 << 20, 5 << 18, 17 << 20, 15 << 20, 51 << 18, 255 << 14,
                               3 << 24, 85 << 20])
def test_large_mixed_radix_sizes(gl, oracle, cuda, n):
    x = gl.fill_uniform(n, seed=0x51E5, offset=n)
    d = to_dev(cuda, x)
    gl.ntt(d)
    assert np.array_equal(from_dev(d), oracle.ntt(x)), gl.strategy(n).describe()
    gl.intt(d)
    assert np.array_equal(from_dev(d), x)


@pytest.mark.parametrize("n", [1536 << 11, 2560 << 11, 3072 << 12, 3840 << 12, 1280 << 10, 1920 << 11,
                               2176 << 11, 2040 << 11, 1088 << 10, 1360 << 11, 1632 << 11, 2720 << 12,
                               3264 << 12, 393216, 327680, 245760, 196608, 278528, 522240, 208896,
                               174080, 417792, 491520])
def test_compiled_mixed_radix_pass_shapes(gl, oracle, cuda, n):
    """Lengths whose default split has a compiled mixed-radix pass (the
    gl_kern_mixed35 and gl_kern_mixed17 shapes), forward and inverse, against
    the oracle."""
    x = gl.fill_uniform(n, seed=0xC0DE, offset=n)
    d = to_dev(cuda, x)
    gl.ntt(d)
    assert np.array_equal(from_dev(d), oracle.ntt(x)), gl.strategy(n).describe()
    gl.intt(d)
    assert np.array_equal(from_dev(d), x)


@pytest.mark.parametrize("n,count", [(15, 1000), (255, 77), (3840, 9), (12288, 5), (17 << 10, 3)])
def test_batched_mixed_radix(gl, oracle, cuda, n, count):
    x = rand_field(n * count, seed=n + count)
    d = to_dev(cuda, x)
    gl.strategy(n).ntt(d)
    assert np.array_equal(from_dev(d), oracle.ntt(x, size=n))


@pytest.mark.parametrize("rows,cols", [(3 << 10, 5), (255, 8), (17 << 12, 3)])
def test_columns_mixed_radix(gl, oracle, cuda, rows, cols):
    L = gl._lib
    x = rand_field(rows * cols, seed=rows * cols)
    d = to_dev(cuda, x)
    rc = L.load().gl_ntt_columns(d.data_ptr(), rows, cols, L.GL_FORWARD, L.GL_MEM_DEVICE,
                                 cuda.cuda.current_stream().cuda_stream)
    assert rc == 0
    got = from_dev(d).reshape(rows, cols)
    xm = x.reshape(rows, cols)
    for c in range(cols):
        assert np.array_equal(got[:, c], oracle.ntt(xm[:, c].copy())), c


@pytest.mark.parametrize("n,cols,blowup", [(3 << 12, 3, 4), (255 << 4, 2, 4), (5 << 14, 1, 2)])
def test_lde_mixed_radix(gl, oracle, cuda, n, cols, blowup):
    L = gl._lib
    x = rand_field(n * cols, seed=n + cols)
    d = to_dev(cuda, x)
    out = cuda.empty(n * blowup * cols, dtype=cuda.int64, device="cuda")
    rc = L.load().gl_coset_lde(d.data_ptr(), out.data_ptr(), n, cols, blowup, 7, L.GL_MEM_DEVICE,
                               cuda.cuda.current_stream().cuda_stream)
    assert rc == 0
    assert np.array_equal(from_dev(out), oracle.coset_lde(x, n, cols, blowup, 7))
