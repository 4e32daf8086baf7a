"""GPU parity of the circular convolution (ntt/src/convolve.rs:13-20) against
the oracle: the reference's KAT (convolve.rs:44-60) on Field words and on
canonical values, then random sequences at every schedule kind (one element,
one pass, two passes, three passes, run-time radices), one b_hat shared by a
batch or one per sequence, device and host memory."""
import numpy as np
import pytest

from conftest import from_dev, rand_field, to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("montgomery", [True, False])
def test_reference_kat(gl, oracle, cuda, montgomery):
    a, b, want = [1, 2, 3], [4, 5, 6], [31, 31, 28]
    conv = oracle.to_mont if montgomery else (lambda v: np.array(v, dtype=np.uint64))
    bh = to_dev(cuda, conv(b))
    gl.ntt(bh)
    d = to_dev(cuda, conv(a))
    gl.convolve(d, bh, montgomery=montgomery)
    got = from_dev(d)
    assert (oracle.from_mont(got) if montgomery else got).tolist() == want


@pytest.mark.parametrize("n,count,shared", [(1, 7, False), (1, 5, True), (2, 3, False), (16, 9, True),
                                            (60, 4, False), (4096, 3, True), (3 << 10, 2, False),
                                            (1 << 14, 3, True), (1 << 16, 2, False),
                                            (255 << 8, 2, True), (1 << 20, 1, True),
                                            (17 << 16, 1, False), (15 << 14, 2, True)])
@pytest.mark.parametrize("montgomery", [True, False])
def test_matches_oracle(gl, oracle, cuda, n, count, shared, montgomery):
    a = rand_field(n * count, seed=n + count)
    b = rand_field(n * (1 if shared else count), seed=3 * n + count)
    d = to_dev(cuda, a)
    gl.convolve(d, to_dev(cuda, b), size=n, montgomery=montgomery)
    assert np.array_equal(from_dev(d), oracle.convolve(a, b, size=n, montgomery=montgomery))


def test_good_thomas_row_pass(gl, oracle, cuda):
    """16 711 680 = 4096 x 4080: the product is fused into the 4080-point row
    pass, which runs its inner 15 x 17 transform in the Good-Thomas form."""
    n = 16711680
    assert "Good-Thomas" in gl.strategy(n).describe()
    a = gl.fill_uniform(n, seed=0xC2, offset=0)
    b = gl.fill_uniform(n, seed=0xC3, offset=0)
    d = to_dev(cuda, a)
    gl.convolve(d, to_dev(cuda, b))
    assert np.array_equal(from_dev(d), oracle.convolve(a, b))


def test_three_pass_size(gl, oracle, cuda):
    n = 1 << 25
    a = gl.fill_uniform(n, seed=0xC0, offset=0)
    b = gl.fill_uniform(n, seed=0xC1, offset=0)
    d = to_dev(cuda, a)
    gl.convolve(d, to_dev(cuda, b))
    assert np.array_equal(from_dev(d), oracle.convolve(a, b))


def test_host_memory(gl, oracle):
    n, count = 1 << 12, 3
    a = rand_field(n * count, seed=5)
    b = rand_field(n, seed=6)
    y = a.copy()
    gl.convolve(y, b, size=n)
    assert np.array_equal(y, oracle.convolve(a, b, size=n))


def test_errors(gl, cuda):
    d = cuda.zeros(12, dtype=cuda.int64, device="cuda")
    with pytest.raises(ValueError, match="is not a supported NTT size"):
        gl.convolve(d[:7], d[:7])
    with pytest.raises(ValueError, match="b_hat must hold"):
        gl.convolve(d, d[:8], size=4)
    with pytest.raises(ValueError, match="both"):
        gl.convolve(d, np.zeros(12, dtype=np.uint64))
