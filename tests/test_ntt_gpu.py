"""GPU parity: the CUDA transforms against the CPU oracle, bit for bit.

Follows the reference's test strategy (ntt/src/ntt/mod.rs:127-139 compare with
the naive DFT; naive.rs:230-275 round trips) at sizes the oracle finishes in
seconds, plus size-independent properties at the configured full sizes.
"""
import numpy as np
import pytest

from conftest import P, from_dev, rand_field, to_dev

pytestmark = pytest.mark.gpu

@pytest.mark.parametrize("n", [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192,
                               1 << 14, 1 << 15, 1 << 16, 1 << 17, 1 << 18, 1 << 20])
def test_forward_matches_oracle(gl, oracle, cuda, n):
    x = rand_field(n, seed=n)
    d = to_dev(cuda, x)
    gl.ntt(d)
    assert np.array_equal(from_dev(d), oracle.ntt(x))


@pytest.mark.parametrize("n", [2, 8, 64, 1024, 4096, 1 << 13, 1 << 16, 1 << 19])
def test_inverse_matches_oracle(gl, oracle, cuda, n):
    x = rand_field(n, seed=n + 1)
    d = to_dev(cuda, x)
    gl.intt(d)
    assert np.array_equal(from_dev(d), oracle.intt(x))


@pytest.mark.parametrize("n", [16, 4096, 1 << 16])
def test_host_memory_path(gl, oracle, n):
    x = rand_field(n, seed=7 * n)
    y = x.copy()
    gl.ntt(y)
    assert np.array_equal(y, oracle.ntt(x))
    gl.intt(y)
    assert np.array_equal(y, x)


@pytest.mark.parametrize("n,count", [(4096, 3), (1 << 16, 2), (1 << 22, 1), (1 << 25, 1), (257 * 16, 3),
                                     (3 << 20, 1)])
def test_pinned_host_memory_in_place(gl, oracle, cuda, n, count):
    """Page-locked host buffers are read and written by the kernels in place
    (no staging copies); pageable ones (numpy) are staged."""
    t = cuda.empty(n * count, dtype=cuda.int64, pin_memory=True)
    h = t.numpy().view(np.uint64)
    x = gl.fill_uniform(n * count, seed=n + count)
    h[:] = x
    gl.strategy(n).ntt(h)
    assert np.array_equal(h, oracle.ntt(x, size=n))
    gl.strategy(n).intt(h)
    assert np.array_equal(h, x)


# Whole-transform lengths 512-4096 run one transform per CTA while the wider
# kernel would leave SMs without a CTA (fewer than 4 x 152 transforms of
# 1024-4096 points, 8 x 152 of 512) and the wide kernel above that.
@pytest.mark.parametrize("n,count", [(8, 1000), (64, 333), (1024, 37), (4096, 9), (1 << 14, 5),
                                     (2048, 1), (512, 3), (4096, 700), (1024, 650), (512, 1300)])
def test_batched_plan(gl, oracle, cuda, n, count):
    x = rand_field(n * count, seed=count)
    d = to_dev(cuda, x)
    gl.strategy(n).ntt(d)
    assert np.array_equal(from_dev(d), oracle.ntt(x, size=n))
    gl.strategy(n).intt(d)
    assert np.array_equal(from_dev(d), x)


def test_mixed_radix_16711680(gl, oracle, cuda):
    n = 16711680
    x = gl.fill_uniform(n, seed=0x5EED0002)
    d = to_dev(cuda, x)
    gl.ntt(d)
    assert np.array_equal(from_dev(d), oracle.ntt(x))
    gl.intt(d)
    assert np.array_equal(from_dev(d), x)


@pytest.mark.parametrize("n", [1 << 20, 1 << 22, 1 << 24, 16711680])
def test_full_sizes_match_oracle(gl, oracle, cuda, n):
    """Bit-exact forward and inverse at the configured full sizes."""
    x = gl.fill_uniform(n, seed=0x5EED0001, offset=n)
    d = to_dev(cuda, x)
    gl.ntt(d)
    f = from_dev(d)
    assert np.array_equal(f, oracle.ntt(x))
    gl.intt(d)
    assert np.array_equal(from_dev(d), x)


def test_linearity_full_size(gl, cuda):
    """NTT(x + y) = NTT(x) + NTT(y) and X[0] = sum(x) at n = 2^24."""
    n = 1 << 24
    x = gl.fill_uniform(n, seed=24)
    y = gl.fill_uniform(n, seed=124)
    outs = []
    for v in (x, y, None):
        if v is None:
            s = x + y
            s = np.where((s < x) | (s >= np.uint64(P)), s - np.uint64(P), s)
            v = s
        d = to_dev(cuda, v)
        gl.ntt(d)
        outs.append(from_dev(d))
    fx, fy, fs = outs
    t = fx + fy
    t = np.where((t < fx) | (t >= np.uint64(P)), t - np.uint64(P), t)
    assert np.array_equal(fs, t)
    lo = int((x & np.uint64(0xFFFFFFFF)).sum())
    hi = int((x >> np.uint64(32)).sum())
    assert int(fx[0]) == (hi * 2**32 + lo) % P


def test_montgomery_words(gl, oracle, cuda):
    """The reference stores x*2^64 mod p; transforms commute with that map."""
    n = 4096
    x = rand_field(n, seed=99)
    mont = np.array([oracle.lib().glo_to_mont(int(v)) for v in x], dtype=np.uint64)
    d = to_dev(cuda, mont)
    gl.ntt(d)
    back = np.array([oracle.lib().glo_from_mont(int(v)) for v in from_dev(d)], dtype=np.uint64)
    assert np.array_equal(back, oracle.ntt(x))


def test_edge_values(gl, oracle, cuda):
    n = 4096
    for fill in (0, 1, P - 1):
        x = np.full(n, fill, dtype=np.uint64)
        d = to_dev(cuda, x)
        gl.ntt(d)
        assert np.array_equal(from_dev(d), oracle.ntt(x))
    x = np.zeros(n, dtype=np.uint64)
    x[1] = 1  # impulse -> powers of omega
    d = to_dev(cuda, x)
    gl.ntt(d)
    assert np.array_equal(from_dev(d), oracle.ntt(x))


@pytest.mark.parametrize("n", [4096, 1 << 16, 1 << 24, 257 * 16, 1 << 25, 3 * 5 * 17])
def test_words_above_p_are_their_residue(gl, oracle, cuda, n):
    """The header accepts words >= p and treats them as their residue mod p."""
    x = gl.fill_uniform(n, seed=n)
    small = np.random.default_rng(n).integers(0, 2**32 - 1, size=(n + 1) // 2, dtype=np.uint64)
    x[::2] = small
    xn = x.copy()
    xn[::2] += np.uint64(P)
    d = to_dev(cuda, xn)
    gl.ntt(d)
    assert np.array_equal(from_dev(d), oracle.ntt(x))
    d = to_dev(cuda, xn)
    gl.intt(d)
    assert np.array_equal(from_dev(d), oracle.intt(x))


def test_unsupported_size_raises(gl, cuda):
    d = cuda.zeros(7, dtype=cuda.int64, device="cuda")
    with pytest.raises(ValueError, match="is not a supported NTT size"):
        gl.ntt(d)
    # Lengths 0 and 1 of intt are no-ops (ntt/src/ntt/mod.rs:105-107).
    gl.intt(cuda.zeros(1, dtype=cuda.int64, device="cuda"))


@pytest.mark.parametrize("n", [1 << 25, 2 * 16711680])
def test_three_pass_sizes_match_oracle(gl, oracle, cuda, n):
    """Beyond 4096^2 the schedule has three passes (COL, COL, ROW)."""
    x = gl.fill_uniform(n, seed=0x3A55, offset=n)
    d = to_dev(cuda, x)
    gl.ntt(d)
    assert np.array_equal(from_dev(d), oracle.ntt(x))
    gl.intt(d)
    assert np.array_equal(from_dev(d), x)
