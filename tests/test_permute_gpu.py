"""GPU: the standalone permutations of the reference's permute module
(ntt/src/permute/mod.rs:46-74) -- the in-place transpose and bit reversal --
against the reference's own known answers (mod.rs tests test_copy_2_3,
test_copy_3_3, test_copy_2_4) and a numpy restatement, in host and device
memory."""
import numpy as np
import pytest

from conftest import from_dev, rand_field, to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rows,cols,want", [
    (2, 3, [0, 3, 1, 4, 2, 5]),            # permute/mod.rs test_copy_2_3
    (3, 3, [0, 3, 6, 1, 4, 7, 2, 5, 8]),   # test_copy_3_3
    (2, 4, [0, 4, 1, 5, 2, 6, 3, 7]),      # test_copy_2_4
])
def test_transpose_reference_cases(gl, cuda, rows, cols, want):
    x = np.arange(rows * cols, dtype=np.uint64)
    gl.transpose(x, (rows, cols))                          # host memory
    assert x.tolist() == want
    d = to_dev(cuda, np.arange(rows * cols, dtype=np.uint64))
    gl.transpose(d, (rows, cols))                          # device memory
    assert from_dev(d).tolist() == want


@pytest.mark.parametrize("rows,cols", [(1, 7), (7, 1), (31, 33), (64, 64), (4096, 4096), (4080, 4096),
                                       (100, 3000), (17, 1 << 16), (1 << 16, 17)])
def test_transpose_matches_numpy(gl, cuda, rows, cols):
    x = rand_field(rows * cols, seed=rows * 7 + cols)
    want = x.reshape(rows, cols).T.copy().ravel()
    d = to_dev(cuda, x)
    gl.transpose(d, (rows, cols))
    assert np.array_equal(from_dev(d), want)


@pytest.mark.parametrize("logn", [0, 1, 2, 3, 10, 17, 24])
def test_bit_reverse(gl, cuda, logn):
    n = 1 << logn
    x = rand_field(n, seed=logn)
    idx = np.arange(n, dtype=np.uint64)
    rev = np.zeros(n, dtype=np.uint64)
    for b in range(logn):
        rev |= ((idx >> np.uint64(b)) & np.uint64(1)) << np.uint64(logn - 1 - b)
    d = to_dev(cuda, x)
    gl.bit_reverse(d)
    assert np.array_equal(from_dev(d), x[rev])
    h = x.copy()
    gl.bit_reverse(h)
    assert np.array_equal(h, x[rev])


def test_bit_reverse_rejects_other_lengths(gl, cuda):
    with pytest.raises(ValueError):
        gl.bit_reverse(to_dev(cuda, rand_field(12, seed=1)))
