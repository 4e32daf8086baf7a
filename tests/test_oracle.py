"""CPU: pin the oracle against the reference's golden artefacts.

* the 860 codelet constants of ntt/src/ntt/small.rs (recomputed by the
  restated generator oracle/codegen_ref.py),
* the known-answer values of the reference's unit tests,
* O(n^2) DFT vectors computed in Python integers,
* the oracle's fast path against its naive DFT on every divisor <= 4096 and on
  the reference's own test sizes, and round trips.
"""
import json
import os
import sys

import numpy as np
import pytest

from conftest import P, ROOT, rand_field

GOLD = os.path.join(ROOT, "tests", "golden")


def load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def test_codelet_constants_match_reference():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import codegen_ref
    gold = load("codelet_constants.json")["constants"]
    assert sorted(int(k) for k in gold) == codegen_ref.CODELET_SIZES
    total = 0
    for size in codegen_ref.CODELET_SIZES:
        assert codegen_ref.constants(size) == gold[str(size)], size
        total += len(gold[str(size)])
    assert total == 860


def test_reference_kats(oracle):
    k = load("reference_kats.json")
    lib = oracle.lib()
    divs = oracle.divisors()
    assert len(divs) == k["divisor_count"]["value"] == 1056
    assert divs[0] == 1 and divs[-1] == P - 1
    for n, want in k["next"]["cases"]:
        assert lib.glo_next(n) == want
    for a, n, want in k["shift"]["cases"]:
        assert lib.glo_shift(a, n) == want
    assert k["generator"]["value"] == 2717
    w5, w4 = lib.glo_root(5), lib.glo_root(4)
    assert lib.glo_pow(w5, 5) == 1
    assert lib.glo_pow(w4, 4) == 1 and lib.glo_pow(w4, 2) == P - 1
    c = k["circular_convolution"]
    a = np.array(c["a"], dtype=np.uint64)
    bh = oracle.ntt(np.array(c["b"], dtype=np.uint64))
    lib.glo_convolve(a.ctypes.data, bh.ctypes.data, 3)
    assert a.tolist() == c["c"]
    # The same KAT on Field (Montgomery) words, as the reference's test runs it.
    am = oracle.to_mont(c["a"])
    bm = oracle.ntt(oracle.to_mont(c["b"]))
    assert oracle.from_mont(oracle.convolve(am, bm, montgomery=True)).tolist() == c["c"]


def test_split_all_divisors(oracle):
    lib = oracle.lib()
    for n in oracle.divisors():
        a = lib.glo_split(n)
        assert a * (n // a) == n and a <= n // a


def test_field_ops_against_integers(oracle):
    lib = oracle.lib()
    rng = np.random.default_rng(0)
    vals = [0, 1, 2, P - 1, P - 2, 2**32 - 1, 2**32, 2**63, P - 2**32] + \
        [int(v) * 2 % P for v in rng.integers(0, 2**63, 300)]
    for a in vals:
        assert lib.glo_inv(a) == (pow(a, P - 2, P) if a else 0)
        assert lib.glo_from_mont(lib.glo_to_mont(a)) == a
        for b in vals[:40]:
            assert lib.glo_mul(a, b) == a * b % P
            assert lib.glo_add(a, b) == (a + b) % P
            assert lib.glo_sub(a, b) == (a - b) % P
        for s in (0, 1, 31, 32, 33, 48, 63, 64, 65, 95, 96, 97, 150, 191, 192, 1000):
            assert lib.glo_shift(a, s) == a * pow(2, s, P) % P
        for i in range(0, 384, 37):
            assert lib.glo_root_384(a, i) == a * pow(lib.glo_root(384), i, P) % P


def test_dft_vectors(oracle):
    for v in load("dft_vectors.json")["vectors"]:
        x = np.array(v["input"], dtype=np.uint64)
        assert oracle.ntt(x).tolist() == v["ntt"], v["n"]
        assert oracle.naive_ntt(x).tolist() == v["ntt"], v["n"]


def test_fast_path_against_naive_all_small_divisors(oracle):
    for n in oracle.divisors():
        if n > 4096:
            break
        x = rand_field(n, seed=n)
        assert np.array_equal(oracle.ntt(x), oracle.naive_ntt(x)), n
        assert np.array_equal(oracle.intt(oracle.ntt(x)), x), n
        assert np.array_equal(oracle.intt(x), oracle.naive_intt(x)), n


def test_reference_plan_trees(oracle):
    assert oracle.strategy_describe(1 << 24) == \
        "CT(4096,4096)[CT(64,64)[small(64),small(64)],CT(64,64)[small(64),small(64)]]"
    assert oracle.strategy_describe(16711680).startswith("CT(4080,4096)[CT(60,68)")
    assert oracle.strategy_describe(257 * 4) == "GT(4,257)[small(4),Rader(257)[CT(16,16)[small(16),small(16)]]]"


@pytest.mark.parametrize("n", [257, 65537 * 2, 3 * 257 * 16])
def test_runtime_rader_sizes(oracle, n):
    x = rand_field(n, seed=n)
    y = oracle.ntt(x)
    assert np.array_equal(oracle.intt(y), x)
    if n <= 4096:
        assert np.array_equal(y, oracle.naive_ntt(x))
    else:  # spot-check outputs with direct sums
        w = oracle.lib().glo_root(n)
        xs = [int(v) for v in x[::-1]]
        for k in (1, n // 3, n - 1):
            wk, acc = pow(w, k, P), 0
            for v in xs:
                acc = (acc * wk + v) % P
            assert int(y[k]) == acc


def test_reverse_inverse_identity(oracle):
    """naive.rs:240-253: reverse [1..], forward, scale = inverse."""
    n = 15
    x = rand_field(n, seed=15)
    r = x.copy()
    r[1:] = r[1:][::-1]
    f = oracle.ntt(r)
    inv_n = pow(n, P - 2, P)
    f = np.array([int(v) * inv_n % P for v in f], dtype=np.uint64)
    assert np.array_equal(f, oracle.intt(x))


def test_coset_lde_composition(oracle):
    """The LDE of a polynomial's evaluations equals direct evaluation on the coset."""
    n, cols, blowup, shift = 16, 3, 4, 7
    x = rand_field(n * cols, seed=3)
    out = oracle.coset_lde(x, n, cols, blowup, shift).reshape(n * blowup, cols)
    for c in range(cols):
        coeffs = oracle.intt(x.reshape(n, cols)[:, c].copy())
        w = oracle.lib().glo_root(n * blowup)
        for k in range(0, n * blowup, 7):
            pt = shift * pow(w, k, P) % P
            val = 0
            for a in coeffs[::-1]:
                val = (val * pt + int(a)) % P
            assert int(out[k, c]) == val
