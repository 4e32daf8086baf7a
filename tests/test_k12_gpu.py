"""GPU parity of the K12 hashing (single-block KangarooTwelve, Merkle layers
and trees, proof-of-work hashes and nonce search) against the oracle and the
reference's known answers."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
KATS = json.load(open(os.path.join(HERE, "golden", "k12_kats.json")))


def rand_bytes(n, seed):
    return np.random.default_rng(seed).integers(0, 256, size=n, dtype=np.uint8).tobytes()


def dev(cuda, b):
    return cuda.tensor(np.frombuffer(b, dtype=np.uint8).copy(), device="cuda")


def host(t):
    return t.cpu().numpy().tobytes()


@pytest.mark.parametrize("case", KATS["k12"]["cases"], ids=lambda c: c["name"])
def test_known_answers(gl, case):
    from goldilocks_gb300 import k12
    assert k12.k12(bytes(case["input"]), case["out_len"]).hex() == case["hash"]


@pytest.mark.parametrize("out_len", [32, 8, 168])
def test_every_message_length(gl, oracle, cuda, out_len):
    from goldilocks_gb300 import k12
    for n in range(0, 167):
        count = 37
        msgs = rand_bytes(n * count, seed=n)
        got = host(k12.k12(dev(cuda, msgs), out_len, msg_len=n, count=count)) if n else \
            k12.k12(b"", out_len, msg_len=0, count=count)
        want = b"".join(oracle.k12(msgs[i * n:(i + 1) * n], out_len) for i in range(count))
        assert got == want, n


@pytest.mark.parametrize("length", [0, 1, 31, 159, 160, 161, 320, 1600, 12345, (1 << 20) + 7])
def test_process_layer(gl, oracle, cuda, length):
    from goldilocks_gb300 import k12
    data = rand_bytes(length, seed=length)
    want = oracle.k12_process_layer(data)
    assert k12.process_layer(data) == want                      # host memory
    if length:
        assert host(k12.process_layer(dev(cuda, data))) == want  # device memory
        # An input that starts off the 16-byte boundary takes the byte path.
        buf = dev(cuda, b"\x00" + data)
        assert host(k12.process_layer(buf[1:])) == want


def test_reference_tree(gl, oracle, cuda):
    """The input of the reference's tree test (mod.rs:71-83)."""
    from goldilocks_gb300 import k12
    values = bytes(i % 0xFA for i in range(1 << 20))
    want = oracle.merkle_tree(values)
    assert k12.merkle_tree(values) == want
    assert [host(x) for x in k12.merkle_tree(dev(cuda, values))] == want
    assert k12.merkle_tree(values[:32]) == [] and k12.merkle_tree(values[:33]) == want[:0] + \
        [oracle.k12(values[:33])]


def test_large_tree_layer_by_layer(gl, oracle, cuda):
    """1 GiB of field elements: sampled blocks of the large layers against the
    oracle, the small layers in full, each from the GPU's previous layer."""
    from goldilocks_gb300 import k12
    n = 1 << 30
    values = cuda.empty(n, dtype=cuda.uint8, device="cuda")
    values.view(cuda.int64).copy_(cuda.tensor(gl.fill_uniform(n // 8, seed=0x7EE).view(np.int64)))
    layers = k12.merkle_tree(values)
    assert len(layers[-1]) == 32
    prev = values
    rng = np.random.default_rng(1)
    for layer in layers:
        nblk = len(layer) // 32
        if nblk <= 4096:
            assert host(layer) == oracle.k12_process_layer(host(prev)), len(layer)
        else:
            for b in list(rng.integers(0, nblk, size=200)) + [0, nblk - 1]:
                b = int(b)
                lo, hi = b * 160, min(b * 160 + 160, prev.numel())
                assert host(layer[b * 32:(b + 1) * 32]) == oracle.k12(host(prev[lo:hi])), (len(layer), b)
        prev = layer


def test_pow_known_answers(gl):
    from goldilocks_gb300.k12 import Pow
    for c in KATS["pow_hash"]["cases"]:
        p = Pow(bytes([c["challenge_byte"]] * 32), 0)
        assert int(p.hashes(c["nonce"], 1)[0]) == c["hash"]
    for c in KATS["pow_verify"]["cases"]:
        assert Pow(bytes([c["challenge_byte"]] * 32), c["threshold"]).verify(c["nonce"]) == c["ok"]
    for c in KATS["pow_solve"]["cases"]:
        assert Pow(bytes([c["challenge_byte"]] * 32), c["threshold"]).solve() == c["nonce"], c["name"]


def test_pow_hashes_and_solve_against_oracle(gl, oracle):
    from goldilocks_gb300.k12 import Pow
    ch = rand_bytes(32, seed=9)
    p = Pow(ch, Pow.threshold_from_bits(12.0))
    start = (1 << 40) + 12345
    got = p.hashes(start, 5000)
    assert [int(v) for v in got[:300]] == [oracle.pow_hash(ch, start + i) for i in range(300)]
    first = next(i for i, v in enumerate(got) if int(v) >= p.threshold)
    assert p.solve(start=start) == start + first
    assert p.solve(start=start, max_count=first) is None     # bounded range without a hit
    assert oracle.pow_solve(ch, p.threshold, start, 20000) == start + first
