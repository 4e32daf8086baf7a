"""CPU: the K12 / proof-of-work oracle against the known answers of the
reference's own tests (tests/golden/k12_kats.json: pcs/src/k12/generic.rs,
pcs/src/k12/aarch64.rs, pcs/src/pow.rs), and the host-side helpers."""
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
KATS = json.load(open(os.path.join(HERE, "golden", "k12_kats.json")))


@pytest.mark.parametrize("case", KATS["k12"]["cases"], ids=lambda c: c["name"])
def test_k12_known_answers(oracle, case):
    assert oracle.k12(bytes(case["input"]), case["out_len"]).hex() == case["hash"]


def test_pow_known_answers(oracle):
    for c in KATS["pow_hash"]["cases"]:
        assert oracle.pow_hash(bytes([c["challenge_byte"]] * 32), c["nonce"]) == c["hash"]
    for c in KATS["pow_verify"]["cases"]:
        ok = oracle.pow_hash(bytes([c["challenge_byte"]] * 32), c["nonce"]) >= c["threshold"]
        assert ok == c["ok"], c
    for c in KATS["pow_solve"]["cases"]:
        ch = bytes([c["challenge_byte"]] * 32)
        if c["nonce"] < 100000:  # the 32-bit case (4.4e8 hashes) runs on the GPU only
            assert oracle.pow_solve(ch, c["threshold"]) == c["nonce"], c["name"]
        else:
            assert oracle.pow_hash(ch, c["nonce"]) >= c["threshold"]


def test_layer_shapes_and_blocks(oracle):
    """mod.rs:71-83: every layer of the tree of (0..0xfa).cycle().take(2^20)
    is a multiple of 32 bytes, ending in one 32-byte root; each layer is the
    per-block hash of the previous one (generic.rs:86-95)."""
    values = bytes(i % 0xFA for i in range(1 << 20))
    layers = oracle.merkle_tree(values)
    sizes = [len(x) for x in layers]
    assert all(s % 32 == 0 for s in sizes) and sizes[-1] == 32
    assert sizes[0] == (len(values) + 159) // 160 * 32
    prev = values
    for layer in layers:
        assert layer[:32] == oracle.k12(prev[:160])
        last = (len(prev) - 1) // 160 * 160
        assert layer[-32:] == oracle.k12(prev[last:])
        prev = layer
    assert oracle.merkle_tree(bytes(32)) == [] and len(oracle.merkle_tree(bytes(33))) == 1


def test_thresholds_host_side(gl):
    from goldilocks_gb300.k12 import Pow
    for c in KATS["pow_solve"]["cases"]:
        if c["bits"] is not None:
            assert Pow.threshold_from_bits(c["bits"]) == c["threshold"]
    assert Pow.threshold_from_probability(1.0) == 0
