"""GPU: the device field primitives (gl_field.cuh, inline PTX) on adversarial
inputs -- words at and above p, all-ones words, words with one half zero --
against exact integer arithmetic; every result must be the canonical value
(gl_sub of a first operand at or above p excepted: it is only congruent).
Random transform inputs almost never reach these words, so the transform
parity tests alone would not catch a wrong carry here."""
import numpy as np
import pytest

from conftest import P, from_dev, to_dev

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1
R_INV = pow(2**64, P - 2, P)  # 2^-64 mod p


def words(n, seed):
    """n words of which most are adversarial: near 2^64, at and just above p,
    near 2^32 multiples, plus uniform ones."""
    rng = np.random.default_rng(seed)
    edge = np.array([0, 1, 2, P - 1, P - 2, P, P + 1, M64, M64 - 1, 2**32 - 1, 2**32, 2**32 + 1, 2**63,
                     0xFFFFFFFF00000000, 0xFFFFFFFEFFFFFFFF, 0x00000000FFFF0000 << 16], dtype=np.uint64)
    x = rng.integers(0, 2**64, size=n, dtype=np.uint64)
    k = np.arange(n) % 8
    x[k == 1] = np.uint64(P) + rng.integers(0, 2**32 - 1, size=int((k == 1).sum()), dtype=np.uint64)
    x[k == 2] = np.uint64(M64) - rng.integers(0, 2**16, size=int((k == 2).sum()), dtype=np.uint64)
    x[k == 3] = rng.integers(0, 2**32, size=int((k == 3).sum()), dtype=np.uint64)
    x[k == 4] = rng.integers(0, 2**32, size=int((k == 4).sum()), dtype=np.uint64) << np.uint64(32)
    x[:edge.size] = edge
    return x


def canonical(n, seed):
    rng = np.random.default_rng(seed)
    b = rng.integers(0, P, size=n, dtype=np.uint64)
    b[::5] = np.uint64(P - 1) - rng.integers(0, 2**16, size=b[::5].size, dtype=np.uint64)
    b[1::7] = 0
    return b


def run(gl, cuda, op, a, b):
    lib = gl._lib.load()
    da, db = to_dev(cuda, a), None if b is None else to_dev(cuda, b)
    out = cuda.empty(a.size, dtype=cuda.int64, device="cuda")
    st = lib.gl_debug_field_op(op, da.data_ptr(), None if db is None else db.data_ptr(), out.data_ptr(), a.size,
                               cuda.cuda.current_stream().cuda_stream)
    assert st == gl._lib.GL_OK
    return from_dev(out)


N = 1 << 14


@pytest.mark.parametrize("name", ["add", "sub", "canon", "mont_mul", "mul"])
def test_binary_primitives(gl, cuda, name):
    L = gl._lib
    op = {"add": L.GL_FOP_ADD, "sub": L.GL_FOP_SUB, "canon": L.GL_FOP_CANON,
          "mont_mul": L.GL_FOP_MONT_MUL, "mul": L.GL_FOP_MUL}[name]
    # gl_add needs both operands canonical; the others accept any first operand.
    a = canonical(N, 1) if name == "add" else words(N, 1)
    b = canonical(N, 2)
    got = run(gl, cuda, op, a, b)
    for x, y, g in zip(a.tolist(), b.tolist(), got.tolist()):
        want = {"add": x + y, "sub": x - y, "canon": x, "mont_mul": x * y * R_INV, "mul": x * y}[name] % P
        assert g % P == want, (name, hex(x), hex(y), hex(g))
        assert g < P or (name == "sub" and x >= P), (name, hex(x), hex(y), hex(g))


@pytest.mark.parametrize("k", [12, 24, 32, 36, 48, 64, 72, 84, 96, 108, 144])
def test_shifts(gl, cuda, k):
    L = gl._lib
    a = canonical(N, k) if k == 96 else words(N, k)  # 2^96 = -1: a negation, canonical operand
    got = run(gl, cuda, L.GL_FOP_SHL + k, a, None)
    for x, g in zip(a.tolist(), got.tolist()):
        assert g % P == x * 2**k % P and g < P, (k, hex(x), hex(g))
