"""CPU oracle for the Goldilocks NTT path -- TEST INFRASTRUCTURE ONLY.

A C restatement of recmo/goldilocks' `goldilocks-ntt` transform path
(gl_oracle.c, codelets_gen.c from codegen_ref.py) and of the `goldilocks-pcs`
K12 Merkle layers and proof of work (k12_oracle.c), loaded through ctypes.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
as the checker; the product (goldilocks_gb300/) never does.

Parity is pinned by the reference's own artefacts (tests/golden/): the 860
codelet constants of ntt/src/ntt/small.rs, the known-answer tests of the
reference's unit tests, and O(n^2) DFT vectors.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgl_oracle.so")
SOURCES = [os.path.join(HERE, "gl_oracle.c"), os.path.join(HERE, "codelets_gen.c"),
           os.path.join(HERE, "k12_oracle.c")]
P = 0xFFFF_FFFF_0000_0001


def build():
    """Compile the oracle with gcc (incremental)."""
    os.makedirs(BUILD, exist_ok=True)
    deps = SOURCES + [os.path.join(HERE, "gl_oracle.h"), os.path.join(HERE, "gl_oracle_internal.h")]
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    objs = []
    procs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        # -O3 without -march=native: the same build recipe runs on the x86
        # container and on the Arm host of the GPU, and must give the same code
        # paths on both (the arithmetic is integer-only, so results agree).
        procs.append(subprocess.Popen(["gcc", "-O3", "-fPIC", "-std=c11", "-c", src, "-o", obj],
                                      stderr=subprocess.PIPE, text=True))
    for p in procs:
        _, err = p.communicate()
        if p.returncode:
            raise RuntimeError("oracle build failed:\n" + err)
    tmp = LIB + ".tmp"
    subprocess.run(["gcc", "-shared", "-o", tmp] + objs + ["-lm", "-lpthread"], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None
_u64 = ctypes.c_uint64
_vp = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        l = ctypes.CDLL(LIB)
        for f in ("glo_add", "glo_sub", "glo_mul", "glo_shift", "glo_root_384", "glo_pow"):
            getattr(l, f).restype = _u64
            getattr(l, f).argtypes = [_u64, _u64]
        for f in ("glo_inv", "glo_root", "glo_split", "glo_next", "glo_to_mont", "glo_from_mont"):
            getattr(l, f).restype = _u64
            getattr(l, f).argtypes = [_u64]
        l.glo_is_divisor.argtypes = [_u64]
        l.glo_divisors.restype = ctypes.c_size_t
        l.glo_divisors.argtypes = [_vp, ctypes.c_size_t]
        for f in ("glo_naive_ntt", "glo_naive_intt"):
            getattr(l, f).argtypes = [_vp, ctypes.c_size_t]
        l.glo_ntt_batch.argtypes = [_vp, ctypes.c_size_t, ctypes.c_size_t]
        l.glo_ntt.argtypes = [_vp, ctypes.c_size_t]
        l.glo_intt.argtypes = [_vp, ctypes.c_size_t]
        l.glo_strategy_describe.argtypes = [_u64, ctypes.c_char_p, ctypes.c_size_t]
        l.glo_coset_lde.argtypes = [_vp, _vp, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_uint32, _u64]
        l.glo_convolve.argtypes = [_vp, _vp, ctypes.c_size_t]
        l.glo_convolve_mont.argtypes = [_vp, _vp, ctypes.c_size_t]
        l.glo_k12.argtypes = [_vp, ctypes.c_size_t, _vp, ctypes.c_size_t]
        l.glo_k12_next_layer_size.restype = ctypes.c_size_t
        l.glo_k12_next_layer_size.argtypes = [ctypes.c_size_t]
        l.glo_k12_process_layer.argtypes = [_vp, ctypes.c_size_t, _vp]
        l.glo_merkle_tree.restype = ctypes.c_size_t
        l.glo_merkle_tree.argtypes = [_vp, ctypes.c_size_t, _vp, ctypes.c_size_t]
        l.glo_pow_hash.restype = _u64
        l.glo_pow_hash.argtypes = [_vp, _u64]
        l.glo_pow_solve.argtypes = [_vp, _u64, _u64, _u64, ctypes.POINTER(_u64)]
        _lib = l
    return _lib


def _arr(x):
    x = np.ascontiguousarray(x, dtype=np.uint64)
    return x


def ntt(x, size=None):
    """Forward transform(s); `size` splits x into len(x)/size contiguous transforms."""
    y = _arr(x).copy()
    n = y.size
    rc = lib().glo_ntt_batch(y.ctypes.data, n, size if size is not None else n) if n else 0
    if rc:
        raise ValueError("oracle: unsupported size")
    return y


def intt(x, size=None):
    y = _arr(x).copy()
    size = size if size is not None else y.size
    for off in range(0, y.size, max(size, 1)):
        seg = y[off:off + size]
        if lib().glo_intt(seg.ctypes.data, size):
            raise ValueError("oracle: unsupported size")
    return y


def naive_ntt(x):
    y = _arr(x).copy()
    lib().glo_naive_ntt(y.ctypes.data, y.size)
    return y


def naive_intt(x):
    y = _arr(x).copy()
    lib().glo_naive_intt(y.ctypes.data, y.size)
    return y


def coset_lde(x, n, cols, blowup, shift):
    x = _arr(x)
    out = np.empty(n * blowup * cols, dtype=np.uint64)
    if lib().glo_coset_lde(x.ctypes.data, out.ctypes.data, n, cols, blowup, shift):
        raise ValueError("oracle: unsupported LDE shape")
    return out


def convolve(a, b_hat, size=None, montgomery=True):
    """Per length-`size` sequence of a: intt(ntt(a) * b_hat); b_hat holds one
    sequence for all or one per sequence; Montgomery or canonical product."""
    y = _arr(a).copy()
    b = _arr(b_hat)
    size = y.size if size is None else size
    f = lib().glo_convolve_mont if montgomery else lib().glo_convolve
    for i in range(y.size // size):
        seg = y[i * size:(i + 1) * size]
        bs = b if b.size == size else b[i * size:(i + 1) * size]
        bs = np.ascontiguousarray(bs)
        if size == 1:  # ntt and intt of one element are the identity
            seg[0] = lib().glo_from_mont(int(seg[0]) * int(bs[0]) % P) if montgomery else \
                int(seg[0]) * int(bs[0]) % P
        elif f(seg.ctypes.data, bs.ctypes.data, size):
            raise ValueError("oracle: unsupported size")
    return y


def to_mont(x):
    """Field::new of each value: x*2^64 mod p."""
    return np.array([lib().glo_to_mont(int(v)) for v in _arr(x)], dtype=np.uint64)


def from_mont(x):
    """u64::from(Field) of each word: x*2^-64 mod p."""
    return np.array([lib().glo_from_mont(int(v)) for v in _arr(x)], dtype=np.uint64)


def k12(msg, out_len=32):
    """k12::<out_len>(msg) for len(msg) <= 166 (pcs/src/k12/generic.rs:62-84)."""
    m = np.frombuffer(bytes(msg), dtype=np.uint8).copy()
    out = np.zeros(out_len, dtype=np.uint8)
    if lib().glo_k12(m.ctypes.data if m.size else None, m.size, out.ctypes.data, out_len):
        raise ValueError("oracle: k12 input longer than 166 bytes or output longer than 168")
    return out.tobytes()


def k12_process_layer(data):
    d = np.frombuffer(bytes(data), dtype=np.uint8).copy()
    out = np.zeros(lib().glo_k12_next_layer_size(d.size), dtype=np.uint8)
    lib().glo_k12_process_layer(d.ctypes.data, d.size, out.ctypes.data)
    return out.tobytes()


def merkle_tree(values):
    """The layers of merkle_tree (pcs/src/k12/mod.rs:41-60) as a list of bytes."""
    v = np.frombuffer(bytes(values), dtype=np.uint8).copy()
    total = lib().glo_merkle_tree(v.ctypes.data, v.size, None, 0)
    out = np.zeros(max(total, 1), dtype=np.uint8)
    lib().glo_merkle_tree(v.ctypes.data, v.size, out.ctypes.data, total)
    layers, off, n = [], 0, v.size
    while n > 32:
        n = lib().glo_k12_next_layer_size(n)
        layers.append(out[off:off + n].tobytes())
        off += n
    return layers


def pow_hash(challenge, nonce):
    c = np.frombuffer(bytes(challenge), dtype=np.uint8).copy()
    return lib().glo_pow_hash(c.ctypes.data, nonce)


def pow_solve(challenge, threshold, start=0, count=1 << 40):
    c = np.frombuffer(bytes(challenge), dtype=np.uint8).copy()
    n = _u64()
    if lib().glo_pow_solve(c.ctypes.data, threshold, start, count, ctypes.byref(n)):
        return None
    return n.value


def strategy_describe(size):
    buf = ctypes.create_string_buffer(1 << 16)
    if lib().glo_strategy_describe(size, buf, len(buf)):
        raise ValueError("oracle: unsupported size")
    return buf.value.decode()


_M64 = (1 << 64) - 1


def _splitmix64(x):
    """splitmix64 finaliser on a numpy uint64 array (wrapping arithmetic)."""
    z = x + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def fill_uniform(n, seed, offset=0):
    """Seeded field elements uniform in [0, p): element i is the first value
    below p of splitmix64(splitmix64(seed) ^ (offset + i + (k << 48))),
    k = 0, 1, ...  The same stream as the GPU library's gl_fill_uniform,
    restated in numpy so that the CPU baseline makes its inputs without
    loading the product library."""
    with np.errstate(over="ignore"):
        s = _splitmix64(np.array([seed & _M64], dtype=np.uint64))[0]
        idx = np.arange(n, dtype=np.uint64) + np.uint64(offset & _M64)
        out = _splitmix64(s ^ idx)
        k = 0
        bad = np.nonzero(out >= np.uint64(P))[0]
        while bad.size:
            k += 1
            out[bad] = _splitmix64(s ^ (idx[bad] + np.uint64((k << 48) & _M64)))
            bad = bad[out[bad] >= np.uint64(P)]
    return out


def divisors():
    buf = (ctypes.c_uint64 * 1056)()
    lib().glo_divisors(ctypes.addressof(buf), 1056)
    return [int(v) for v in buf]
