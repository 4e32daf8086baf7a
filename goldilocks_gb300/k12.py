"""K12 Merkle layers and proof of work on the GPU: the `goldilocks-pcs`
crate's hashing (pcs/src/k12/mod.rs, pcs/src/k12/generic.rs, pcs/src/pow.rs).

Data may be host bytes (bytes / numpy uint8) -- copied to the GPU and back --
or a CUDA tensor, which stays on the device (results are CUDA uint8 tensors).
"""
import ctypes

import numpy as np

from . import _lib as L
from .ntt import GoldilocksError, _check

BLOCK_SIZE = 160  # pcs/src/k12/mod.rs:28
HASH_SIZE = 32    # pcs/src/k12/mod.rs:29


def next_layer_size(size):
    """pcs/src/k12/mod.rs:33-35."""
    return L.load().gl_k12_next_layer_size(size)


def _bytes_arg(data):
    """(pointer, length, mem, stream, keepalive, torch or None)."""
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    if torch is not None and isinstance(data, torch.Tensor):
        if not data.is_cuda or not data.is_contiguous():
            raise ValueError("tensors must be contiguous CUDA tensors")
        stream = torch.cuda.current_stream(data.device).cuda_stream
        return data.data_ptr(), data.numel() * data.element_size(), L.GL_MEM_DEVICE, stream, data, torch
    arr = np.frombuffer(bytes(data), dtype=np.uint8) if not isinstance(data, np.ndarray) else \
        np.ascontiguousarray(data).view(np.uint8).reshape(-1)
    arr = np.ascontiguousarray(arr)
    return (arr.ctypes.data if arr.size else None), arr.size, L.GL_MEM_HOST, None, arr, None


def _out(torch, nbytes, like):
    if torch is None:
        return np.zeros(nbytes, dtype=np.uint8)
    return torch.empty(nbytes, dtype=torch.uint8, device=like.device)


def _ptr(buf):
    if isinstance(buf, np.ndarray):
        return buf.ctypes.data if buf.size else None
    return buf.data_ptr()


def process_layer(data):
    """pcs/src/k12/generic.rs:86-95: each 160-byte block to a 32-byte hash."""
    ptr, n, mem, stream, keep, torch = _bytes_arg(data)
    out = _out(torch, next_layer_size(n), keep)
    _check(L.load().gl_k12_process_layer(ptr, n, _ptr(out), mem, stream), "k12 process_layer")
    return out.tobytes() if torch is None else out


def k12(messages, out_len=32, msg_len=None, count=None):
    """k12::<out_len> (generic.rs:62-84).  `messages`: one message, or
    `msg_len`-byte messages back to back (`count` of them when msg_len is 0);
    returns the hashes back to back."""
    ptr, n, mem, stream, keep, torch = _bytes_arg(messages)
    if msg_len is None:
        msg_len, count = n, 1
    elif msg_len:
        if n % msg_len:
            raise ValueError("message bytes are not a multiple of msg_len")
        count = n // msg_len
    elif count is None:
        raise ValueError("count is required for empty messages")
    out = _out(torch, count * out_len, keep)
    _check(L.load().gl_k12_hash_many(ptr, msg_len, count, _ptr(out), out_len, mem, stream), "k12")
    return out.tobytes() if torch is None else out


def merkle_tree(values):
    """pcs/src/k12/mod.rs:41-60: the list of layers (first layer first, the
    32-byte root last); empty when values fit in one hash."""
    ptr, n, mem, stream, keep, torch = _bytes_arg(values)
    total = L.load().gl_merkle_tree_bytes(n)
    if total == 0:
        return []
    out = _out(torch, total, keep)
    _check(L.load().gl_merkle_tree(ptr, n, _ptr(out), total, mem, stream), "merkle_tree")
    layers, off, size = [], 0, n
    while size > HASH_SIZE:
        size = next_layer_size(size)
        seg = out[off:off + size]
        layers.append(seg.tobytes() if torch is None else seg)
        off += size
    return layers


class Pow:
    """pcs/src/pow.rs:9-60: proof of work by partial inversion of K12."""

    def __init__(self, challenge, threshold):
        challenge = bytes(challenge)
        if len(challenge) != 32:
            raise ValueError("challenge must be 32 bytes")
        self.challenge = challenge
        self.threshold = int(threshold)
        self._c = (ctypes.c_uint8 * 32).from_buffer_copy(challenge)

    @staticmethod
    def threshold_from_bits(bits):
        """pow.rs:15-17: u64::MAX - 2^(64 - bits) (the f64 power, truncated)."""
        return (2**64 - 1) - min(int(2.0 ** (64.0 - bits)), 2**64 - 1)

    @staticmethod
    def threshold_from_probability(probability):
        """pow.rs:19-23."""
        if not 0.0 < probability <= 1.0:
            raise ValueError("probability must be in (0, 1]")
        return (2**64 - 1) - min(int(float(2**64 - 1) * probability), 2**64 - 1)

    def hashes(self, start, count):
        out = np.zeros(count, dtype=np.uint64)
        _check(L.load().gl_pow_hashes(self._c, start, count, out.ctypes.data, L.GL_MEM_HOST, None),
               "pow hashes")
        return out

    def verify(self, nonce):
        ok = ctypes.c_int()
        _check(L.load().gl_pow_verify(self._c, self.threshold, nonce, ctypes.byref(ok), None), "pow verify")
        return bool(ok.value)

    def solve(self, start=0, max_count=2**64 - 1):
        """The smallest satisfying nonce >= start (None if there is none in
        [start, start + max_count))."""
        n = ctypes.c_uint64()
        st = L.load().gl_pow_solve(self._c, self.threshold, start, max_count, ctypes.byref(n), None)
        if st == L.GL_ERR_NOT_FOUND:
            return None
        _check(st, "pow solve")
        return n.value
