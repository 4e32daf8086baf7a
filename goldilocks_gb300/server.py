"""Continuous-batching request server (gl_server_*) and a load generator.

    srv = Server(budget_bytes=64 << 30, slots=4, max_batch=64)
    rid = srv.submit(GL_OP_NTT, n, cols, inp, out)      # device tensors
    srv.wait(rid)                                       # status, or raises

`serve_stream` replays a request list with Poisson arrival times against a
server and reports throughput and p50/p99 latency; `serial_baseline` runs the
same requests one at a time through the plain per-call API on the same GPU.
"""
import ctypes
import time

import numpy as np

from . import _lib as L
from .ntt import GoldilocksError

GL_OP_NTT, GL_OP_INTT, GL_OP_LDE = L.GL_OP_NTT, L.GL_OP_INTT, L.GL_OP_LDE


class Server:
    def __init__(self, budget_bytes=64 << 30, slots=4, max_batch=64):
        self._lib = L.load()
        h = ctypes.c_void_p()
        st = self._lib.gl_server_create(budget_bytes, slots, max_batch, ctypes.byref(h))
        if st != L.GL_OK:
            raise GoldilocksError(st, "server create")
        self._h = h

    @staticmethod
    def request(op, n, cols, inp, out, blowup=4, shift=7):
        r = L.Request()
        r.op, r.n, r.cols = op, n, cols
        r.inp, r.out = inp.data_ptr(), out.data_ptr()
        r.blowup, r.shift = blowup, shift
        return r

    def submit(self, op, n, cols, inp, out, blowup=4, shift=7):
        r = self.request(op, n, cols, inp, out, blowup, shift)
        rid = ctypes.c_uint64()
        st = self._lib.gl_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid))
        if st != L.GL_OK:
            raise GoldilocksError(st, "submit")
        return rid.value

    def poll(self, rid):
        s = ctypes.c_int()
        st = self._lib.gl_server_poll(self._h, rid, ctypes.byref(s))
        if st != L.GL_OK:
            raise GoldilocksError(st, "poll")
        return s.value

    def wait(self, rid, timeout_ms=60000):
        s = ctypes.c_int()
        st = self._lib.gl_server_wait(self._h, rid, timeout_ms, ctypes.byref(s))
        if st != L.GL_OK:
            raise GoldilocksError(st, "wait")
        return s.value

    def cancel(self, rid):
        return self._lib.gl_server_cancel(self._h, rid)

    def stats(self):
        s = L.ServerStats()
        self._lib.gl_server_get_stats(self._h, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in L.ServerStats._fields_}

    def close(self):
        if self._h:
            self._lib.gl_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def request_bytes(op, n, cols, blowup=4):
    r = L.Request()
    r.op, r.n, r.cols, r.blowup = op, n, cols, blowup
    r.inp = r.out = 1  # non-null placeholders: only the shape matters
    b = ctypes.c_uint64()
    st = L.load().gl_server_request_bytes(ctypes.byref(r), ctypes.byref(b))
    if st != L.GL_OK:
        raise GoldilocksError(st, "request bytes")
    return b.value


def make_requests(count, seed, log_min=10, log_max=24, max_cols=64, mix=(0.4, 0.3, 0.3),
                  blowup=4):
    """The serving mix: op NTT/iNTT/LDE with probabilities `mix`, log2 n uniform
    in [log_min, log_max], columns uniform in [1, max_cols]."""
    rng = np.random.default_rng(seed)
    ops = rng.choice([GL_OP_NTT, GL_OP_INTT, GL_OP_LDE], size=count, p=list(mix))
    logs = rng.integers(log_min, log_max + 1, size=count)
    cols = rng.integers(1, max_cols + 1, size=count)
    return [(int(o), 1 << int(k), int(c), blowup) for o, k, c in zip(ops, logs, cols)]


def poisson_arrivals(count, rate_per_s, seed):
    rng = np.random.default_rng(seed + 1)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, size=count))


def _buffers(torch, reqs, pool):
    """Per request: input = a slice of a resident pool, output = its own buffer."""
    outs, ins = [], []
    for op, n, cols, blowup in reqs:
        words = n * cols
        ins.append(pool[:words])
        outs.append(torch.empty(words * (blowup if op == GL_OP_LDE else 1), dtype=torch.int64,
                                device="cuda"))
    return ins, outs


def serve_stream(reqs, arrivals, pool, budget_bytes=64 << 30, slots=4, max_batch=64):
    """Submit each request at its arrival time (seconds from start), wait for
    all; returns (elements/s, stats, wall seconds).  Outputs are returned too."""
    import torch
    ins, outs = _buffers(torch, reqs, pool)
    torch.cuda.synchronize()
    ids = []
    with Server(budget_bytes, slots, max_batch) as srv:
        t0 = time.perf_counter()
        for (op, n, cols, blowup), a, i, o in zip(reqs, arrivals, ins, outs):
            now = time.perf_counter() - t0
            if a > now:
                time.sleep(a - now)
            ids.append(srv.submit(op, n, cols, i, o, blowup))
        for rid in ids:
            st = srv.wait(rid, timeout_ms=600000)
            if st != L.GL_OK:
                raise GoldilocksError(st, "request")
        wall = time.perf_counter() - t0
        stats = srv.stats()
    elements = sum(n * cols for _, n, cols, _ in reqs)
    return elements / wall, stats, wall, outs


def serial_baseline(reqs, pool):
    """The same requests one at a time through the plain API (gl_ntt_columns,
    gl_coset_lde, gl_ntt/gl_intt), each synchronised before the next starts."""
    import torch
    lib = L.load()
    ins, outs = _buffers(torch, reqs, pool)
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    lat = []
    t0 = time.perf_counter()
    for (op, n, cols, blowup), i, o in zip(reqs, ins, outs):
        t = time.perf_counter()
        if op == GL_OP_LDE:
            st = lib.gl_coset_lde(i.data_ptr(), o.data_ptr(), n, cols, blowup, 7, L.GL_MEM_DEVICE, stream)
        else:
            o.copy_(i)
            d = L.GL_INVERSE if op == GL_OP_INTT else L.GL_FORWARD
            st = lib.gl_ntt_columns(o.data_ptr(), n, cols, d, L.GL_MEM_DEVICE, stream)
        if st != L.GL_OK:
            raise GoldilocksError(st, "serial")
        torch.cuda.synchronize()
        lat.append((time.perf_counter() - t) * 1e3)
    wall = time.perf_counter() - t0
    elements = sum(n * cols for _, n, cols, _ in reqs)
    lat.sort()
    return elements / wall, {"p50_ms": lat[len(lat) // 2], "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))]}, wall, outs
