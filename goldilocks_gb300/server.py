"""Continuous-batching request server (gl_server_*) and a load generator.

    srv = Server(budget_bytes=64 << 30, slots=4, max_batch=64)
    rid = srv.submit(GL_OP_NTT, n, cols, inp, out)      # device tensors
    srv.wait(rid)                                       # status, or raises

`serve_stream` replays a request list with Poisson arrival times against a
server and reports throughput and p50/p99 latency; `serial_baseline` runs the
same requests one at a time through the plain per-call API on the same GPU.
"""
import collections
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


def _out_words(op, n, cols, blowup):
    return n * cols * (blowup if op == GL_OP_LDE else 1)


def _buffers(torch, reqs, pool):
    """Per request: input = a slice of a resident pool, output = its own buffer."""
    outs, ins = [], []
    for op, n, cols, blowup in reqs:
        ins.append(pool[:n * cols])
        outs.append(torch.empty(_out_words(op, n, cols, blowup), dtype=torch.int64, device="cuda"))
    return ins, outs


class _Ring:
    """Output regions carved in submission order from one device buffer.  A
    region is handed out again only after the request that wrote it has been
    waited for, so the requests in flight are bounded by the buffer's size
    (the submitter blocks on the oldest request when it runs out)."""

    def __init__(self, torch, words):
        self.buf = torch.empty(words, dtype=torch.int64, device="cuda")
        self.words, self.head = words, 0
        self.live = collections.deque()  # (rid, start, end), oldest first

    def take(self, words, wait):
        if words > self.words:
            raise ValueError("request output (%d words) exceeds the output ring (%d)" % (words, self.words))
        if self.head + words > self.words:
            self.head = 0
        start, end = self.head, self.head + words
        # After a wrap the oldest region may lie past the new one while a newer
        # one overlaps it: wait oldest first until none overlaps.
        while any(lo < end and start < hi for _, lo, hi in self.live):
            wait(self.live.popleft()[0])
        self.head = end
        return self.buf[start:end], start, end


def serve_stream(reqs, arrivals, pool, budget_bytes=64 << 30, slots=4, max_batch=64, ring_words=0):
    """Submit each request at its arrival time (seconds from start), wait for
    all; returns (elements/s, stats, wall seconds, outputs).  With ring_words
    > 0 the outputs share a ring of that many words: each returned output is
    a view of the ring, which a later request may have overwritten."""
    import torch
    if ring_words:
        ins, outs, ring = [pool[:n * c] for _, n, c, _ in reqs], [], _Ring(torch, ring_words)
    else:
        (ins, outs), ring = _buffers(torch, reqs, pool), None
    torch.cuda.synchronize()
    pending = collections.OrderedDict()
    with Server(budget_bytes, slots, max_batch) as srv:
        def wait(rid):
            st = srv.wait(rid, timeout_ms=600000)
            pending.pop(rid, None)
            if st != L.GL_OK:
                raise GoldilocksError(st, "request")
        t0 = time.perf_counter()
        for k, ((op, n, cols, blowup), a, i) in enumerate(zip(reqs, arrivals, ins)):
            now = time.perf_counter() - t0
            if a > now:
                time.sleep(a - now)
            if ring:
                o, lo, hi = ring.take(_out_words(op, n, cols, blowup), wait)
                outs.append(o)
            else:
                o = outs[k]
            rid = srv.submit(op, n, cols, i, o, blowup)
            pending[rid] = True
            if ring:
                ring.live.append((rid, lo, hi))
        for rid in list(pending):
            wait(rid)
        wall = time.perf_counter() - t0
        stats = srv.stats()
    elements = sum(n * cols for _, n, cols, _ in reqs)
    return elements / wall, stats, wall, outs


def serial_baseline(reqs, pool, ring_words=0):
    """The same requests one at a time through the plain API (gl_ntt_columns,
    gl_coset_lde, gl_ntt/gl_intt), each synchronised before the next starts.
    With ring_words > 0 every output reuses one buffer (no outputs returned)."""
    import torch
    lib = L.load()
    if ring_words:
        ins, outs = [pool[:n * c] for _, n, c, _ in reqs], None
        scratch = torch.empty(max(_out_words(*r) for r in reqs), dtype=torch.int64, device="cuda")
    else:
        ins, outs = _buffers(torch, reqs, pool)
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    lat = []
    t0 = time.perf_counter()
    for k, ((op, n, cols, blowup), i) in enumerate(zip(reqs, ins)):
        o = outs[k] if outs is not None else scratch[:_out_words(op, n, cols, blowup)]
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


def main(argv=None):
    """The serving workload at full size: NTT/iNTT/LDE (40/30/30, blowup 4,
    shift 7), log2 n uniform in [10, 24], 1..64 columns, Poisson arrivals at
    0.5x and 2x the rate the serial path sustains, a 64 GB admission budget;
    outputs share a ring (default 96 GiB).  Prints one JSON line."""
    import argparse
    import json

    import torch

    from .ntt import fill_uniform
    ap = argparse.ArgumentParser(prog="python -m goldilocks_gb300.server")
    ap.add_argument("--requests", type=int, default=20000)
    ap.add_argument("--log-min", type=int, default=10)
    ap.add_argument("--log-max", type=int, default=24)
    ap.add_argument("--max-cols", type=int, default=64)
    ap.add_argument("--loads", type=str, default="0.5,2.0", help="offered load as multiples of the serial rate")
    ap.add_argument("--ring-gib", type=int, default=96)
    ap.add_argument("--seed", type=int, default=0x5E77)
    args = ap.parse_args(argv)
    torch.cuda.set_device(0)
    reqs = make_requests(args.requests, seed=args.seed, log_min=args.log_min, log_max=args.log_max,
                         max_cols=args.max_cols)
    pool = torch.from_numpy(fill_uniform(max(n * c for _, n, c, _ in reqs), seed=5).view(np.int64)).cuda()
    ring = (args.ring_gib << 30) // 8
    ser_rate, ser_lat, ser_wall, _ = serial_baseline(reqs, pool, ring_words=ring)
    res = {"workload": "serving", "requests": args.requests, "log2_n": [args.log_min, args.log_max],
           "cols": [1, args.max_cols], "mix": "40/30/30 ntt/intt/lde, blowup 4", "budget_gb": 64,
           "ring_gib": args.ring_gib, "elements": sum(n * c for _, n, c, _ in reqs),
           "serial": {"elem_s": ser_rate, "wall_s": ser_wall, "p50_ms": ser_lat["p50_ms"],
                      "p99_ms": ser_lat["p99_ms"]}, "served": []}
    offered = args.requests / ser_wall
    for load in (float(x) for x in args.loads.split(",")):
        arrivals = poisson_arrivals(args.requests, rate_per_s=offered * load, seed=args.seed)
        rate, stats, wall, _ = serve_stream(reqs, arrivals, pool, budget_bytes=64 << 30, slots=4,
                                            max_batch=64, ring_words=ring)
        res["served"].append({"offered_req_s": offered * load, "elem_s": rate, "wall_s": wall,
                              "p50_ms": stats["p50_ms"], "p99_ms": stats["p99_ms"],
                              "batches": stats["batches"]})
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
