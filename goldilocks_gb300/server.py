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
        return self.wait_timed(rid, timeout_ms)[0]

    def wait_timed(self, rid, timeout_ms=60000):
        """(status, submit-to-completion milliseconds) of a request."""
        s, lat = ctypes.c_int(), ctypes.c_double()
        st = self._lib.gl_server_wait_timed(self._h, rid, timeout_ms, ctypes.byref(s), ctypes.byref(lat))
        if st != L.GL_OK:
            raise GoldilocksError(st, "wait")
        return s.value, lat.value

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


SMALL_WORDS = 1 << 21  # the server's small-request class: at most this many output words


def _is_small(req):
    return _out_words(*req) <= SMALL_WORDS


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


def _percentiles(lat_ms):
    v = sorted(lat_ms)
    if not v:
        return {"p50_ms": 0.0, "p99_ms": 0.0, "max_ms": 0.0}
    q = lambda f: v[min(len(v) - 1, int(f * len(v)))]
    return {"p50_ms": q(0.50), "p99_ms": q(0.99), "max_ms": v[-1]}


def serve_stream(reqs, arrivals, pool, budget_bytes=64 << 30, slots=4, max_batch=64, ring_words=0,
                 keep=()):
    """Submit each request at its arrival time (seconds from start), wait for
    all; returns (elements/s, stats, wall seconds, outputs).  stats adds to the
    server's counters each request's latency from its arrival to its
    completion (`latency_ms`, and p50/p99 of it).  With ring_words > 0 the
    outputs share a ring of that many words: each returned output is a view of
    the ring, which a later request may have overwritten -- except the
    requests whose indices are in `keep`, which get buffers of their own.
    Small and large requests (the server's classes) are submitted by two
    client threads, each with an output ring of its own (the small one a
    sixteenth of ring_words, at least 2^22 words, at most half), so that a
    client waiting for ring space never delays the other class's
    submissions."""
    import threading

    import torch
    keep = set(keep)
    classes = {True: [k for k in range(len(reqs)) if _is_small(reqs[k])],
               False: [k for k in range(len(reqs)) if not _is_small(reqs[k])]}
    ins = [pool[:n * c] for _, n, c, _ in reqs]
    if ring_words:
        small_words = min(ring_words // 2, max(ring_words // 16, 1 << 22))
        ring = {True: _Ring(torch, small_words), False: _Ring(torch, ring_words - small_words)}
        own = {k: torch.empty(_out_words(*reqs[k]), dtype=torch.int64, device="cuda") for k in sorted(keep)}
    else:
        ring, own = None, {}
        _, outs_all = _buffers(torch, reqs, pool)
        own = dict(enumerate(outs_all))
    torch.cuda.synchronize()
    outs = [None] * len(reqs)
    lat = [0.0] * len(reqs)
    sub = [None] * len(reqs)  # (rid, submit time) per request
    lock = threading.Lock()
    waited = set()
    errors = []
    with Server(budget_bytes, slots, max_batch) as srv:
        def wait(k):
            with lock:
                if k in waited:
                    return
                waited.add(k)
            rid, t_sub = sub[k]
            st, ms = srv.wait_timed(rid, timeout_ms=600000)
            if st != L.GL_OK:
                raise GoldilocksError(st, "request")
            lat[k] = (t_sub - arrivals[k]) * 1e3 + ms  # from arrival, not from submission

        def client(small):
            try:
                r = ring[small] if ring else None
                for k in classes[small]:
                    op, n, cols, blowup = reqs[k]
                    now = time.perf_counter() - t0
                    if arrivals[k] > now:
                        time.sleep(arrivals[k] - now)
                    if k in own:
                        o = own[k]
                    else:
                        o, lo, hi = r.take(_out_words(op, n, cols, blowup), wait)
                    outs[k] = o
                    t_sub = time.perf_counter() - t0
                    rid = srv.submit(op, n, cols, ins[k], o, blowup)
                    sub[k] = (rid, max(t_sub, float(arrivals[k])))
                    if r is not None and k not in own:
                        r.live.append((k, lo, hi))
            except Exception as e:  # reported by the caller
                errors.append(e)

        t0 = time.perf_counter()
        threads = [threading.Thread(target=client, args=(c,)) for c in (True, False)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if errors:
            raise errors[0]
        for k in range(len(reqs)):
            wait(k)
        wall = time.perf_counter() - t0
        stats = srv.stats()
    stats["latency_ms"] = lat
    stats.update({"arrival_" + k: v for k, v in _percentiles(lat).items()})
    elements = sum(n * cols for _, n, cols, _ in reqs)
    return elements / wall, stats, wall, outs


def plain_call(lib, stream, op, n, cols, blowup, inp, out):
    """One request through the plain per-call API: gl_coset_lde, or a copy
    and the in-place column transform (the reference's ntt/intt are in place)."""
    if op == GL_OP_LDE:
        return lib.gl_coset_lde(inp.data_ptr(), out.data_ptr(), n, cols, blowup, 7, L.GL_MEM_DEVICE, stream)
    out.copy_(inp)
    d = L.GL_INVERSE if op == GL_OP_INTT else L.GL_FORWARD
    return lib.gl_ntt_columns(out.data_ptr(), n, cols, d, L.GL_MEM_DEVICE, stream)


def serial_baseline(reqs, pool, ring_words=0):
    """The same requests one at a time through the plain API (gl_ntt_columns,
    gl_coset_lde), each synchronised before the next starts.  Returns
    (elements/s, latency percentiles, wall seconds, outputs); the latencies
    are service times (no queueing), also listed per request as
    `service_ms`.  With ring_words > 0 every output reuses one buffer (no
    outputs returned)."""
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
        st = plain_call(lib, stream, op, n, cols, blowup, i, o)
        if st != L.GL_OK:
            raise GoldilocksError(st, "serial")
        torch.cuda.synchronize()
        lat.append((time.perf_counter() - t) * 1e3)
    wall = time.perf_counter() - t0
    elements = sum(n * cols for _, n, cols, _ in reqs)
    pct = _percentiles(lat)
    pct["service_ms"] = lat
    return elements / wall, pct, wall, outs


def serial_fifo(service_ms, arrivals):
    """Latencies of the serial path under the same arrivals: one request at a
    time in arrival order (a single FIFO server), request k taking its
    measured serial service time: finish_k = max(arrival_k, finish_(k-1)) +
    service_k.  Returns (latency percentiles and per-request latencies, wall
    seconds from the first arrival to the last finish)."""
    finish, lat = 0.0, []
    for a, s in zip(arrivals, service_ms):
        finish = max(float(a), finish) + s * 1e-3
        lat.append((finish - float(a)) * 1e3)
    pct = _percentiles(lat)
    pct["latency_ms"] = lat
    return pct, finish - float(arrivals[0]) if len(arrivals) else 0.0


def check_sample(reqs, count, seed, max_words):
    """Indices of requests whose served outputs are kept and checked: the
    largest request of each operation whose output is at most a quarter of
    max_words, then a seeded sample, while the kept outputs total at most
    max_words."""
    rng = np.random.default_rng(seed)
    order = []
    for op in (GL_OP_LDE, GL_OP_NTT, GL_OP_INTT):
        ks = [k for k, r in enumerate(reqs) if r[0] == op and _out_words(*r) <= max_words // 4]
        if ks:
            order.append(max(ks, key=lambda k: _out_words(*reqs[k])))
    order += [int(k) for k in rng.permutation(len(reqs))]
    chosen, words = [], 0
    for k in order:
        w = _out_words(*reqs[k])
        if k in chosen or words + w > max_words:
            continue
        chosen.append(k)
        words += w
        if len(chosen) >= count:
            break
    return sorted(chosen)


def check_outputs(reqs, pool, outs, indices):
    """Compare served outputs with the plain per-call API's result for the
    same request (ntt/src/ntt/mod.rs:98-120 restated on the GPU: the path the
    GPU tests check against the oracle), bit for bit, on the device.  Returns
    the indices that differ."""
    import torch
    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    bad = []
    for k in indices:
        op, n, cols, blowup = reqs[k]
        ref = torch.empty(_out_words(op, n, cols, blowup), dtype=torch.int64, device="cuda")
        st = plain_call(lib, stream, op, n, cols, blowup, pool[:n * cols], ref)
        if st != L.GL_OK:
            raise GoldilocksError(st, "check")
        if not torch.equal(ref, outs[k]):
            bad.append(k)
        del ref
    torch.cuda.synchronize()
    return bad


def compare_at_loads(reqs, pool, loads, seed, budget_bytes=64 << 30, slots=4, max_batch=64,
                     ring_words=0, check=0, check_words=0, p99_bound=2.0):
    """The serving comparison: serial plain calls back to back (service
    times), then for each offered load (a multiple of the rate the serial path
    sustains) the served stream at those Poisson arrivals beside the serial
    path under the same arrivals (a FIFO queue of the measured service times).
    With check > 0, that many served outputs per load (seeded sample,
    including the largest request of each operation) are compared with the
    plain call's.  Reports elements/s and p50/p99 latency from arrival, and
    the best served rate whose p99 is within p99_bound times the serial
    p99 at the same load."""
    ser_rate, ser_lat, ser_wall, _ = serial_baseline(reqs, pool, ring_words=ring_words or 1)
    elements = sum(n * c for _, n, c, _ in reqs)
    small = [k for k, r in enumerate(reqs) if _is_small(r)]
    res = {"requests": len(reqs), "elements": elements,
           "serial": {"elem_s": ser_rate, "wall_s": ser_wall, "service_p50_ms": ser_lat["p50_ms"],
                      "service_p99_ms": ser_lat["p99_ms"]},
           "loads": [], "checked": 0, "mismatches": []}
    offered = len(reqs) / ser_wall  # requests/s the serial path sustains
    for load in loads:
        arrivals = poisson_arrivals(len(reqs), rate_per_s=offered * load, seed=seed)
        fifo, fifo_wall = serial_fifo(ser_lat["service_ms"], arrivals)
        keep = check_sample(reqs, check, seed + int(load * 1000), check_words) if check else []
        rate, stats, wall, outs = serve_stream(reqs, arrivals, pool, budget_bytes=budget_bytes, slots=slots,
                                               max_batch=max_batch, ring_words=ring_words, keep=keep)
        if keep:
            res["mismatches"] += [int(k) for k in check_outputs(reqs, pool, outs, keep)]
            res["checked"] += len(keep)
        del outs
        sl = stats["latency_ms"]
        entry = {"load": load, "offered_req_s": offered * load,
                 "served": {"elem_s": rate, "wall_s": wall, "p50_ms": stats["arrival_p50_ms"],
                            "p99_ms": stats["arrival_p99_ms"], "batches": stats["batches"],
                            "small_p99_ms": _percentiles([sl[k] for k in small])["p99_ms"]},
                 "serial_same_arrivals": {"elem_s": elements / fifo_wall if fifo_wall else 0.0,
                                          "p50_ms": fifo["p50_ms"], "p99_ms": fifo["p99_ms"],
                                          "small_p99_ms": _percentiles([fifo["latency_ms"][k] for k in small])["p99_ms"]}}
        res["loads"].append(entry)
    ok = [e for e in res["loads"] if e["served"]["p99_ms"] <= p99_bound * e["serial_same_arrivals"]["p99_ms"]]
    best = max(ok, key=lambda e: e["served"]["elem_s"]) if ok else None
    res["p99_bound"] = "served p99 <= %g x serial p99 at the same arrivals" % p99_bound
    res["best_within_bound"] = None if best is None else {
        "load": best["load"], "served_elem_s": best["served"]["elem_s"],
        "serial_elem_s_same_arrivals": best["serial_same_arrivals"]["elem_s"],
        "serial_elem_s_back_to_back": ser_rate,
        "served_p99_ms": best["served"]["p99_ms"], "serial_p99_ms": best["serial_same_arrivals"]["p99_ms"]}
    return res


def main(argv=None):
    """The serving workload at full size: NTT/iNTT/LDE (40/30/30, blowup 4,
    shift 7), log2 n uniform in [10, 24], 1..64 columns, Poisson arrivals at
    multiples of the rate the serial path sustains, a 64 GB admission budget;
    outputs share a ring (default 96 GiB), except a seeded sample (with the
    largest request of each operation) kept and compared bit for bit with the
    plain per-call result.  Prints one JSON line."""
    import argparse
    import json

    import torch

    from .ntt import fill_uniform
    ap = argparse.ArgumentParser(prog="python -m goldilocks_gb300.server")
    ap.add_argument("--requests", type=int, default=20000)
    ap.add_argument("--log-min", type=int, default=10)
    ap.add_argument("--log-max", type=int, default=24)
    ap.add_argument("--max-cols", type=int, default=64)
    ap.add_argument("--loads", type=str, default="0.5,0.9,1.0,2.0",
                    help="offered load as multiples of the serial rate")
    ap.add_argument("--ring-gib", type=int, default=96)
    ap.add_argument("--check", type=int, default=64, help="served outputs compared per load")
    ap.add_argument("--check-gib", type=int, default=48, help="memory for the kept outputs")
    ap.add_argument("--seed", type=int, default=0x5E77)
    args = ap.parse_args(argv)
    torch.cuda.set_device(0)
    reqs = make_requests(args.requests, seed=args.seed, log_min=args.log_min, log_max=args.log_max,
                         max_cols=args.max_cols)
    pool = torch.from_numpy(fill_uniform(max(n * c for _, n, c, _ in reqs), seed=5).view(np.int64)).cuda()
    res = compare_at_loads(reqs, pool, [float(x) for x in args.loads.split(",")], args.seed,
                           ring_words=(args.ring_gib << 30) // 8, check=args.check,
                           check_words=(args.check_gib << 30) // 8)
    res.update({"workload": "serving", "log2_n": [args.log_min, args.log_max], "cols": [1, args.max_cols],
                "mix": "40/30/30 ntt/intt/lde, blowup 4", "budget_gb": 64, "ring_gib": args.ring_gib})
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
