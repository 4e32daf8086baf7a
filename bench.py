#!/usr/bin/env python
"""Benchmark of the GB300 Goldilocks NTT on the large-transform workload.

Workload ("large single transforms, plain per-call"): one step is a forward
and an inverse NTT at each of n = 2^20, 2^22, 2^24 and 16,711,680
(= 2^16*3*5*17), on seeded synthetic field elements uniform in [0, p).
Metric: elements transformed per second (each transform counts n).

  value      device-resident inputs, CUDA events on the launching stream around
             each step, L2 flushed (256 MiB write) between steps outside the
             timed events.
  e2e        the same step through the public API with pinned HOST buffers
             (gl_host_pipeline: one copy in and one copy out per buffer,
             overlapped with the transforms, synchronised, inside the timed
             region); e2e.per_call: one synchronous gl_plan_execute with
             GL_MEM_HOST per transform.
  issue_roofline  the same kernel against the instruction-issue peak (the
             bound these integer kernels meet), from the ncu instruction count
             per element.
  roofline   the kernel with the largest share of device time, its algorithmic
             bytes per launch (16 B per element per pass: one read + one write)
             over its mean CUDA-event launch time, against the measured HBM
             copy bandwidth.
  cpu_baseline  the CPU oracle (a C restatement of the reference's CPU path,
             kind "port") on the same step, transforms spread over host threads.

--impl reference times the reference's CPU algorithm (the C restatement; the
reference is Rust and no Rust toolchain exists here) on all usable host
threads, for the same metric and workload.
"""
import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIZES = [1 << 20, 1 << 22, 1 << 24, 16711680]
METRIC = "bit-exact NTT elem/s (fwd+inv at 2^20, 2^22, 2^24, 16711680)"
UNIT = "elem/s"
WORKLOAD = {"workload": "large single transforms, plain per-call: forward+inverse NTT at "
                        "n=2^20, 2^22, 2^24, 16711680 (2^16*3*5*17)",
            "sizes": SIZES, "transforms_per_step": 2 * len(SIZES),
            "elements_per_step": 2 * sum(SIZES), "field": "Goldilocks p=2^64-2^32+1",
            "inputs": "uniform in [0,p), seeded splitmix64 stream (gl_fill_uniform; oracle.fill_uniform for the CPU legs)",
            "l2": "flushed between steps (256 MiB write, outside timed events)"}


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(dist, x, device):
    """The largest value of x over all ranks (x itself without a process
    group): a step counts as long as its slowest replica."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, units_per_rank, seconds):
    """Units processed by all replicas per second of the slowest one."""
    return world * units_per_rank / seconds


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names[1:], parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "samples": len(sm),
                "reasons": sorted(reasons)}


# Sources whose change invalidates the committed ncu figures of the pass kernels.
KERNEL_SOURCES = ("gl_pass3.cuh", "gl_pass.cuh", "gl_field.cuh", "gl_codelets.cuh", "gl_kernels_impl.cuh",
                  "gl_kern_pass_fwd.cu", "gl_kern_pass_inv.cu", "gl_kern_mixed17_fwd.cu", "gl_kern_mixed17_inv.cu")


def kernel_source_sha():
    """sha256 (first 16 hex digits) of the pass-kernel sources, in a fixed
    order, with comments and runs of white space removed (an edit of a
    comment does not change the kernels)."""
    import hashlib
    import re
    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        with open(os.path.join(ROOT, "goldilocks_gb300", "csrc", name), "rb") as f:
            code = re.sub(rb"/\*.*?\*/", b" ", f.read(), flags=re.S)
        code = re.sub(rb"\s+", b" ", re.sub(rb"//[^\n]*", b" ", code)).strip()
        h.update(name.encode() + b"\0" + code)
    return h.hexdigest()[:16]


def ncu_per_element():
    """Per-element figures of each pass kernel from the committed ncu capture
    (profiles/ncu_pass_kernels.json: DRAM bytes read + written and thread
    instructions executed per element), or ({}, reason) when the file is
    missing or was measured on other kernel sources than these."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_pass_kernels.json")) as f:
            d = json.load(f)
    except Exception as e:
        return {}, "no committed ncu figures (%s)" % type(e).__name__
    if d.get("source_sha") != kernel_source_sha():
        return {}, "committed ncu figures are for other kernel sources (sha %s, now %s)" % (
            d.get("source_sha"), kernel_source_sha())
    return d.get("kernels", {}), None


def host_cpu():
    """The host's usable threads and CPU model (x86 'model name', or the Arm
    implementer/part codes when /proc/cpuinfo has no model name)."""
    try:
        usable = len(os.sched_getaffinity(0))
    except Exception:
        usable = os.cpu_count() or 1
    model, arm = None, {}
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k, _, v = line.partition(":")
                k, v = k.strip(), v.strip()
                if k == "model name" and model is None:
                    model = v
                elif k in ("CPU implementer", "CPU part") and k not in arm:
                    arm[k] = v
    except OSError:
        pass
    if model is None:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=5).stdout
            for line in out.splitlines():
                if line.startswith("Model name:"):
                    model = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    if model is None and arm:
        model = "arm implementer %s part %s" % (arm.get("CPU implementer"), arm.get("CPU part"))
    return {"nproc": os.cpu_count(), "usable_threads": usable, "model": model}


def cpu_oracle_run(steps, threads):
    """`steps` steps of the workload on the CPU oracle, every transform of
    every step one job on a pool of `threads` host threads (a transform runs
    on one thread, as the reference's does below its parallel work size
    MIN_WORK_SIZE = 2^24 elements); returns (elements, seconds).  The inputs
    come from the oracle's own generator (the same seeded stream as the GPU
    arm's), so this leg never loads the product library."""
    import oracle
    oracle.build()
    inputs = [oracle.fill_uniform(n, seed=0xC0 + i) for i, n in enumerate(SIZES)]

    def job(args):
        i, inv = args
        x = inputs[i]
        return (oracle.intt(x) if inv else oracle.ntt(x)).size

    jobs = [(i, inv) for _ in range(steps) for i in range(len(SIZES)) for inv in (0, 1)]
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        total = sum(ex.map(job, jobs))
    return total, time.perf_counter() - t0


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    cpu = host_cpu()
    threads = cpu["usable_threads"]
    if args.warmup > 0:
        cpu_oracle_run(1, threads)
    tot_el, tot_s = cpu_oracle_run(args.steps, threads)
    v = tot_el / tot_s
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (mod p)",
            "data": "synthetic", "config": WORKLOAD,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "host": cpu,
                             "sample": "%d steps of 8 transforms on a pool of %d host threads (one "
                                       "transform per thread); C restatement of the reference CPU "
                                       "algorithm (no Rust toolchain to build the reference itself)"
                                       % (args.steps, threads)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def bench_batched(gl, torch, reps=3):
    """Config 3: 1024 polynomials, log2 n ~ U[12, 18] (seeded), odd index
    inverse, one batch per step; elements/s per execution mode."""
    import numpy as np
    from goldilocks_gb300 import batch as B
    rng = np.random.default_rng(0xBA7C)
    sizes = [1 << int(k) for k in rng.integers(12, 19, 1024)]
    pool = torch.from_numpy(gl.fill_uniform(sum(sizes), seed=0xBA7C).view(np.int64)).cuda()
    items, off = [], 0
    for i, n in enumerate(sizes):
        items.append((pool[off:off + n], i % 2))
        off += n
    out = {"polys": len(sizes), "elements": int(sum(sizes))}
    stream = torch.cuda.current_stream()
    for name, mode in (("per_call", B.PER_CALL), ("buckets", B.BUCKETS), ("persistent", B.PERSISTENT)):
        B.run(items, mode=mode)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            B.run(items, mode=mode)
        b.record(stream)
        b.synchronize()
        out[name + "_elem_s"] = out["elements"] * reps / (a.elapsed_time(b) * 1e-3)
    out["persistent_vs_per_call"] = out["persistent_elem_s"] / out["per_call_elem_s"]
    # Roofline of the batch: sum of B(n_i) = 16 n_i P(n_i) bytes over the batch's
    # time, against the measured HBM copy bandwidth.
    import math
    peak, peak_kind = peaks()
    out["algorithmic_bytes"] = alg = sum(16 * n * math.ceil(math.log2(n) / 14) for n in sizes)
    # The same batch through run_packed: (offset, length, direction) arrays
    # over the pool, so the host builds the descriptor array in one numpy
    # step instead of one Python call per polynomial.
    offs = np.cumsum([0] + sizes[:-1])
    dirs = [i % 2 for i in range(len(sizes))]
    for name, mode in (("buckets_packed", B.BUCKETS), ("persistent_packed", B.PERSISTENT)):
        B.run_packed(pool, offs, sizes, dirs, mode=mode)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            B.run_packed(pool, offs, sizes, dirs, mode=mode)
        b.record(stream)
        b.synchronize()
        out[name + "_elem_s"] = out["elements"] * reps / (a.elapsed_time(b) * 1e-3)
    for name in ("buckets_packed", "persistent_packed", "buckets", "persistent"):
        t = out["elements"] / out[name + "_elem_s"]
        out[name + "_frac"] = alg / t / 1e9 / peak
    out["peak_gbs"], out["peak_kind"] = peak, peak_kind
    # The schedules of the batch's lengths measured first (gl_plan_autotune),
    # then buckets again, and AUTO with the mode gl_batch_autotune measured.
    from goldilocks_gb300 import tune
    try:
        for n in sorted(set(sizes)):
            tune.autotune(n, reps=10)
        for name, mode in (("buckets_tuned", B.BUCKETS), ("auto_tuned", B.AUTO)):
            if mode == B.AUTO:
                B.autotune(items, reps=2)
            B.run(items, mode=mode)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                B.run(items, mode=mode)
            b.record(stream)
            b.synchronize()
            out[name + "_elem_s"] = out["elements"] * reps / (a.elapsed_time(b) * 1e-3)
    finally:
        tune.clear()
    return out


def bench_serving(gl, torch, count=1500, log_max=24, loads=(0.5, 0.9, 1.5)):
    """Config 5 (the configured size distribution, fewer requests): Poisson
    stream of NTT/iNTT/LDE (40/30/30) requests, log2 n ~ U[10, 24], 1..64
    columns, 64 GB admission budget; served (continuous batching, small
    requests on a high-priority slot) against serial plain launches -- back
    to back, and as a FIFO queue under the same arrivals; latencies from
    arrival.  A seeded sample of served outputs (with the largest request of
    each operation) is compared with the plain per-call result."""
    from goldilocks_gb300 import server as S
    import numpy as np
    reqs = S.make_requests(count, seed=0x5E77, log_min=10, log_max=log_max, max_cols=64)
    pool = torch.from_numpy(gl.fill_uniform(max(n * c for _, n, c, _ in reqs), seed=5).view(np.int64)).cuda()
    res = S.compare_at_loads(reqs, pool, loads, seed=0x5E77, budget_bytes=64 << 30, slots=4, max_batch=64,
                             ring_words=(64 << 30) // 8, check=24, check_words=(40 << 30) // 8)
    res.update({"log2_n": [10, log_max], "cols": [1, 64], "mix": "40/30/30 ntt/intt/lde, blowup 4"})
    del pool
    torch.cuda.empty_cache()
    return res


def _time_ms(torch, fn, reps):
    stream = torch.cuda.current_stream()
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        fn()
    b.record(stream)
    b.synchronize()
    return a.elapsed_time(b) / reps


def bench_commit(gl, torch, reps=3):
    """Config 4 and the step after it: coset LDE of a 2^20 x 256 row-major
    matrix (blowup 4, shift 7) to 2^22 x 256, then the K12 Merkle tree of the
    8 GiB result (pcs/src/k12/mod.rs:41-60)."""
    import numpy as np
    from goldilocks_gb300 import _lib as L
    lib = L.load()
    n, cols, blowup = 1 << 20, 256, 4
    s = torch.cuda.current_stream().cuda_stream
    inp = torch.from_numpy(gl.fill_uniform(n * cols, seed=0xC0417).view(np.int64)).cuda()
    out = torch.empty(n * blowup * cols, dtype=torch.int64, device="cuda")
    leaves = out.numel() * 8
    tree_bytes = lib.gl_merkle_tree_bytes(leaves)
    tree = torch.empty(tree_bytes, dtype=torch.uint8, device="cuda")

    def lde():
        assert lib.gl_coset_lde(inp.data_ptr(), out.data_ptr(), n, cols, blowup, 7, L.GL_MEM_DEVICE, s) == 0

    def merkle():
        assert lib.gl_merkle_tree(out.data_ptr(), leaves, tree.data_ptr(), tree_bytes, L.GL_MEM_DEVICE, s) == 0

    lde_ms = _time_ms(torch, lde, reps)
    merkle_ms = _time_ms(torch, merkle, reps)
    import math
    alg = cols * sum(16 * m * math.ceil(math.log2(m) / 14) for m in (n, n * blowup))
    peak, peak_kind = peaks()
    res = {"shape": "2^20 x 256 -> 2^22 x 256, blowup 4, shift 7",
           "lde_ms": lde_ms, "lde_rows_cols_per_s": n * cols / (lde_ms * 1e-3),
           "lde_algorithmic_gbs": alg / (lde_ms * 1e-3) / 1e9,
           "lde_frac": alg / (lde_ms * 1e-3) / 1e9 / peak, "peak_gbs": peak, "peak_kind": peak_kind,
           "merkle_ms": merkle_ms, "merkle_leaf_bytes": leaves,
           "merkle_leaf_gbs": leaves / (merkle_ms * 1e-3) / 1e9,
           "merkle_permutations_per_s": (leaves + tree_bytes) / 160 / (merkle_ms * 1e-3),
           "commit_ms": lde_ms + merkle_ms}
    del inp, out, tree
    torch.cuda.empty_cache()
    return res


def bench_convolve(gl, torch, reps=5):
    """convolve::circular at n = 2^24 (ntt, fused pointwise product, intt)."""
    import numpy as np
    n = 1 << 24
    a = torch.from_numpy(gl.fill_uniform(n, seed=0xC011).view(np.int64)).cuda()
    b = torch.from_numpy(gl.fill_uniform(n, seed=0xC012).view(np.int64)).cuda()
    ms = _time_ms(torch, lambda: gl.convolve(a, b), reps)
    return {"n": n, "ms": ms, "elem_s": n / (ms * 1e-3), "repr": "montgomery"}


def bench_pow(torch):
    """Pow::solve (pcs/src/pow.rs:39-60): the reference's 32-bit case
    (challenge 0xaa * 32, answer 440258853) and the raw hash rate over 2^33
    nonces with a threshold nothing meets."""
    from goldilocks_gb300.k12 import Pow
    p = Pow(bytes([0xAA] * 32), Pow.threshold_from_bits(32.0))
    p.solve()
    t = time.perf_counter()
    nonce = p.solve()
    solve_s = time.perf_counter() - t
    scan = Pow(bytes([0x11] * 32), 2**64 - 1)
    t = time.perf_counter()
    scan.solve(max_count=1 << 33)
    scan_s = time.perf_counter() - t
    return {"solve_32bit_nonce": nonce, "solve_32bit_s": solve_s,
            "hashes_per_s": (1 << 33) / scan_s}


def bench_small(gl, torch):
    """The reference's CPU-runnable case: one transform of n = 2^16 and a round
    trip.  Device-resident time per forward call, 200 back to back, through
    the C ABI (gl_plan_execute_ws with a workspace: the device time, the host
    issues a call in less) and through the Python API (pl.ntt: bound by its
    host time); the synchronous round trip of a host buffer through the
    drop-in API; and the oracle's single-thread forward time on the same
    input."""
    import numpy as np
    import oracle
    from goldilocks_gb300 import _lib as L
    n = 1 << 16
    x = gl.fill_uniform(n, seed=0x5EED0001)
    d = torch.from_numpy(x.view(np.int64)).cuda()
    pl = gl.strategy(n)
    lib = L.load()
    wsb = pl.workspace_bytes(1)
    ws = torch.empty(max(wsb // 8, 1), dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    args = (pl._h, d.data_ptr(), n, L.GL_FORWARD, ws.data_ptr(), wsb, s)
    fwd_ms = _time_ms(torch, lambda: lib.gl_plan_execute_ws(*args), 200)
    py_ms = _time_ms(torch, lambda: pl.ntt(d), 200)
    h = torch.empty(n, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    h[:] = x
    pl.ntt(h)
    pl.intt(h)
    t = time.perf_counter()
    for _ in range(50):
        pl.ntt(h)
        pl.intt(h)
    rt_us = (time.perf_counter() - t) / 50 * 1e6
    assert np.array_equal(h, x)
    oracle.build()
    oracle.ntt(x)
    t = time.perf_counter()
    for _ in range(5):
        oracle.ntt(x)
    cpu_us = (time.perf_counter() - t) / 5 * 1e6
    return {"n": n, "fwd_us_device": fwd_ms * 1e3, "fwd_us_python_api": py_ms * 1e3,
            "roundtrip_us_host_memory": rt_us, "cpu_oracle_fwd_us_1_thread": cpu_us}


def cpu_oracle_k12_rate(seconds=2.0):
    """Single-thread rate of the K12 oracle (C restatement of
    pcs/src/k12/generic.rs) on 160-byte blocks."""
    import oracle
    data = bytes(range(256)) * 640  # 1024 blocks
    oracle.k12_process_layer(data)
    t, reps = time.perf_counter(), 0
    while time.perf_counter() - t < seconds:
        oracle.k12_process_layer(data)
        reps += 1
    return reps * 1024 / (time.perf_counter() - t)


def run_ours(args):
    import numpy as np
    import torch

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from goldilocks_gb300 import build as gbuild
    gbuild.build()
    import goldilocks_gb300 as gl
    from goldilocks_gb300 import _lib as L

    lib = L.load()
    stream = torch.cuda.current_stream()
    plans = [gl.strategy(n) for n in SIZES]
    bufs = []
    for i, n in enumerate(SIZES):
        x = gl.fill_uniform(n, seed=0xBE00 + i + 16 * rank)
        bufs.append(torch.from_numpy(x.view(np.int64)).cuda())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    elements_per_step = 2 * sum(SIZES)

    def step():
        for pl, b in zip(plans, bufs):
            pl.ntt(b)
            pl.intt(b)

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    clocks = ClockSampler(local)
    clocks.start()
    evs = []
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    gc.collect()
    gc.disable()  # no collector pauses between the timed launches (see timed() below)
    for _ in range(args.steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        evs.append((a, b))
    torch.cuda.synchronize()
    gc.enable()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    total_ms = sum(a.elapsed_time(b) for a, b in evs)
    # Per-kernel launch times: the same steps again, every launch bracketed by
    # CUDA events on its stream (the library's profile).  Kept out of the steps
    # timed above: an event between two passes stops the second from starting
    # early (programmatic dependent launch), so bracketed steps run slower.
    lib.gl_profile_enable(1)
    gc.disable()
    for _ in range(args.steps):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    gc.enable()
    n_ent = lib.gl_profile_read(None, 0)
    ents = (L.ProfileEntry * max(n_ent, 1))()
    lib.gl_profile_read(ents, n_ent)
    lib.gl_profile_enable(0)
    prof = [{"name": e.name.decode(), "launches": int(e.launches), "elements": int(e.elements),
             "total_ms": float(e.total_ms)} for e in ents[:n_ent]]
    launches = sum(p["launches"] for p in prof)

    total_ms = max_over_ranks(dist, total_ms, "cuda")
    value = whole_job_rate(world, elements_per_step * args.steps, total_ms * 1e-3)

    # ---- end to end through the public API with pinned host buffers ----
    def pinned_set(seed):
        out = []
        for i, n in enumerate(SIZES):
            h = torch.empty(n, dtype=torch.int64, pin_memory=True)
            h.numpy().view(np.uint64)[:] = gl.fill_uniform(n, seed=seed + i)
            out.append(h.numpy().view(np.uint64))
        return out
    hosts = pinned_set(0xE2E0)
    hosts_b = pinned_set(0xE2F0)  # the second step in flight
    e2e_steps = max(1, min(args.steps, 20))

    def host_step():
        # gl_host_pipeline: each buffer goes to the GPU once, gets the forward
        # and the inverse transform there, and comes back once; the copies of
        # one buffer overlap the compute and the opposite-direction copies of
        # the others.
        gl.host_pipeline([(h, n, ("fwd", "inv")) for h, n in zip(hosts, SIZES)])

    def host_step_per_call():
        # The drop-in path: one synchronous host-memory call per transform
        # (each a full round trip), as a caller of the reference's ntt/intt does.
        for pl, h in zip(plans, hosts):
            pl.ntt(h)
            pl.intt(h)

    step_ms = {}

    def timed(fn, name):
        # Two untimed calls, then e2e_steps timed ones (each synchronous);
        # the value is the total over the timed steps, and every step's time
        # is reported beside it so that an outlier is visible.
        # Python's garbage collector is paused inside the timed loop (as timeit
        # does): a full collection of this process's objects takes 10-20 ms,
        # host time that is not part of the work measured.
        fn()
        fn()
        if dist:
            dist.barrier()
        times = []
        gc.collect()
        gc.disable()
        try:
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                t = time.perf_counter()
                fn()
                times.append((time.perf_counter() - t) * 1e3)
            total = time.perf_counter() - t0
        finally:
            gc.enable()
        step_ms[name] = [round(x, 3) for x in times]
        return max_over_ranks(dist, total, "cuda")
    def timed_stream(name):
        # A stream of steps through gl_host_pipeline_submit / _wait: step s+1
        # is queued before step s is waited on (two steps in flight, on two
        # sets of pinned buffers), so one step's copy-ins run beside the
        # previous step's passes and copy-outs.  Every step's buffers still go
        # to the GPU and back inside the timed region; the reported step times
        # are the intervals between step completions.
        sets = (hosts, hosts_b)

        def run(k, marks=None):
            pend = None
            for st in range(k):
                tk = gl.host_pipeline_submit([(h, n, ("fwd", "inv")) for h, n in zip(sets[st % 2], SIZES)])
                if pend is not None:
                    pend.wait()
                    if marks is not None:
                        marks.append(time.perf_counter())
                pend = tk
            pend.wait()
            if marks is not None:
                marks.append(time.perf_counter())
        run(8)
        if dist:
            dist.barrier()
        gc.collect()
        gc.disable()
        try:
            marks = []
            t0 = time.perf_counter()
            run(e2e_steps, marks)
            total = time.perf_counter() - t0
        finally:
            gc.enable()
        step_ms[name] = [round((b - a) * 1e3, 3) for a, b in zip([t0] + marks[:-1], marks)]
        return max_over_ranks(dist, total, "cuda")
    # The per-call and one-step-at-a-time forms run first: on a fresh box the
    # first tens of milliseconds of copies from newly pinned host memory ran
    # slower (stream steps of 2.5 ms instead of 1.9 ms right after the device
    # steps above, 1.9 ms once warm), and they warm that up for the stream.
    per_call_s = timed(host_step_per_call, "per_call")
    sync_s = timed(host_step, "pipeline")
    e2e_s = timed_stream("stream")
    # Every step was a forward and an inverse transform: the buffers must hold
    # their inputs again.
    checked = all(np.array_equal(h, gl.fill_uniform(n, seed=seed + i))
                  for hs, seed in ((hosts, 0xE2E0), (hosts_b, 0xE2F0))
                  for i, (h, n) in enumerate(zip(hs, SIZES)))
    step_bytes = 8 * sum(SIZES)  # every buffer in once and out once
    e2e = {"value": whole_job_rate(world, elements_per_step * e2e_steps, e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": step_bytes, "d2h_bytes_per_step": step_bytes,
           "steps": e2e_steps, "step_ms": step_ms.get("stream"), "memory": "pinned host",
           "api": "gl_host_pipeline_submit / gl_host_pipeline_wait, two steps in flight",
           "round_trip_checked": checked,
           "one_step_at_a_time": {"value": whole_job_rate(world, elements_per_step * e2e_steps, sync_s),
                                  "step_ms": step_ms.get("pipeline"),
                                  "api": "gl_host_pipeline (synchronous, one step per call)"},
           "per_call": {"value": whole_job_rate(world, elements_per_step * e2e_steps, per_call_s),
                        "h2d_bytes_per_step": 2 * step_bytes, "d2h_bytes_per_step": 2 * step_bytes,
                        "step_ms": step_ms.get("per_call"),
                        "api": "gl_plan_execute per transform (GL_MEM_HOST)"}}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    peak, peak_kind = peaks()
    dom = max(prof, key=lambda p: p["total_ms"]) if prof else None
    roofline = None
    if dom:
        per_launch_el = dom["elements"] / dom["launches"]
        mean_ms = dom["total_ms"] / dom["launches"]
        achieved = 16.0 * per_launch_el / (mean_ms * 1e-3) / 1e9
        figs, stale = ncu_per_element()
        tr = figs.get(dom["name"], {}).get("dram_bytes_per_element")
        roofline = {"bound": "hbm", "kernel": dom["name"], "achieved": achieved, "peak": peak,
                    "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                    "traffic": (tr * per_launch_el) if tr else None,
                    "traffic_basis": stale or "ncu DRAM bytes per element of this kernel (committed capture of "
                                              "these sources, profiles/ncu_pass_kernels.json) x elements per launch",
                    "algorithmic_bytes_per_launch": 16.0 * per_launch_el,
                    "mean_launch_ms": mean_ms,
                    "launch_times": "CUDA events around every launch, on its stream, over a second run of "
                                    "the same %d steps (launches bracketed, so without programmatic "
                                    "dependent launch)" % args.steps,
                    "share": dom["total_ms"] / max(sum(p["total_ms"] for p in prof), 1e-12)}
    # The bound the passes actually meet: instruction issue (4 warp
    # instructions per SM per clock), from the ncu instruction count per
    # element and the live launch time, at the SM clock sampled during the run.
    issue = None
    inst = ncu_per_element()[0].get(dom["name"], {}).get("inst_per_element") if dom else None
    if inst and clk and clk.get("sm_mhz"):
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        per_launch_el = dom["elements"] / dom["launches"]
        mean_s = dom["total_ms"] / dom["launches"] * 1e-3
        achieved_i = inst / 32.0 * per_launch_el / mean_s / 1e9
        peak_i = sms * 4 * clk["sm_mhz"] * 1e6 / 1e9
        issue = {"bound": "integer issue", "kernel": dom["name"], "inst_per_element": inst,
                 "achieved": achieved_i, "peak": peak_i, "unit": "G warp-instructions/s",
                 "frac": achieved_i / peak_i,
                 "basis": "thread instructions per element from the committed ncu capture of these "
                          "kernel sources; 4 warp instructions per SM per clock at the sampled SM clock"}
    # whole-transform roofline: 16 B * n * passes(n) per transform, passes = ceil(log2 n / 14)
    import math
    alg_bytes = sum(2 * 16 * n * math.ceil(math.log2(n) / 14) for n in SIZES)
    step_ms = total_ms / args.steps

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64 (mod p)", "data": "synthetic",
            "config": WORKLOAD, "parallelism": "replicas" if world > 1 else "single GPU",
            "roofline": roofline,
            "issue_roofline": issue,
            "step_roofline": {"algorithmic_bytes_per_step": alg_bytes,
                              "achieved_gbs": alg_bytes / (step_ms * 1e-3) / 1e9,
                              "frac": alg_bytes / (step_ms * 1e-3) / 1e9 / peak},
            "e2e": e2e, "gpu_launches": launches, "clocks": clk,
            "kernels": prof}
    if world == 1 and not args.no_extras:
        try:
            line["batched"] = bench_batched(gl, torch)
        except Exception as e:  # reported, not fatal to the headline line
            line["batched"] = {"error": str(e)}
        try:
            line["serving"] = bench_serving(gl, torch)
        except Exception as e:
            line["serving"] = {"error": str(e)}
        for key, fn in (("small_2p16", lambda: bench_small(gl, torch)),
                        ("commit", lambda: bench_commit(gl, torch)),
                        ("convolve", lambda: bench_convolve(gl, torch)),
                        ("pow", lambda: bench_pow(torch))):
            try:
                line[key] = fn()
            except Exception as e:
                line[key] = {"error": str(e)}
        if not args.no_cpu_baseline:
            k12_rate = cpu_oracle_k12_rate()
            line["commit"]["cpu_oracle_k12_blocks_per_s_1_thread"] = k12_rate
            line["pow"]["cpu_oracle_hashes_per_s_1_thread"] = k12_rate
    if world == 1 and not args.no_cpu_baseline:
        cpu = host_cpu()
        threads = cpu["usable_threads"]
        el, s = cpu_oracle_run(2, threads)
        line["cpu_baseline"] = {"value": el / s, "unit": UNIT, "cores": threads, "kind": "port",
                                "host": cpu,
                                "sample": "two steps (16 transforms) of the C restatement of the "
                                          "reference CPU algorithm on a pool of %d host threads, one "
                                          "transform per thread" % threads}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the small-transform, batched, serving, commit, convolve and "
                         "proof-of-work figures")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
