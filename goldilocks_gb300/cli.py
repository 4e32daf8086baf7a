"""Command-line timing of single transforms, after the reference's bench binary
(bench/src/main.rs:111-189: sweep the divisors up to 2^max_exponent -- the
smooth ones, without the factors 17, 257, 65537, unless --all -- and print
`size,duration,throughput`).

  python -m goldilocks_gb300.cli --sizes 16777216 --reps 3     # one size
  python -m goldilocks_gb300.cli --max-exponent 24 --all       # every divisor
  python -m goldilocks_gb300.cli --algo merkle --max-exponent 24
  python -m goldilocks_gb300.cli --sizes 1048576 --cols 256 --lde 4
  python -m goldilocks_gb300.cli --max-exponent 26 --tune tuning.json   # tuned schedules
  python -m goldilocks_gb300.cli --batch 1024 --batch-mode persistent     # uneven batches

Algorithms (the reference's `--algo`): ntt, inverse, merkle (the K12 tree of
the size*8 bytes of field elements).  Inputs are device-resident; durations
are CUDA-event medians (seconds).
"""
import argparse
import statistics
import sys


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", type=str, default="", help="comma-separated sizes")
    ap.add_argument("--max-exponent", type=int, default=20)
    ap.add_argument("--all", action="store_true", help="all divisors, not only smooth ones")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--inverse", action="store_true", help="same as --algo inverse")
    ap.add_argument("--algo", choices=["ntt", "inverse", "merkle"], default="ntt")
    ap.add_argument("--cols", type=int, default=1, help="transform the columns of a rows x cols matrix")
    ap.add_argument("--lde", type=int, default=0, help="coset LDE with this blowup (shift 7)")
    ap.add_argument("--batch", type=int, default=0,
                    help="time batches of this many polynomials, log2 n uniform in [12, 18] (seeded)")
    ap.add_argument("--batch-mode", choices=["auto", "persistent", "buckets", "per_call"], default="auto")
    ap.add_argument("--batch-api", choices=["packed", "list"], default="packed",
                    help="batch.run_packed (offsets into one pool) or batch.run (a list of tensors)")
    ap.add_argument("--tune", type=str, default="",
                    help="autotune each size's schedule first and save the choices to this JSON file")
    args = ap.parse_args(argv)
    if args.inverse:
        args.algo = "inverse"

    import numpy as np
    import torch

    import goldilocks_gb300 as gl
    from goldilocks_gb300 import _lib as L

    lib = L.load()
    if args.batch:
        return _run_batch(args, gl, torch, np)
    if args.sizes:
        sizes = [int(s) for s in args.sizes.split(",")]
    else:
        smooth = 64424509440  # 2^32 * 3 * 5 (divisors.rs:7): no factor 17, 257, 65537
        sizes = [d for d in gl.divisors() if 2 <= d <= (1 << args.max_exponent)
                 and (args.all or smooth % d == 0)]
    stream = torch.cuda.current_stream()
    print("size,cols,duration,throughput")
    for n in sizes:
        x = gl.fill_uniform(n * args.cols, seed=n)
        d = torch.from_numpy(x.view(np.int64)).cuda()
        out = None
        if args.lde:
            out = torch.empty(n * args.cols * args.lde, dtype=torch.int64, device="cuda")

        tree = None
        if args.algo == "merkle":
            tree = torch.empty(max(lib.gl_merkle_tree_bytes(n * args.cols * 8), 1), dtype=torch.uint8,
                               device="cuda")

        def run():
            if tree is not None:
                rc = lib.gl_merkle_tree(d.data_ptr(), n * args.cols * 8, tree.data_ptr(), tree.numel(),
                                        L.GL_MEM_DEVICE, stream.cuda_stream)
            elif args.lde:
                rc = lib.gl_coset_lde(d.data_ptr(), out.data_ptr(), n, args.cols, args.lde, 7,
                                      L.GL_MEM_DEVICE, stream.cuda_stream)
            elif args.cols > 1:
                rc = lib.gl_ntt_columns(d.data_ptr(), n, args.cols,
                                        L.GL_INVERSE if args.algo == "inverse" else L.GL_FORWARD,
                                        L.GL_MEM_DEVICE, stream.cuda_stream)
            else:
                pl = gl.strategy(n)
                (pl.intt if args.algo == "inverse" else pl.ntt)(d)
                rc = 0
            if rc:
                raise gl.GoldilocksError(rc, "cli")

        if args.tune and args.algo != "merkle":
            from . import tune
            tune.autotune(n, reps=max(args.reps, 3))
            tune.save(args.tune)
        try:
            for _ in range(args.warmup):
                run()
            times = []
            for _ in range(args.reps):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                run()
                b.record(stream)
                b.synchronize()
                times.append(a.elapsed_time(b) * 1e-3)
        except ValueError as e:
            print("%d,%d,unsupported,%s" % (n, args.cols, e), file=sys.stderr)
            continue
        t = statistics.median(times)
        print("%d,%d,%.9f,%.6e" % (n, args.cols, t, n * args.cols / t))
        sys.stdout.flush()
    return 0


def _run_batch(args, gl, torch, np):
    """Batches of uneven lengths (gl_batch_execute): one line with the batch
    time and elements/s.  Odd-indexed polynomials are inverse transforms."""
    from . import batch as B
    rng = np.random.default_rng(0xBA7C)
    sizes = [1 << int(k) for k in rng.integers(12, 19, args.batch)]
    pool = torch.from_numpy(gl.fill_uniform(sum(sizes), seed=0xBA7C).view(np.int64)).cuda()
    items, off = [], 0
    for i, n in enumerate(sizes):
        items.append((pool[off:off + n], B.INVERSE if i % 2 else B.FORWARD))
        off += n
    mode = {"auto": B.AUTO, "persistent": B.PERSISTENT, "buckets": B.BUCKETS, "per_call": B.PER_CALL}[args.batch_mode]
    stream = torch.cuda.current_stream()
    offs = np.cumsum([0] + sizes[:-1])
    dirs = [i % 2 for i in range(len(sizes))]

    def run():
        if args.batch_api == "packed":
            B.run_packed(pool, offs, sizes, dirs, mode=mode)
        else:
            B.run(items, mode=mode)
    for _ in range(args.warmup):
        run()
    times = []
    for _ in range(args.reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        run()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b) * 1e-3)
    t = statistics.median(times)
    print("polys,mode,api,elements,duration,throughput")
    print("%d,%s,%s,%d,%.9f,%.6e" % (len(sizes), args.batch_mode, args.batch_api, sum(sizes), t, sum(sizes) / t))
    return 0


if __name__ == "__main__":
    sys.exit(main())
