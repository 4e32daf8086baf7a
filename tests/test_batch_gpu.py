"""GPU parity of batched transforms of uneven lengths: every mode against the
oracle per polynomial, and the modes against each other at the configured
batch shape (1024 polynomials, log2 n uniform in [12, 18], half inverse)."""
import numpy as np
import pytest

from conftest import from_dev, rand_field, to_dev

pytestmark = pytest.mark.gpu


def make_batch(cuda, sizes, seed):
    xs, items = [], []
    for i, n in enumerate(sizes):
        x = rand_field(n, seed=seed * 1000 + i)
        xs.append(x)
        items.append((to_dev(cuda, x), i % 2))
    return xs, items


@pytest.mark.parametrize("mode_name", ["PERSISTENT", "BUCKETS", "PER_CALL", "AUTO"])
def test_modes_match_oracle(gl, oracle, cuda, mode_name):
    from goldilocks_gb300 import batch as B
    sizes = [4096, 8192, 1 << 16, 64, 4096, 1 << 13, 1 << 18, 1 << 14, 16, 1 << 15, 8192, 2048]
    xs, items = make_batch(cuda, sizes, seed=3)
    B.run(items, mode=getattr(B, mode_name))
    for x, (d, direction) in zip(xs, items):
        want = oracle.intt(x) if direction else oracle.ntt(x)
        assert np.array_equal(from_dev(d), want), (len(x), direction)


def test_persistent_matches_per_call_config_shape(gl, oracle, cuda):
    """1024 polynomials, log2 n ~ U[12, 18], odd index inverse: persistent and
    bucketed results are bit-identical to per-call results, and a seeded
    sample of 48 polynomials (with the longest of each direction) equals the
    oracle in every mode."""
    from goldilocks_gb300 import batch as B
    rng = np.random.default_rng(2024)
    sizes = [1 << int(k) for k in rng.integers(12, 19, 1024)]
    outs = {}
    for mode in (B.PER_CALL, B.PERSISTENT, B.BUCKETS):
        xs, items = make_batch(cuda, sizes, seed=5)
        B.run(items, mode=mode)
        outs[mode] = [from_dev(d) for d, _ in items]
    for a, b, c in zip(outs[B.PER_CALL], outs[B.PERSISTENT], outs[B.BUCKETS]):
        assert np.array_equal(a, b) and np.array_equal(a, c)
    longest = [max((i for i in range(len(sizes)) if i % 2 == d), key=lambda i: sizes[i]) for d in (0, 1)]
    sample = sorted(set(longest) | set(rng.choice(len(sizes), 46, replace=False).tolist()))
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=8) as ex:
        wants = list(ex.map(lambda i: oracle.intt(xs[i]) if i % 2 else oracle.ntt(xs[i]), sample))
    for i, want in zip(sample, wants):
        for mode in (B.PER_CALL, B.PERSISTENT, B.BUCKETS):
            assert np.array_equal(outs[mode][i], want), (mode, i, sizes[i])


def test_autotune_picks_a_mode(gl, cuda):
    from goldilocks_gb300 import batch as B
    sizes = [4096, 1 << 14, 1 << 16] * 8
    _, items = make_batch(cuda, sizes, seed=9)
    ms = B.autotune(items, reps=2)
    assert set(ms) == {"persistent", "buckets", "per_call"} and all(v > 0 for v in ms.values())
    _, items2 = make_batch(cuda, sizes, seed=9)
    B.run(items2, mode=B.AUTO)


def test_bounded_wait_reports_timeout_and_context_survives(gl, oracle, cuda):
    """A row item whose column pass never runs: the persistent kernel's wait
    gives up after the limit, reports GL_ERR_TIMEOUT, and the GPU context keeps
    working (no fault, no hang)."""
    import ctypes
    import time
    L = gl._lib
    st = ctypes.c_uint32(0)
    t0 = time.perf_counter()
    assert L.load().gl_batch_wait_selftest(50_000_000, ctypes.byref(st)) == L.GL_OK   # 50 ms
    elapsed = time.perf_counter() - t0
    assert st.value == L.GL_ERR_TIMEOUT
    assert 0.04 < elapsed < 5.0
    x = gl.fill_uniform(1 << 16, seed=9)
    d = cuda.tensor(x.view(np.int64), device="cuda")
    gl.ntt(d)
    assert np.array_equal(d.cpu().numpy().view(np.uint64), oracle.ntt(x))


def test_injected_allocation_failures_propagate(gl, cuda):
    """An allocation refused on the host side (injected) comes back as
    GL_ERR_OOM from every kind of call, leaves the data untouched, and the
    next call succeeds."""
    from goldilocks_gb300 import batch as B
    L = gl._lib
    lib = L.load()
    x = gl.fill_uniform(1 << 16, seed=4)
    d = cuda.tensor(x.view(np.int64), device="cuda")
    s = cuda.cuda.current_stream().cuda_stream
    try:
        lib.gl_debug_inject_alloc_failures(1)
        with pytest.raises(gl.GoldilocksError) as e:      # two-pass plan: scratch
            gl.ntt(d)
        assert e.value.status == L.GL_ERR_OOM
        assert np.array_equal(d.cpu().numpy().view(np.uint64), x)
        lib.gl_debug_inject_alloc_failures(1)
        h = x.copy()                                      # pageable host memory: staging
        with pytest.raises(gl.GoldilocksError) as e:
            gl.ntt(h)
        assert e.value.status == L.GL_ERR_OOM and np.array_equal(h, x)
        lib.gl_debug_inject_alloc_failures(1)
        assert lib.gl_ntt_columns(d.data_ptr(), 1 << 13, 8, L.GL_FORWARD, L.GL_MEM_DEVICE, s) == L.GL_ERR_OOM
        lib.gl_debug_inject_alloc_failures(1)
        with pytest.raises(gl.GoldilocksError) as e:
            B.run([(d, B.FORWARD)], mode=B.BUCKETS)
        assert e.value.status == L.GL_ERR_OOM
        assert np.array_equal(d.cpu().numpy().view(np.uint64), x)
    finally:
        lib.gl_debug_inject_alloc_failures(0)
    gl.ntt(d)                                             # and the library keeps working
    gl.intt(d)
    assert np.array_equal(d.cpu().numpy().view(np.uint64), x)


@pytest.mark.parametrize("mode_name", ["persistent", "buckets", "auto"])
def test_batch_with_three_pass_and_rader_lengths(gl, oracle, cuda, mode_name):
    """Lengths the persistent and bucket kernels have no shape for (three
    passes, Rader steps, run-time radices) run as plain calls inside the
    batch, in order with the rest."""
    from goldilocks_gb300 import batch as B
    mode = {"persistent": B.PERSISTENT, "buckets": B.BUCKETS, "auto": B.AUTO}[mode_name]
    sizes = [1 << 25, 4096, 257 * 16, 1 << 16, 3 << 10, 65537, 1 << 18]
    xs = [gl.fill_uniform(n, seed=i) for i, n in enumerate(sizes)]
    ds = [to_dev(cuda, x) for x in xs]
    dirs = [i % 2 for i in range(len(sizes))]
    B.run(list(zip(ds, dirs)), mode=mode)
    for x, d, inv in zip(xs, ds, dirs):
        assert np.array_equal(from_dev(d), (oracle.intt if inv else oracle.ntt)(x)), x.size


@pytest.mark.parametrize("mode_name", ["PERSISTENT", "BUCKETS", "PER_CALL", "AUTO"])
def test_packed_batches_match_oracle(gl, oracle, cuda, mode_name):
    """run_packed over one pool tensor, with gaps between the polynomials that
    must stay untouched, against the oracle per polynomial."""
    from goldilocks_gb300 import batch as B
    sizes = [4096, 8192, 1 << 16, 64, 3 << 12, 1 << 13, 1 << 18, 17 << 10, 16, 1 << 15]
    gap = 5
    offs, off = [], 0
    for n in sizes:
        offs.append(off)
        off += n + gap
    x = rand_field(off, seed=77)
    pool = to_dev(cuda, x)
    dirs = [i % 2 for i in range(len(sizes))]
    B.run_packed(pool, offs, sizes, dirs, mode=getattr(B, mode_name))
    y = from_dev(pool)
    for o, n, d in zip(offs, sizes, dirs):
        src = x[o:o + n]
        want = oracle.intt(src) if d else oracle.ntt(src)
        assert np.array_equal(y[o:o + n], want), (n, d)
        assert np.array_equal(y[o + n:o + n + gap], x[o + n:o + n + gap]), n


def test_packed_batch_argument_checks(gl, cuda):
    from goldilocks_gb300 import batch as B
    pool = cuda.zeros(100, dtype=cuda.int64, device="cuda")
    with pytest.raises(ValueError):
        B.run_packed(pool, [0, 64], [64, 64], [0, 1])          # past the end of the pool
    with pytest.raises(ValueError):
        B.run_packed(pool, [0], [64, 32], [0])                 # ragged arrays
    with pytest.raises(ValueError):
        B.run_packed(pool[::2], [0], [32], [0])                # not contiguous
    with pytest.raises(ValueError, match="not a supported NTT size"):
        B.run_packed(pool, [0], [7], [0])
    B.run_packed(pool, [], [], [])                             # empty: nothing to do
