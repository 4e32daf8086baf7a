"""GPU: the continuous-batching server.  Each result is the same when the
request runs alone (plain API) and when it runs in the mix with others;
admission control, rejection, cancellation and bounded waits behave."""
import numpy as np
import pytest

from conftest import from_dev, to_dev

pytestmark = pytest.mark.gpu


def test_mixed_stream_matches_requests_run_alone(gl, cuda):
    from goldilocks_gb300 import server as S
    reqs = S.make_requests(60, seed=7, log_min=6, log_max=16, max_cols=8)
    pool = to_dev(cuda, gl.fill_uniform(max(n * c for _, n, c, _ in reqs), seed=11))
    arrivals = S.poisson_arrivals(len(reqs), rate_per_s=2000.0, seed=7)
    _, stats, _, mixed = S.serve_stream(reqs, arrivals, pool, budget_bytes=1 << 26, slots=3,
                                        max_batch=16)
    _, _, _, alone = S.serial_baseline(reqs, pool)
    for r, a, b in zip(reqs, mixed, alone):
        assert np.array_equal(from_dev(a), from_dev(b)), r
    assert stats["completed"] == len(reqs) and stats["batches"] >= 1
    assert stats["max_in_use_bytes"] <= 1 << 26


def test_lde_request_matches_oracle(gl, oracle, cuda):
    from goldilocks_gb300 import server as S
    n, cols = 1024, 3
    x = gl.fill_uniform(n * cols, seed=3)
    inp = to_dev(cuda, x)
    out = cuda.empty(4 * n * cols, dtype=cuda.int64, device="cuda")
    with S.Server(budget_bytes=1 << 30, slots=2, max_batch=4) as srv:
        rid = srv.submit(S.GL_OP_LDE, n, cols, inp, out, blowup=4, shift=7)
        assert srv.wait(rid) == gl._lib.GL_OK
    assert np.array_equal(from_dev(out), oracle.coset_lde(x, n, cols, 4, 7))


def test_rejections_cancellation_and_bounded_wait(gl, cuda):
    from goldilocks_gb300 import server as S
    L = gl._lib
    buf = cuda.zeros(1 << 16, dtype=cuda.int64, device="cuda")
    with S.Server(budget_bytes=1 << 20, slots=1, max_batch=1) as srv:
        with pytest.raises(gl.GoldilocksError) as e:   # needs more than the whole budget
            srv.submit(S.GL_OP_NTT, 1 << 18, 1, buf, buf)
        assert e.value.status == L.GL_ERR_BUDGET
        with pytest.raises(gl.GoldilocksError) as e:   # not a divisor of p - 1
            srv.submit(S.GL_OP_NTT, 7, 1, buf, buf)
        assert e.value.status == L.GL_ERR_UNSUPPORTED_SIZE
        # A queue behind a busy slot: the later request can be cancelled.
        ids = [srv.submit(S.GL_OP_NTT, 4096, 8, buf, buf) for _ in range(6)]
        cancelled = [rid for rid in ids[1:] if srv.cancel(rid) == L.GL_OK]
        for rid in ids:
            st = srv.wait(rid, timeout_ms=60000)
            assert st == (L.GL_ERR_CANCELLED if rid in cancelled else L.GL_OK)
        with pytest.raises(gl.GoldilocksError) as e:
            srv.wait(123456789)
        assert e.value.status == L.GL_ERR_NOT_FOUND
        assert srv.stats()["rejected"] == 2


def test_ring_outputs_and_full_mix_entry_point(gl, cuda, capsys):
    """Outputs carved from a ring equal outputs in their own buffers: with a
    ring that holds every output all of them are compared; with a ring of
    three outputs (so that the submitter waits for older requests) the last
    output is.  The full-mix entry point runs end to end on a small case."""
    import json
    from goldilocks_gb300 import server as S
    reqs = S.make_requests(40, seed=21, log_min=6, log_max=14, max_cols=8)
    pool = to_dev(cuda, gl.fill_uniform(max(n * c for _, n, c, _ in reqs), seed=4))
    _, _, _, alone = S.serial_baseline(reqs, pool)
    arrivals = S.poisson_arrivals(len(reqs), rate_per_s=5000.0, seed=21)
    total = sum(S._out_words(*r) for r in reqs)
    # (All of these requests are small: they share the small-request ring,
    # half of a ring this short.)
    for ring_words, check in ((2 * total, range(len(reqs))), (6 * max(S._out_words(*r) for r in reqs), [-1])):
        rate, stats, _, outs = S.serve_stream(reqs, arrivals, pool, budget_bytes=1 << 26, slots=2,
                                              max_batch=8, ring_words=ring_words)
        assert rate > 0 and stats["completed"] == len(reqs)
        for k in check:
            assert np.array_equal(from_dev(outs[k]), from_dev(alone[k])), (ring_words, k, reqs[k])
    _, _, _, none = S.serial_baseline(reqs, pool, ring_words=total)
    assert none is None
    S.main(["--requests", "30", "--log-max", "12", "--max-cols", "4", "--ring-gib", "1", "--check", "8",
            "--check-gib", "1"])
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["requests"] == 30 and len(line["loads"]) == 4
    assert line["checked"] == 4 * 8 and line["mismatches"] == []


def test_full_size_mix_matches_requests_run_alone(gl, cuda):
    """Requests at the configured serving sizes -- up to 2^24 rows and 64
    columns, LDE included -- submitted together so that they overlap on the
    GPU (large ones on the low-priority slots, small ones on the
    high-priority one), each output equal to the plain per-call result."""
    from goldilocks_gb300 import server as S
    cuda.cuda.empty_cache()
    big = [(S.GL_OP_LDE, 1 << 24, 64, 4), (S.GL_OP_NTT, 1 << 24, 64, 4), (S.GL_OP_INTT, 1 << 24, 33, 4),
           (S.GL_OP_LDE, 1 << 22, 17, 4), (S.GL_OP_NTT, 1 << 24, 1, 4), (S.GL_OP_INTT, 1 << 23, 1, 4),
           (S.GL_OP_LDE, 1 << 24, 1, 4), (S.GL_OP_INTT, 1 << 20, 64, 4)]
    small = S.make_requests(28, seed=0xF5, log_min=10, log_max=18, max_cols=64)
    reqs = [r for pair in zip(small[:len(big)], big) for r in pair] + small[len(big):]
    pool = to_dev(cuda, gl.fill_uniform(max(n * c for _, n, c, _ in reqs), seed=0xF5))
    arrivals = np.zeros(len(reqs))  # all at once: maximal overlap
    _, stats, _, outs = S.serve_stream(reqs, arrivals, pool, budget_bytes=64 << 30, slots=4, max_batch=16)
    assert stats["completed"] == len(reqs)
    bad = S.check_outputs(reqs, pool, outs, range(len(reqs)))
    assert bad == [], [reqs[k] for k in bad]
    del outs, pool
    cuda.cuda.empty_cache()


def test_new_length_does_not_wait_for_a_busy_slot(gl, oracle, cuda):
    """The first request of a length never used before builds its twiddle
    tables on the library's table stream (no device-wide synchronisation),
    its kernels were loaded when the server was created, and its scratch
    comes from a pool that never waits for another stream's free: so it
    completes while a long request on another slot is still running."""
    from goldilocks_gb300 import server as S
    L = gl._lib
    big_n, big_cols = 1 << 24, 64
    pool = to_dev(cuda, gl.fill_uniform(big_n * big_cols, seed=0xB16))
    big_out = cuda.empty(4 * big_n * big_cols, dtype=cuda.int64, device="cuda")
    n = 85 * 2 ** 13  # 696320: a length no other test plans
    x = gl.fill_uniform(n, seed=0x5A11)
    inp, out = to_dev(cuda, x), cuda.empty(n, dtype=cuda.int64, device="cuda")
    with S.Server(budget_bytes=64 << 30, slots=2, max_batch=4) as srv:
        big = srv.submit(S.GL_OP_LDE, big_n, big_cols, pool, big_out, blowup=4)
        small = srv.submit(S.GL_OP_NTT, n, 1, inp, out)
        assert srv.wait(small, timeout_ms=60000) == L.GL_OK
        still_running = srv.poll(big) == L.GL_ERR_BUSY
        assert srv.wait(big, timeout_ms=120000) == L.GL_OK
    assert still_running
    assert np.array_equal(from_dev(out), oracle.ntt(x))
    del pool, big_out
    cuda.cuda.empty_cache()
