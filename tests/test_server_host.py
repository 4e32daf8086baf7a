"""Host-side logic of the request server (no GPU): the admission footprint
of a request (gl_server_request_bytes) and its validation."""
import pytest


def test_footprint_of_transforms_and_lde(gl):
    from goldilocks_gb300 import server as S
    n, cols = 1 << 20, 8
    # a two-pass transform needs one scratch buffer of n * cols words
    assert S.request_bytes(S.GL_OP_NTT, n, cols) == n * cols * 8
    assert S.request_bytes(S.GL_OP_INTT, n, cols) == n * cols * 8
    # a single-pass transform needs none
    assert S.request_bytes(S.GL_OP_NTT, 2048, cols) == 0
    # LDE: the coefficients plus scratch; from 2^16 coefficients one length-n
    # transform per coset (scratch n x cols), below that one zero-padded
    # transform of length 4n (scratch 4n x cols)
    assert S.request_bytes(S.GL_OP_LDE, n, cols, blowup=4) == (n * cols + n * cols) * 8
    m = 1 << 14
    assert S.request_bytes(S.GL_OP_LDE, m, cols, blowup=4) == (m * cols + 4 * m * cols) * 8


def test_invalid_requests(gl):
    from goldilocks_gb300 import server as S
    from goldilocks_gb300.ntt import GoldilocksError
    L = gl._lib
    cases = [((S.GL_OP_NTT, 1 << 10, 0), L.GL_ERR_INVALID),          # no columns
             ((7, 1 << 10, 1), L.GL_ERR_INVALID),                    # unknown operation
             ((S.GL_OP_LDE, 1 << 10, 1, 0), L.GL_ERR_INVALID),       # blowup 0
             ((S.GL_OP_NTT, 7, 1), L.GL_ERR_UNSUPPORTED_SIZE),       # 7 does not divide p - 1
             ((S.GL_OP_LDE, 1 << 10, 1, 7), L.GL_ERR_UNSUPPORTED_SIZE)]  # 7 * 2^10 does not either
    for args, want in cases:
        with pytest.raises(GoldilocksError) as e:
            S.request_bytes(*args)
        assert e.value.status == want, args


def test_serial_fifo_queue_model():
    """The serial path under given arrivals is a single FIFO server: each
    request starts at max(its arrival, the previous finish)."""
    from goldilocks_gb300 import server as S
    arrivals = [0.0, 0.001, 0.010, 0.0105]          # seconds
    service_ms = [5.0, 2.0, 1.0, 3.0]
    pct, wall = S.serial_fifo(service_ms, arrivals)
    # finishes: 5 ms, 7 ms, 11 ms, 14 ms -> latencies 5, 6, 1, 3.5 ms
    assert [round(x, 6) for x in pct["latency_ms"]] == [5.0, 6.0, 1.0, 3.5]
    assert abs(wall - 0.014) < 1e-12
    assert pct["max_ms"] == 6.0


def test_check_sample_covers_each_operation_within_its_memory():
    from goldilocks_gb300 import server as S
    reqs = S.make_requests(2000, seed=0x5E77)
    cap = (8 << 30) // 8
    ks = S.check_sample(reqs, 40, seed=3, max_words=cap)
    assert 0 < len(ks) <= 40 and len(set(ks)) == len(ks)
    assert sum(S._out_words(*reqs[k]) for k in ks) <= cap
    for op in (S.GL_OP_LDE, S.GL_OP_NTT, S.GL_OP_INTT):
        fitting = [S._out_words(*r) for r in reqs if r[0] == op and S._out_words(*r) <= cap // 4]
        assert max(S._out_words(*reqs[k]) for k in ks if reqs[k][0] == op) == max(fitting)


def test_request_classes_match_the_server():
    """The load generator's small class is the server's: at most 2^21 output
    words (LDE outputs count blowup times the rows)."""
    from goldilocks_gb300 import server as S
    assert S._is_small((S.GL_OP_NTT, 1 << 15, 64, 4))          # 2^21 words
    assert not S._is_small((S.GL_OP_NTT, 1 << 16, 64, 4))
    assert S._is_small((S.GL_OP_LDE, 1 << 13, 64, 4))          # 4 * 2^19
    assert not S._is_small((S.GL_OP_LDE, 1 << 14, 64, 4))
    src = open(__import__("os").path.join(S.__file__.rsplit("/", 1)[0], "csrc", "gl_server.cu")).read()
    assert "kSmallWords = 1ull << 21" in src
