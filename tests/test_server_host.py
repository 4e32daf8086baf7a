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
    assert S.request_bytes(S.GL_OP_NTT, 4096, cols) == 0
    # LDE: the coefficients plus the scratch of the larger (blown-up) transform
    assert S.request_bytes(S.GL_OP_LDE, n, cols, blowup=4) == (n * cols + 4 * n * cols) * 8


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
