"""GPU: gl_host_pipeline (host buffers, one round trip each, copies
overlapped) gives the same words as the per-call transforms."""
import numpy as np
import pytest

from conftest import rand_field

pytestmark = pytest.mark.gpu


def pinned(cuda, x):
    t = cuda.empty(x.size, dtype=cuda.int64, pin_memory=True)
    h = t.numpy().view(np.uint64)
    h[:] = x
    return h


@pytest.mark.parametrize("depth", [0, 1, 2, 5])
def test_pipeline_matches_oracle(gl, oracle, cuda, depth):
    specs = [(1 << 20, 1, ("fwd",)), (4096, 7, ("fwd", "inv")), (1 << 16, 2, ("inv",)),
             (257 * 16, 3, ("fwd",)), (16711680, 1, ("fwd", "inv", "fwd")), (3 << 10, 5, ("inv", "fwd"))]
    xs, jobs = [], []
    for i, (n, count, dirs) in enumerate(specs):
        x = rand_field(n * count, seed=i + 10 * depth)
        xs.append(x)
        h = pinned(cuda, x) if i % 2 == 0 else x.copy()   # page-locked and pageable buffers
        jobs.append((h, n, dirs))
    gl.host_pipeline(jobs, depth=depth)
    for (h, n, dirs), x in zip(jobs, xs):
        want = x
        for d in dirs:
            want = (oracle.ntt if d == "fwd" else oracle.intt)(want, size=n)
        assert np.array_equal(h, want), (n, dirs)


def test_pipeline_column_blocks(gl, oracle, cuda):
    """Large two-pass transforms move in column blocks (2D copies) around the
    first column pass and the last row pass; 4080 columns split into blocks
    of 510, not a multiple of the kernel's lanes."""
    specs = [(1 << 22, ("fwd", "inv")), (3 << 20, ("fwd",)), (16711680, ("inv",)), (1 << 24, ("fwd", "inv", "fwd"))]
    xs, jobs = [], []
    for i, (n, dirs) in enumerate(specs):
        x = gl.fill_uniform(n, seed=0xB10C + i)
        xs.append(x)
        jobs.append((pinned(cuda, x) if i != 1 else x.copy(), n, dirs))
    gl.host_pipeline(jobs)
    for (h, n, dirs), x in zip(jobs, xs):
        want = x
        for d in dirs:
            want = (oracle.ntt if d == "fwd" else oracle.intt)(want)
        assert np.array_equal(h, want), (n, dirs)


def test_pipeline_errors(gl, cuda):
    x = rand_field(16, seed=1)
    with pytest.raises(ValueError, match="is not a supported NTT size"):
        gl.host_pipeline([(x[:7].copy(), 7, ("fwd",))])
    with pytest.raises(ValueError, match="at most"):
        gl.host_pipeline([(x, 16, ("fwd",) * 5)])
    gl.host_pipeline([])


def test_submitted_calls_overlap_and_match_oracle(gl, oracle, cuda):
    """Three host_pipeline_submit calls in flight at once (the later ones'
    copy-ins run beside the earlier ones' passes and copy-outs), each on its
    own buffers, waited on out of order."""
    calls = [[(1 << 22, ("fwd", "inv")), (1 << 16, ("fwd",))],
             [(16711680, ("fwd",)), (4096 * 3, ("inv",))],
             [(1 << 20, ("inv", "fwd")), (1 << 22, ("fwd",))]]
    xs, tickets, jobs_of = [], [], []
    for c, specs in enumerate(calls):
        jobs = []
        for i, (n, dirs) in enumerate(specs):
            x = gl.fill_uniform(n, seed=0x5B + 10 * c + i)
            xs.append((x, n, dirs))
            jobs.append((pinned(cuda, x), n, dirs))
        jobs_of.append(jobs)
        tickets.append(gl.host_pipeline_submit(jobs))
    outs = [None] * len(tickets)
    for c in (1, 0, 2):
        outs[c] = tickets[c].wait()
    got = [h for o in outs for h in o]
    for h, (x, n, dirs) in zip(got, xs):
        want = x
        for d in dirs:
            want = (oracle.ntt if d == "fwd" else oracle.intt)(want)
        assert np.array_equal(h, want), (n, dirs)
