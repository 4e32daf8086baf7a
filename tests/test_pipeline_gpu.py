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
            # one pageable buffer (its copies are staged, not overlapped)
            jobs.append((x.copy() if (c, i) == (1, 1) else pinned(cuda, x), n, dirs))
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


def test_stream_of_calls_reuses_device_blocks(gl, cuda):
    """Two calls in flight at a time, twenty calls: the pipeline reuses its
    device blocks once their last use has completed, so free device memory
    does not shrink after the first calls (a pool that does not reuse blocks
    freed on another stream grew by one block per call)."""
    n = 1 << 22
    xs = [gl.fill_uniform(n, seed=0x57 + s) for s in range(2)]
    sets = [pinned(cuda, x) for x in xs]

    def run(k):
        pend = None
        for i in range(k):
            t = gl.host_pipeline_submit([(sets[i % 2], n, ("fwd", "inv"))])
            if pend is not None:
                pend.wait()
            pend = t
        pend.wait()
    run(6)
    cuda.cuda.synchronize()
    free0 = cuda.cuda.mem_get_info()[0]
    run(20)
    cuda.cuda.synchronize()
    assert cuda.cuda.mem_get_info()[0] >= free0 - (16 << 20)
    for h, x in zip(sets, xs):
        assert np.array_equal(h, x)  # forward then inverse: the inputs again
