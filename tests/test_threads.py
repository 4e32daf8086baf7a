"""Thread safety (the header: every function is thread-safe; plans are cached
under a mutex and shared, ntt/src/ntt/mod.rs:23).  CPU: concurrent plan
creation, including Rader lengths whose plans create sub-plans, with the cache
cleared meanwhile.  GPU: transforms from several host threads on their own
streams at once."""
import ctypes
import threading

import numpy as np
import pytest

from conftest import from_dev, rand_field, to_dev


def test_concurrent_plan_creation(gl):
    L = gl._lib
    lib = L.load()
    sizes = [n for n in gl.divisors() if 2 <= n <= 1 << 30][::3]
    assert any(n % 257 == 0 for n in sizes) and any(n % 65537 == 0 for n in sizes)
    errors, handles = [], {}
    lock = threading.Lock()

    def worker(seed):
        rng = np.random.default_rng(seed)
        for n in rng.permutation(sizes)[:200]:
            h = ctypes.c_void_p()
            st = lib.gl_plan_create(int(n), ctypes.byref(h))
            if st != L.GL_OK or lib.gl_plan_len(h) != n:
                errors.append((int(n), st))
            with lock:
                handles.setdefault(int(n), set()).add(h.value)

    def clearer():
        for _ in range(20):
            lib.gl_clear_cache()

    threads = [threading.Thread(target=worker, args=(s,)) for s in range(8)] + [threading.Thread(target=clearer)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors
    # without a concurrent clear, one size maps to one shared plan
    h1, h2 = ctypes.c_void_p(), ctypes.c_void_p()
    lib.gl_plan_create(4096, ctypes.byref(h1))
    lib.gl_plan_create(4096, ctypes.byref(h2))
    assert h1.value == h2.value


@pytest.mark.gpu
def test_concurrent_transforms_on_streams(gl, oracle, cuda):
    sizes = [1 << 12, 1 << 16, 3 << 14, 257 * 16, 1 << 20, 17 << 12]
    inputs = [rand_field(n, seed=n) for n in sizes]
    wants = [oracle.ntt(x) for x in inputs]
    failures = []

    def worker(k):
        torch = cuda
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            for rep in range(10):
                i = (k + rep) % len(sizes)
                d = to_dev(torch, inputs[i])
                gl.ntt(d)
                gl.intt(d)
                gl.ntt(d)
                s.synchronize()
                if not np.array_equal(from_dev(d), wants[i]):
                    failures.append((k, sizes[i]))

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not failures
