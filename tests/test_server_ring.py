"""Host logic of the serving load generator's output ring (no GPU)."""
import types

import numpy as np

from goldilocks_gb300 import server as S


def _fake_torch():
    return types.SimpleNamespace(int64=np.int64, empty=lambda n, dtype=None, device=None: np.zeros(n, dtype))


def test_ring_never_hands_out_a_live_region():
    rng = np.random.default_rng(3)
    ring = S._Ring(_fake_torch(), 1000)
    waited, next_rid = [], 0
    live = {}

    def wait(rid):
        waited.append(rid)
        live.pop(rid)

    for _ in range(2000):
        w = int(rng.integers(1, 400))
        buf, lo, hi = ring.take(w, wait)
        assert hi - lo == w and len(buf) == w and 0 <= lo < hi <= 1000
        for a, b in live.values():  # disjoint from every region still in flight
            assert hi <= a or b <= lo
        live[next_rid] = (lo, hi)
        ring.live.append((next_rid, lo, hi))
        next_rid += 1
    # Requests are waited for oldest first.
    assert waited == sorted(waited)


def test_ring_rejects_oversized_outputs():
    ring = S._Ring(_fake_torch(), 100)
    try:
        ring.take(101, lambda rid: None)
    except ValueError:
        pass
    else:
        raise AssertionError("expected ValueError")

