"""Batches of polynomials of uneven lengths on the GPU (gl_batch_execute).

    import goldilocks_gb300.batch as B
    B.run([(t1, B.FORWARD), (t2, B.INVERSE), ...], mode=B.PERSISTENT)

Each entry is a contiguous CUDA int64/uint64 tensor transformed in place (its
length must divide p - 1).  Modes: PERSISTENT (one launch, device work queue),
BUCKETS (per-size launches replayed from a CUDA graph), PER_CALL (one call per
polynomial), AUTO (the mode `autotune` measured fastest for this batch shape,
else BUCKETS).
"""
import ctypes

from . import _lib as L
from .ntt import GoldilocksError, _check

FORWARD, INVERSE = L.GL_FORWARD, L.GL_INVERSE
AUTO, PERSISTENT, BUCKETS, PER_CALL = (L.GL_BATCH_AUTO, L.GL_BATCH_PERSISTENT, L.GL_BATCH_BUCKETS,
                                       L.GL_BATCH_PER_CALL)


def _polys(items):
    import torch
    arr = (L.Poly * len(items))()
    dev = items[0][0].device if isinstance(items[0][0], torch.Tensor) else None
    for i, (t, d) in enumerate(items):
        if not isinstance(t, torch.Tensor) or t.device != dev or not t.is_cuda or t.element_size() != 8:
            raise TypeError("batch entries must be 64-bit integer tensors on one CUDA device")
        if not t.is_contiguous():
            raise ValueError("batch entries must be contiguous")
        p = arr[i]
        p.data = t.data_ptr()
        p.len = t.numel()
        p.dir = d
    return arr, torch.cuda.current_stream(dev).cuda_stream


def run(items, mode=AUTO):
    """Transform every (tensor, direction) entry in place; returns when done."""
    if not items:
        return
    arr, stream = _polys(items)
    st = L.load().gl_batch_execute(ctypes.addressof(arr), len(items), int(mode), stream)
    if st == L.GL_ERR_UNSUPPORTED_SIZE:
        _check(st, "batch", size=next((t.numel() for t, _ in items), 0))
    if st != L.GL_OK:
        raise GoldilocksError(st, "batch")


def autotune(items, reps=3):
    """Time PERSISTENT, BUCKETS and PER_CALL on this batch (transforming it
    1 + reps times per mode), remember the fastest for AUTO; returns
    {mode name: mean ms}."""
    arr, stream = _polys(items)
    ms = (ctypes.c_double * 3)()
    st = L.load().gl_batch_autotune(ctypes.addressof(arr), len(items), reps, stream, ms)
    if st != L.GL_OK:
        raise GoldilocksError(st, "batch autotune")
    return {"persistent": ms[0], "buckets": ms[1], "per_call": ms[2]}
