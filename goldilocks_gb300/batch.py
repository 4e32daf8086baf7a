"""Batches of polynomials of uneven lengths on the GPU (gl_batch_execute).

    import goldilocks_gb300.batch as B
    B.run([(t1, B.FORWARD), (t2, B.INVERSE), ...], mode=B.PERSISTENT)

Each entry is a contiguous CUDA int64/uint64 tensor transformed in place (its
length must divide p - 1).  Modes: PERSISTENT (one launch, device work queue),
BUCKETS (per-size launches replayed from a CUDA graph), PER_CALL (one call per
polynomial), AUTO (the mode `autotune` measured fastest for this batch shape,
else BUCKETS).  `run_packed` takes the polynomials as (offset, length,
direction) arrays over one pool tensor.
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


# numpy view of gl_poly (include/goldilocks_gpu.h): data, len, dir, reserved.
POLY_DTYPE = None


def _poly_dtype():
    global POLY_DTYPE
    if POLY_DTYPE is None:
        import numpy as np
        POLY_DTYPE = np.dtype([("data", np.uint64), ("len", np.uint64), ("dir", np.int32),
                               ("reserved", np.int32)])
        assert POLY_DTYPE.itemsize == ctypes.sizeof(L.Poly)
    return POLY_DTYPE


def run_packed(pool, offsets, lengths, dirs, mode=AUTO):
    """The same as `run` for polynomials stored in one contiguous CUDA tensor:
    polynomial i is pool[offsets[i] : offsets[i] + lengths[i]], transformed in
    the direction dirs[i] (FORWARD / INVERSE).  The descriptor array is built
    with numpy in one step instead of one Python call per polynomial, so a
    batch of 1024 polynomials costs microseconds on the host instead of about
    half a millisecond."""
    import numpy as np
    import torch
    if not isinstance(pool, torch.Tensor) or not pool.is_cuda or pool.element_size() != 8:
        raise TypeError("pool must be a 64-bit integer CUDA tensor")
    if not pool.is_contiguous():
        raise ValueError("pool must be contiguous")
    offsets = np.asarray(offsets, dtype=np.int64)
    lengths = np.asarray(lengths, dtype=np.int64)
    dirs = np.asarray(dirs, dtype=np.int32)
    if not (offsets.shape == lengths.shape == dirs.shape) or offsets.ndim != 1:
        raise ValueError("offsets, lengths and dirs must be 1-D arrays of one length")
    if offsets.size == 0:
        return
    if (offsets < 0).any() or (lengths < 0).any() or (offsets + lengths > pool.numel()).any():
        raise ValueError("a polynomial lies outside the pool")
    arr = np.zeros(offsets.size, dtype=_poly_dtype())
    arr["data"] = np.uint64(pool.data_ptr()) + offsets.astype(np.uint64) * np.uint64(8)
    arr["len"] = lengths
    arr["dir"] = dirs
    stream = torch.cuda.current_stream(pool.device).cuda_stream
    st = L.load().gl_batch_execute(arr.ctypes.data, offsets.size, int(mode), stream)
    if st == L.GL_ERR_UNSUPPORTED_SIZE:
        bad = next((int(n) for n in lengths if not L.load().gl_is_divisor(int(n))), 0)
        _check(st, "batch", size=bad)
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
