"""Python mirror of the reference's `goldilocks_ntt::ntt` interface.

Reference (recmo/goldilocks, ntt crate):
  strategy(size) -> Arc<dyn Ntt> ......... ntt/src/ntt/mod.rs:48-78   -> strategy()/Plan
  Ntt::len / Ntt::ntt .................... ntt/src/ntt/mod.rs:25-31   -> Plan.len()/Plan.ntt()
  ntt(values) / intt(values) ............. ntt/src/ntt/mod.rs:98-120  -> ntt()/intt()
  clear_cache() .......................... ntt/src/ntt/mod.rs:43-46
  divisors / is_divisor / split / next ... ntt/src/divisors.rs:21-89

`values` is either a host numpy array of dtype uint64 (C-contiguous; the call
stages it through the GPU and returns when the result is back, like the
reference), or a CUDA torch tensor of dtype int64/uint64 (the work is queued on
the tensor's current stream).  Unsupported sizes raise ValueError with the
reference's panic message.
"""
import ctypes

import numpy as np

from . import _lib as L

MODULUS = 0xFFFF_FFFF_0000_0001


class GoldilocksError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = L.load().gl_status_string(status).decode()
        super().__init__("%s%s (status %d)" % (what + ": " if what else "", msg, status))


def _check(status, what="", size=None):
    if status == L.GL_OK:
        return
    if status == L.GL_ERR_UNSUPPORTED_SIZE and size is not None:
        raise ValueError("%d is not a supported NTT size (does not divide multiplicative order)" % size)
    raise GoldilocksError(status, what)


def _buffer(values):
    """(pointer, length, mem, stream) for a numpy array or CUDA tensor."""
    if isinstance(values, np.ndarray):
        if values.dtype != np.uint64:
            raise TypeError("host values must be a numpy uint64 array")
        if not values.flags.c_contiguous or not values.flags.writeable:
            raise ValueError("host values must be C-contiguous and writeable")
        return values.ctypes.data, values.size, L.GL_MEM_HOST, None
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    if torch is not None and isinstance(values, torch.Tensor):
        if not values.is_cuda:
            raise ValueError("torch tensors must live on a CUDA device (use numpy for host data)")
        if values.element_size() != 8 or values.dtype.is_floating_point:
            raise TypeError("device values must be a 64-bit integer tensor")
        if not values.is_contiguous():
            raise ValueError("device values must be contiguous")
        stream = torch.cuda.current_stream(values.device).cuda_stream
        return values.data_ptr(), values.numel(), L.GL_MEM_DEVICE, stream
    raise TypeError("values must be a numpy uint64 array or a CUDA torch tensor")


def is_divisor(n):
    return bool(L.load().gl_is_divisor(n))


def split(n):
    if not is_divisor(n):
        raise ValueError("%d does not divide multiplicative group order." % n)
    return int(L.load().gl_split(n))


def next(n):  # noqa: A001 -- the reference's name (divisors::next)
    return int(L.load().gl_next(n))


def divisors():
    buf = (ctypes.c_uint64 * 1056)()
    n = L.load().gl_divisors(buf, 1056)
    return [int(x) for x in buf[:n]]


class Plan:
    """A cached transform plan for one size (the reference's `Arc<dyn Ntt>`)."""

    def __init__(self, size):
        h = ctypes.c_void_p()
        _check(L.load().gl_plan_create(size, ctypes.byref(h)), "plan", size=size)
        self._h = h
        self.size = size

    def len(self):
        return int(L.load().gl_plan_len(self._h))

    def describe(self):
        buf = ctypes.create_string_buffer(1 << 16)
        L.load().gl_plan_describe(self._h, buf, len(buf))
        return buf.value.decode()

    def workspace_bytes(self, count=1):
        return int(L.load().gl_plan_workspace_bytes(self._h, count))

    def _run(self, values, direction):
        ptr, n, mem, stream = _buffer(values)
        if n % self.size:
            raise ValueError("length %d is not a multiple of the plan size %d" % (n, self.size))
        _check(L.load().gl_plan_execute(self._h, ptr, n, direction, mem, stream), "execute")
        return values

    def ntt(self, values):
        """Forward transforms of len(values)/size contiguous blocks, in place."""
        return self._run(values, L.GL_FORWARD)

    def intt(self, values):
        """Inverse transforms (1/n scaled) of contiguous blocks, in place."""
        return self._run(values, L.GL_INVERSE)


def strategy(size):
    return Plan(size)


def ntt(values):
    ptr, n, mem, stream = _buffer(values)
    _check(L.load().gl_ntt(ptr, n, mem, stream), "ntt", size=n)
    return values


def intt(values):
    ptr, n, mem, stream = _buffer(values)
    _check(L.load().gl_intt(ptr, n, mem, stream), "intt", size=n)
    return values


def convolve(a, b_hat, size=None, montgomery=True):
    """convolve::circular (ntt/src/convolve.rs:13-20): a <- intt(ntt(a) * b_hat)
    in place, for each length-`size` sequence of `a` (default: all of `a`).
    `b_hat` (already in NTT form) holds one sequence shared by all, or one per
    sequence.  `montgomery`: words are the reference's Field words (the
    product is a*b*2^-64); False: canonical values."""
    ptr, n, mem, stream = _buffer(a)
    bptr, bn, bmem, _ = _buffer(b_hat)
    if bmem != mem:
        raise ValueError("a and b_hat must both be host arrays or both device tensors")
    size = n if size is None else size
    if size == 0 or n % size:
        _check(L.GL_ERR_UNSUPPORTED_SIZE if size == 0 else L.GL_ERR_INVALID, "convolve", size=size)
    count = n // size
    if bn % size or bn // size not in (1, count):
        raise ValueError("b_hat must hold one sequence or one per sequence of a")
    repr_ = L.GL_REPR_MONTGOMERY if montgomery else L.GL_REPR_CANONICAL
    _check(L.load().gl_convolve(ptr, bptr, size, count, bn // size, repr_, mem, stream),
           "convolve", size=size)
    return a


def _host_jobs(jobs):
    """ctypes gl_host_job array for host_pipeline / host_pipeline_submit."""
    arr = (L.HostJob * max(len(jobs), 1))()
    for i, (a, size, dirs) in enumerate(jobs):
        if not isinstance(a, np.ndarray) or a.dtype != np.uint64 or not a.flags.c_contiguous:
            raise TypeError("jobs need C-contiguous numpy uint64 arrays")
        if size <= 0 or a.size % size:
            raise ValueError("array length is not a multiple of the transform size")
        if len(dirs) > L.GL_HOST_JOB_MAX_OPS:
            raise ValueError("at most %d transforms per job" % L.GL_HOST_JOB_MAX_OPS)
        arr[i].data = a.ctypes.data if a.size else None
        arr[i].len, arr[i].count, arr[i].nops = size, a.size // size, len(dirs)
        for k, d in enumerate(dirs):
            arr[i].dirs[k] = L.GL_INVERSE if d in ("inv", L.GL_INVERSE) else L.GL_FORWARD
    return arr


def _host_jobs_check(st, jobs, what):
    bad = [s for _, s, _ in jobs if not is_divisor(s)]
    _check(st, what, size=bad[0] if bad else None)


def host_pipeline(jobs, depth=0):
    """Transform host buffers with the copies overlapped: `jobs` is a list of
    (numpy uint64 array, size, [directions...]) -- each array holds
    len/size transforms and gets the listed transforms (ntt/intt by
    "fwd"/"inv") in order, in place, with one copy in and one copy out."""
    arr = _host_jobs(jobs)
    st = L.load().gl_host_pipeline(ctypes.addressof(arr), len(jobs), depth)
    _host_jobs_check(st, jobs, "host_pipeline")
    return [a for a, _, _ in jobs]


class PipelineTicket:
    """A host_pipeline call in flight (host_pipeline_submit).  wait() returns
    the arrays once they hold their results; until then they must not be
    read, written or freed (the ticket keeps them alive)."""

    def __init__(self, handle, arrays):
        self._h = handle
        self._arrays = arrays

    def wait(self):
        if self._h is None:
            raise RuntimeError("host pipeline ticket already waited on")
        h, self._h = self._h, None
        _check(L.load().gl_host_pipeline_wait(h), "host_pipeline_wait")
        return self._arrays

    def __del__(self):
        if getattr(self, "_h", None) is not None:
            L.load().gl_host_pipeline_wait(self._h)  # never leave copies into freed arrays


def host_pipeline_submit(jobs, depth=0):
    """host_pipeline without the wait: queues the jobs and returns a
    PipelineTicket.  Calls submitted back to back overlap (the next call's
    copy-ins run while this one computes and copies out); calls in flight
    must not share an array."""
    arr = _host_jobs(jobs)
    h = ctypes.c_void_p()
    st = L.load().gl_host_pipeline_submit(ctypes.addressof(arr), len(jobs), depth, ctypes.byref(h))
    _host_jobs_check(st, jobs, "host_pipeline_submit")
    return PipelineTicket(h.value, [a for a, _, _ in jobs])


def transpose(values, shape):
    """permute::transpose (ntt/src/permute/mod.rs:53-58): the row-major
    rows x cols matrix `values` transposed in place (it becomes cols x rows)."""
    rows, cols = shape
    ptr, n, mem, stream = _buffer(values)
    if n != rows * cols:
        raise ValueError("matrix of %d values is not %d x %d" % (n, rows, cols))
    _check(L.load().gl_transpose(ptr, rows, cols, mem, stream), "transpose")
    return values


def bit_reverse(values):
    """permute::bit_reverse (ntt/src/permute/mod.rs:70-74): values[i] and
    values[rev(i)] exchanged, for a power-of-two length."""
    ptr, n, mem, stream = _buffer(values)
    st = L.load().gl_bit_reverse(ptr, n, mem, stream)
    if st == L.GL_ERR_UNSUPPORTED_SIZE:
        raise ValueError("bit_reverse needs a power-of-two length, got %d" % n)
    _check(st, "bit_reverse")
    return values


def clear_cache():
    L.load().gl_clear_cache()


def fill_uniform(n, seed, offset=0):
    """Seeded field elements uniform in [0, p) (see gl_fill_uniform)."""
    out = np.empty(n, dtype=np.uint64)
    L.load().gl_fill_uniform(out.ctypes.data, n, seed, offset)
    return out
