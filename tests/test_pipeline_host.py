"""Host-side validation of gl_host_pipeline (no GPU): invalid jobs are
rejected before anything is queued."""
import ctypes

import numpy as np
import pytest


def test_python_wrapper_checks(gl):
    x = np.zeros(64, dtype=np.uint64)
    with pytest.raises(TypeError):
        gl.host_pipeline([(x.astype(np.int64), 64, ("fwd",))])
    with pytest.raises(TypeError):
        gl.host_pipeline([(x[::2], 32, ("fwd",))])
    with pytest.raises(ValueError):
        gl.host_pipeline([(x, 48, ("fwd",))])          # 64 is not a multiple of 48
    with pytest.raises(ValueError):
        gl.host_pipeline([(x, 64, ("fwd",) * 5)])      # more transforms than a job holds


def test_unsupported_size_is_rejected_before_any_copy(gl):
    x = np.arange(14, dtype=np.uint64)
    with pytest.raises(ValueError, match="not a supported NTT size"):
        gl.host_pipeline([(x, 7, ("fwd",))])
    assert np.array_equal(x, np.arange(14, dtype=np.uint64))


def test_c_abi_rejects_bad_jobs(gl):
    L = gl._lib
    lib = L.load()
    x = np.zeros(16, dtype=np.uint64)
    job = L.HostJob()
    job.data, job.len, job.count, job.nops = x.ctypes.data, 16, 1, 1
    job.dirs[0] = 5                                      # neither GL_FORWARD nor GL_INVERSE
    assert lib.gl_host_pipeline(ctypes.addressof(job), 1, 0) == L.GL_ERR_INVALID
    job.dirs[0] = L.GL_FORWARD
    job.nops = L.GL_HOST_JOB_MAX_OPS + 1
    assert lib.gl_host_pipeline(ctypes.addressof(job), 1, 0) == L.GL_ERR_INVALID
    job.nops, job.data = 1, None                         # null data with elements
    assert lib.gl_host_pipeline(ctypes.addressof(job), 1, 0) == L.GL_ERR_INVALID
    assert lib.gl_host_pipeline(None, 1, 0) == L.GL_ERR_INVALID
    assert lib.gl_host_pipeline(None, 0, 0) == L.GL_OK  # nothing to do


def test_submit_rejects_bad_jobs_without_a_ticket(gl):
    L = gl._lib
    lib = L.load()
    x = np.zeros(16, dtype=np.uint64)
    job = L.HostJob()
    job.data, job.len, job.count, job.nops = x.ctypes.data, 16, 1, 1
    job.dirs[0] = 5
    t = ctypes.c_void_p(1234)
    assert lib.gl_host_pipeline_submit(ctypes.addressof(job), 1, 0, ctypes.byref(t)) == L.GL_ERR_INVALID
    assert t.value is None                               # no ticket for a refused call
    job.dirs[0] = L.GL_FORWARD
    assert lib.gl_host_pipeline_submit(ctypes.addressof(job), 1, 0, None) == L.GL_ERR_INVALID
    assert lib.gl_host_pipeline_wait(None) == L.GL_ERR_INVALID
    # nothing to do: a ticket that is already complete
    assert lib.gl_host_pipeline_submit(None, 0, 0, ctypes.byref(t)) == L.GL_OK and t.value
    assert lib.gl_host_pipeline_wait(t) == L.GL_OK
    with pytest.raises(ValueError, match="not a supported NTT size"):
        gl.host_pipeline_submit([(np.arange(14, dtype=np.uint64), 7, ("fwd",))])
    tk = gl.host_pipeline_submit([])
    assert tk.wait() == []
    with pytest.raises(RuntimeError, match="already waited"):
        tk.wait()
