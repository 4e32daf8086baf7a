"""Host-side checks of the batch wrappers (no GPU)."""


def test_packed_batch_needs_a_cuda_tensor():
    import numpy as np
    import pytest
    import torch
    from goldilocks_gb300 import batch as B
    with pytest.raises(TypeError):
        B.run_packed(torch.zeros(8, dtype=torch.int64), [0], [8], [0])
    with pytest.raises(TypeError):
        B.run_packed(np.zeros(8, dtype=np.uint64), [0], [8], [0])


def test_c_abi_rejects_bad_batches(gl):
    import ctypes
    L = gl._lib
    lib = L.load()
    arr = (L.Poly * 2)()
    arr[0].data, arr[0].len, arr[0].dir = None, 1024, L.GL_FORWARD      # null data with elements
    arr[1].data, arr[1].len, arr[1].dir = 8, 1024, L.GL_FORWARD
    assert lib.gl_batch_execute(ctypes.addressof(arr), 2, L.GL_BATCH_BUCKETS, None) == L.GL_ERR_INVALID
    arr[0].data, arr[0].dir = 8, 5                                      # bad direction
    assert lib.gl_batch_execute(ctypes.addressof(arr), 2, L.GL_BATCH_BUCKETS, None) == L.GL_ERR_INVALID
    arr[0].dir = L.GL_FORWARD
    assert lib.gl_batch_execute(ctypes.addressof(arr), 2, 9, None) == L.GL_ERR_INVALID   # bad mode
    assert lib.gl_batch_execute(None, 3, L.GL_BATCH_AUTO, None) == L.GL_ERR_INVALID
    assert lib.gl_batch_execute(None, 0, L.GL_BATCH_AUTO, None) == L.GL_OK
