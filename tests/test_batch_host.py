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
