"""lm_transpose_100_noalloc: the no-allocation entry point.

For callers that cannot allocate device memory while they run (an allocator
converting layouts from inside its own allocation path, a real-time pipeline
that reserves all memory at start-up), the 100 transposition is also offered
with its done bits in a fixed 4 MiB device array.  This test calls it through
the C ABI twice in a row per shape and checks each result against
lm_transpose_100 (the regular entry point) bit for bit, and that a shape
larger than the array is refused without touching the buffer.
"""
import numpy as np
import pytest

from oracle import lm_oracle as O

pytestmark = pytest.mark.gpu


def test_no_alloc_matches_regular_entry_point(cuda):
    import torch
    from libmarshal_gb300 import lm
    lib = lm.lib()
    shapes = [(1000, 777, 1, 4), (512, 300, 32, 4), (64, 48, 3, 8),
              (97, 1031, 2, 2), (33, 65, 5000, 1), (4096, 2048, 1, 4)]
    for (A, B, b, e) in shapes:
        src = O.random_bits(A * B * b, e, A + B)
        raw = torch.from_numpy(src.view(np.uint8).copy())
        d_new = raw.to(cuda)
        d_ref = raw.to(cuda)
        for call in range(2):  # two calls in a row on the same buffers
            assert lib.lm_transpose_100_noalloc(
                None, d_new.data_ptr(), e, A, B, b) is False, lm.last_error()
            assert lib.lm_transpose_100(None, d_ref.data_ptr(), e, A, B, b,
                                        None) is False, lm.last_error()
            torch.cuda.synchronize()
            assert torch.equal(d_new, d_ref), (A, B, b, e, call)
    # beyond the array's capacity: refused, buffer unchanged
    A, B = 8192, 8192  # 67 M units > 33.5 M
    d = torch.zeros(A * B, dtype=torch.uint8, device=cuda)
    assert lib.lm_transpose_100_noalloc(None, d.data_ptr(), 1, A, B, 1) is True
    assert "at most" in lm.last_error()
    torch.cuda.synchronize()
    assert int(d.count_nonzero()) == 0
