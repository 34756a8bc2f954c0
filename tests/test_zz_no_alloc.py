"""lm_transpose_100_noalloc: the no-allocation entry point.

Some callers cannot allocate device memory while they run: an allocator or
memory manager that converts layouts from inside its own allocation path
(calling cudaMalloc there would re-enter it), or a real-time pipeline that
reserves all device memory at start-up and forbids allocation afterwards.
For them the 100 transposition is also offered with its done bits in a fixed
4 MiB device array.  This file (collected last) calls it through the C ABI:

* after one zero-size warm-up call, two calls in a row per shape, each result
  compared bit for bit with lm_transpose_100 (the regular entry point) and
  with the oracle;
* across those calls neither the device's default memory pool nor the free
  device memory changes (the entry point allocates nothing);
* a shape larger than the array is refused with an error, and the buffer
  (random bytes) is left exactly as it was.
"""
import ctypes

import numpy as np
import pytest

from oracle import lm_oracle as O

pytestmark = pytest.mark.gpu


def _pool_usage():
    """(used, reserved) bytes of device 0's default memory pool, read through
    the driver API."""
    cu = ctypes.CDLL("libcuda.so.1")
    dev = ctypes.c_int()
    pool = ctypes.c_void_p()
    assert cu.cuDeviceGet(ctypes.byref(dev), 0) == 0
    assert cu.cuDeviceGetDefaultMemPool(ctypes.byref(pool), dev) == 0
    out = []
    for attr in (7, 5):  # CU_MEMPOOL_ATTR_USED_MEM_CURRENT, _RESERVED_MEM_CURRENT
        v = ctypes.c_uint64()
        assert cu.cuMemPoolGetAttribute(pool, attr, ctypes.byref(v)) == 0
        out.append(v.value)
    return tuple(out)


def test_no_alloc_matches_regular_entry_point(cuda):
    import torch
    from libmarshal_gb300 import lm
    lib = lm.lib()
    shapes = [(1000, 777, 1, 4), (512, 300, 32, 4), (64, 48, 3, 8),
              (97, 1031, 2, 2), (33, 65, 5000, 1), (4096, 2048, 1, 4)]
    # warm-up: the first call on the device sets it up and converts nothing
    assert lib.lm_transpose_100_noalloc(None, None, 4, 0, 0, 0) is False, \
        lm.last_error()
    cases = []
    for (A, B, b, e) in shapes:
        src = O.random_bits(A * B * b, e, A + B)
        raw = torch.from_numpy(src.view(np.uint8).copy())
        cases.append((A, B, b, e, src, raw.to(cuda), raw.to(cuda)))
    torch.cuda.synchronize()
    for call in range(2):  # two calls in a row on the same buffers
        # the no-allocation calls alone, with the pool and free memory read
        # on both sides
        before = (_pool_usage(), torch.cuda.mem_get_info(cuda)[0])
        for (A, B, b, e, src, d_new, d_ref) in cases:
            assert lib.lm_transpose_100_noalloc(
                None, d_new.data_ptr(), e, A, B, b) is False, lm.last_error()
        torch.cuda.synchronize()
        after = (_pool_usage(), torch.cuda.mem_get_info(cuda)[0])
        assert before == after, (call, before, after)
        for (A, B, b, e, src, d_new, d_ref) in cases:
            assert lib.lm_transpose_100(None, d_ref.data_ptr(), e, A, B, b,
                                        None) is False, lm.last_error()
        torch.cuda.synchronize()
        for (A, B, b, e, src, d_new, d_ref) in cases:
            assert torch.equal(d_new, d_ref), (A, B, b, e, call)
            # the oracle: one 100(A, B, b) per call so far (the second call
            # converts the first call's output again as an [A][B][b] array)
            want = O.t100(src, A, B, b)
            if call == 1:
                want = O.t100(want, A, B, b)
            got = d_new.cpu().numpy().view(O.DTYPES[e])
            assert np.array_equal(got, want), (A, B, b, e, call)
    assert lib.lm_device_status(None) == 0

    # beyond the array's capacity: refused, buffer unchanged
    A, B = 8192, 8192  # 67 M units > 33.5 M
    keep = torch.from_numpy(O.random_bits(A * B, 1, 99)).to(cuda)
    d = keep.clone()
    assert lib.lm_transpose_100_noalloc(None, d.data_ptr(), 1, A, B, 1) is True
    assert "at most" in lm.last_error()
    torch.cuda.synchronize()
    assert torch.equal(d, keep)
