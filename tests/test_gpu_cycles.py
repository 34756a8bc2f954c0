"""Whole-cycle moves (method 5, lm_cycles.cu): shapes whose cycles are all
short, bit-exact against the oracle for every element width, tile counts
and unaligned bases; the planner picks it for the SoA->ASTA shape."""
import numpy as np
import pytest

from oracle import lm_oracle as O

pytestmark = pytest.mark.gpu

CASES = [  # (T, a, B, b, e): order of a modulo a*B - 1 is at most 32
    (1, 4, 64, 32, 4),        # SoA->ASTA shape, 128-byte units
    (1, 64, 4, 32, 4),        # its inverse
    (1, 2, 4096, 8, 8),       # order 13
    (1, 4, 1 << 16, 32, 4),   # order 9, 32 MiB
    (3, 8, 8, 5, 2),          # 0100 with 3 tiles, 10-byte units
    (1, 16, 16, 3, 1),        # 3-byte units
    (2, 4, 1024, 6, 8),       # 48-byte units, 2 tiles
    (1, 4, 1 << 15, 32, 4),   # order 17: cycles beyond 16 units
    (1, 2, 1 << 20, 16, 2),   # order 21, 32-byte units
]


def _run(cuda, T, a, B, b, e, method, offset=0):
    import torch
    from libmarshal_gb300 import lm
    n = T * a * B * b
    src = O.random_bits(n, e, 31 + a + B + b + e)
    raw = torch.zeros(n * e + 64, dtype=torch.uint8, device=cuda)
    view = raw[offset:offset + n * e]
    view.copy_(torch.from_numpy(src.view(np.uint8).copy()).to(cuda))
    bad = lm.lib().lm_transpose_0100_method(None, view.data_ptr(), e, T, a, B,
                                             b, method, None)
    if bad:
        raise lm.LMError(lm.last_error())
    torch.cuda.synchronize()
    got = view.cpu().numpy().view(O.DTYPES[e])
    want = O.t0100(src, T, a, B, b)
    assert np.array_equal(got, want), (T, a, B, b, e, method, offset)


@pytest.mark.parametrize("T,a,B,b,e", CASES)
def test_cycles_method(cuda, T, a, B, b, e):
    _run(cuda, T, a, B, b, e, 5)


@pytest.mark.parametrize("offset", [8, 4])
def test_cycles_unaligned_base(cuda, offset):
    # 128-byte units at a base that is only 8- or 4-byte aligned
    _run(cuda, 1, 4, 256, 32, 4, 5, offset=offset)


def test_cycles_rejects_long_cycles(cuda):
    from libmarshal_gb300 import lm
    with pytest.raises(lm.LMError):
        _run(cuda, 1, 7, 1000, 32, 4, 5)  # order of 7 mod 6999 is long


def test_planner_picks_cycles_for_soa_asta(cuda):
    import torch
    from libmarshal_gb300 import lm
    h, w, t = 1 << 21, 4, 32  # 32 MiB: beyond any on-chip tile
    src = O.random_bits(h * w, 4, 77)
    buf = torch.from_numpy(src.view(np.int32).copy()).to(cuda)
    lm.prof_collect()
    lm.prof_enable(True)
    bad = lm.lib().gpu_soa_asta_pttwac(buf.data_ptr(), h, w, t, None)
    torch.cuda.synchronize()
    lm.prof_enable(False)
    kernels = lm.prof_collect()
    assert not bad
    assert "cycle_move" in kernels, kernels
    got = buf.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, O.soa_asta(src, h, w, t))


def test_cycles_cached_leaders_across_streams(cuda):
    """The leader list of a shape is computed once and reused from another
    stream (which waits for it); finalize drops it and it is rebuilt."""
    import torch
    from libmarshal_gb300 import lm
    T, a, B, b, e = 1, 4, 1 << 14, 32, 4
    n = a * B * b
    srcs = [O.random_bits(n, e, 600 + k) for k in range(3)]
    want = [O.t0100(s, T, a, B, b) for s in srcs]
    bufs = [torch.from_numpy(s.view(np.uint8).copy()).to(cuda) for s in srcs]
    streams = [torch.cuda.Stream() for _ in range(2)]
    torch.cuda.synchronize()
    for k, buf in enumerate(bufs):
        if k == 2:
            lm.finalize()
        st = streams[k % 2]
        assert not lm.lib().lm_transpose_0100_method(
            st.cuda_stream, buf.data_ptr(), e, T, a, B, b, 5, None), \
            lm.last_error()
    torch.cuda.synchronize()
    for buf, w in zip(bufs, want):
        assert np.array_equal(buf.cpu().numpy().view(O.DTYPES[e]), w)


def test_soa_asta_full_size_2p27x4_int32(cuda):
    """The SoA->ASTA configuration at its full size: 2^27 records of 4 int32
    fields (2 GiB), tile 32, i.e. 100(4, 2^22, 32), through the reference's
    drop-in entry point, against the oracle's cpu_soa_asta over all host
    threads; then back (ASTA->SoA) to the input."""
    import os
    import torch
    from libmarshal_gb300 import lm
    h, w, t = 1 << 27, 4, 32
    src = O.random_bits(h * w, 4, 2027)
    want = np.empty_like(src)
    assert O.lib().lmo_soa_asta_mt(src.ctypes.data, want.ctypes.data, h, w,
                                   t, 4, os.cpu_count() or 1) == 0
    buf = torch.from_numpy(src.view(np.int32)).to(cuda)
    assert not lm.lib().gpu_soa_asta_pttwac(buf.data_ptr(), h, w, t, None), \
        lm.last_error()
    torch.cuda.synchronize()
    assert np.array_equal(buf.cpu().numpy().view(np.uint32), want)
    del want
    lm.transpose_100(buf, h // t, w, t, elem_bytes=4)  # ASTA -> SoA
    torch.cuda.synchronize()
    assert np.array_equal(buf.cpu().numpy().view(np.uint32), src)
    assert lm.lib().lm_device_status(None) == 0
    del buf
    torch.cuda.empty_cache()
