"""Per-shape plan tables kept across calls (stash row offsets): reused from
another stream, kept apart for buffers at different addresses modulo 16,
dropped by finalize; every result bit-exact against the oracle."""
import numpy as np
import pytest

from oracle import lm_oracle as O

pytestmark = pytest.mark.gpu


def test_stash_offsets_cached_across_streams_and_alignments(cuda):
    import torch
    from libmarshal_gb300 import lm
    A, B, e = 1200, 1100, 4  # stash plan (method 3)
    n = A * B
    offsets = (0, 4, 8, 0, 12)  # the 4th repeats the 1st: a cache hit
    raw = torch.zeros(len(offsets) * (n * e + 64), dtype=torch.uint8,
                      device=cuda)
    streams = [torch.cuda.Stream() for _ in range(2)]
    cases = []
    for k, off in enumerate(offsets):
        src = O.random_bits(n, e, 900 + k)
        view = raw[k * (n * e + 64) + off:][: n * e]
        view.copy_(torch.from_numpy(src.view(np.uint8).copy()).to(cuda))
        cases.append((src, view))
    torch.cuda.synchronize()
    for k, (src, view) in enumerate(cases):
        if k == 4:
            lm.finalize()
        st = streams[k % 2]
        assert not lm.lib().lm_transpose_0100_method(
            st.cuda_stream, view.data_ptr(), e, 1, A, B, 1, 3, None), \
            lm.last_error()
        torch.cuda.synchronize()
        got = view.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, O.t100(src, A, B, 1)), k
    assert lm.lib().lm_device_status(None) == 0
