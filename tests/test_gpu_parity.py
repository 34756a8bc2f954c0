"""GPU parity: every elementary op, conversion and staged transposition,
through the C ABI, bit-exact against the oracle and against golden digests of
the reference's own CPU code (tests/golden/golden.json)."""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import lm_oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                     "golden.json")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()
                          ).hexdigest()


def make(c, n):
    if c["fill"] == "index":
        return O.index_fill(n, c["e"])
    return O.random_bits(n, c["e"], c["seed"])


def to_dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()
                            ).cuda()


def from_dev(t, e):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy().view(O.DTYPES[e])


@pytest.fixture(scope="module")
def L(cuda):
    from libmarshal_gb300 import lm
    return lm


# ---- AoS <-> ASTA (010) ------------------------------------------------------

@pytest.mark.parametrize("c", GOLDEN["aos_asta"],
                         ids=lambda c: "%s-%dx%d-t%d-e%d" % (
                             c["tag"], c["h"], c["w"], c["t"], c["e"]))
def test_aos_asta_bs_golden(L, c):
    src = make(c, c["h"] * c["w"])
    d = to_dev(src)
    L.aos_asta_bs(d, c["h"], c["w"], c["t"], elem_bytes=c["e"])
    assert sha(from_dev(d, c["e"])) == c["sha256"]


@pytest.mark.parametrize("c", [c for c in GOLDEN["aos_asta"]
                               if c["tag"] in ("cfg1", "bug525", "bug536",
                                               "widths")],
                         ids=lambda c: "%s-%dx%d-t%d-e%d" % (
                             c["tag"], c["h"], c["w"], c["t"], c["e"]))
def test_aos_asta_pttwac_golden(L, c):
    src = make(c, c["h"] * c["w"])
    d = to_dev(src)
    L.aos_asta_pttwac(d, c["h"], c["w"], c["t"], R=1, P=1, elem_bytes=c["e"])
    assert sha(from_dev(d, c["e"])) == c["sha256"]


@pytest.mark.parametrize("R", [1, 2, 4, 8, 16])
def test_010_pttwac_spreading_factors(L, R):
    # bug536 (test/cl_unittest.cc:225-292): w=197, t=32, S_f = R, P = 1
    c = [c for c in GOLDEN["aos_asta"] if c["tag"] == "bug536"
         and c["w"] == 197 and c["t"] == 32][0]
    src = make(c, c["h"] * c["w"])
    d = to_dev(src)
    L.transpose_010_pttwac(d, c["h"] // c["t"], c["t"], c["w"], R=R, P=1,
                           elem_bytes=4)
    assert sha(from_dev(d, 4)) == c["sha256"]


def test_cuda_dropins_cfg1(L, cuda):
    import torch
    c = GOLDEN["aos_asta"][0]
    assert c["tag"] == "cfg1"
    lib = L.lib()
    for fn in ("gpu_aos_asta_bs_float", "gpu_aos_asta_pttwac"):
        src = make(c, c["h"] * c["w"])
        d = to_dev(src)
        assert getattr(lib, fn)(d.data_ptr(), c["h"], c["w"], c["t"], None) \
            is False, L.last_error()
        assert sha(from_dev(d, 4)) == c["sha256"], fn
    # ASTA -> AoS restores the input
    src = make(c, c["h"] * c["w"])
    d = to_dev(src)
    lib.gpu_aos_asta_bs_float(d.data_ptr(), c["h"], c["w"], c["t"], None)
    L.transpose_010_bs(d, c["h"] // c["t"], c["w"], c["t"], elem_bytes=4)
    assert np.array_equal(from_dev(d, 4), src)
    # double variant
    src8 = O.random_bits(16 * 1024 * 6, 8, 5)
    d = to_dev(src8)
    assert lib.gpu_aos_asta_bs_double(d.data_ptr(), 16 * 1024, 6, 16, None) \
        is False
    assert np.array_equal(from_dev(d, 8), O.aos_asta(src8, 16 * 1024, 6, 16))
    # height not a multiple of the tile: error, buffer untouched
    d = to_dev(src)
    assert lib.gpu_aos_asta_bs_float(d.data_ptr(), 1000, 7, 33, None) is True
    assert np.array_equal(from_dev(d, 4), src)
    torch.cuda.synchronize()


# ---- SoA -> ASTA (100) -------------------------------------------------------

@pytest.mark.parametrize("c", GOLDEN["soa_asta"],
                         ids=lambda c: "%s-%dx%d-t%d-e%d" % (
                             c["tag"], c["h"], c["w"], c["t"], c["e"]))
def test_soa_asta_golden(L, c):
    src = make(c, c["h"] * c["w"])
    d = to_dev(src)
    if c["e"] == 4:
        assert L.lib().gpu_soa_asta_pttwac(d.data_ptr(), c["h"], c["w"],
                                           c["t"], None) is False
    else:
        L.transpose_100(d, c["w"], c["h"] // c["t"], c["t"],
                        elem_bytes=c["e"])
    assert sha(from_dev(d, c["e"])) == c["sha256"]


# ---- full transposition (staged planner) -------------------------------------

@pytest.mark.parametrize("c", GOLDEN["full"],
                         ids=lambda c: "%s-%dx%d-e%d" % (c["tag"], c["M"],
                                                         c["N"], c["e"]))
def test_full_transpose_planner_golden(L, c):
    M, N, e = c["M"], c["N"], c["e"]
    A, a, B, b, ph, pw = O.alg5(M, N)
    src = make(c, M * N)
    d = to_dev(src)
    if ph == 0 and pw == 0:
        stages = O.alg3(A, a, B, b)
        L.transpose(d, A, a, B, b, R=1, stages=stages, elem_bytes=e)
    else:
        L.transpose(d, M, 1, N, 1, R=1, stages=0, elem_bytes=e)
    assert sha(from_dev(d, e)) == c["sha256"]


@pytest.mark.parametrize("e", [1, 2, 4, 8])
@pytest.mark.parametrize("stages", [2, 22, 3, 32, 4, 0])
@pytest.mark.parametrize("variant", [1, 2])
def test_cfg2_every_stage_and_variant(L, e, stages, variant):
    # the 7200x1800 staged transposition with index fill; a=100, A=72, b=100, B=18
    c = [c for c in GOLDEN["full"] if c["tag"] == "cfg2" and c["e"] == e][0]
    src = make(c, 7200 * 1800)
    d = to_dev(src)
    # the 010 steps each stage runs: (tiles, a, B)
    steps010 = {2: [(72, 100, 1800)], 22: [(18, 7200, 100)],
                3: [(1296, 100, 100)], 32: [(1296, 100, 100)],
                4: [(1296, 100, 100)], 0: []}[stages]
    if variant == 1 and not all(L.bs_feasible(T, a, B, 1, e)
                                for (T, a, B) in steps010):
        # forcing BS on a tile that cannot be staged on chip is an error,
        # as in the reference past MAX_MEM
        from libmarshal_gb300.lm import LMError
        with pytest.raises(LMError):
            L.transpose(d, 72, 100, 18, 100, R=1, stages=stages,
                        variant010=variant, elem_bytes=e)
        return
    L.transpose(d, 72, 100, 18, 100, R=1, stages=stages, variant010=variant,
                elem_bytes=e)
    assert sha(from_dev(d, e)) == c["sha256"]


# ---- exhaustive small shapes, every width and method ------------------------

def small_shapes(seed, count):
    rng = np.random.default_rng(seed)
    out = [(1, 1, 1, 1), (0, 3, 4, 5), (2, 1, 7, 3), (2, 7, 1, 3),
           (1, 2, 3, 1), (3, 16, 16, 1), (1, 33, 65, 2), (5, 4, 3, 1000),
           (1, 3, 5, 2049)]
    for _ in range(count):
        A = int(rng.integers(1, 6))
        a = int(rng.integers(1, 40))
        B = int(rng.integers(1, 40))
        b = int(rng.choice([1, 1, 2, 3, 4, 7, 16, 33, 64, 100]))
        out.append((A, a, B, b))
    return out


@pytest.mark.parametrize("e", [1, 2, 4, 8])
@pytest.mark.parametrize("method", [0, 1, 2])
def test_0100_small_shapes(L, e, method):
    for (A, a, B, b) in small_shapes(100 * e + method, 60):
        n = A * a * B * b
        src = O.random_bits(max(n, 1), e, A + a + B + b)[:n]
        d = to_dev(src) if n else None
        if n == 0:
            import torch
            d = torch.zeros(8, dtype=torch.uint8, device="cuda")
            L.transpose_0100(d, A, a, B, b, method=method, elem_bytes=e)
            continue
        L.transpose_0100(d, A, a, B, b, method=method, elem_bytes=e)
        assert np.array_equal(from_dev(d, e), O.t0100(src, A, a, B, b)), \
            (A, a, B, b, e, method)


@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_unaligned_buffers(L, e):
    import torch
    for (A, B, b) in ((37, 29, 32), (64, 48, 16), (100, 77, 3)):
        n = A * B * b
        src = O.random_bits(n, e, 9)
        big = torch.zeros((n + 16) * e, dtype=torch.uint8, device="cuda")
        off = e  # one element past the allocation's alignment
        big[off:off + n * e] = to_dev(src)
        ptr = big.data_ptr() + off
        assert L.lib().lm_transpose_100(None, ptr, e, A, B, b, None) is False, \
            L.last_error()
        got = big[off:off + n * e].cpu().numpy().view(O.DTYPES[e])
        assert np.array_equal(got, O.t100(src, A, B, b))


def test_large_tiles_use_clusters(L):
    # 010 tiles of 32 x 12289 fp32 (1.57 MB) and 16 x 16000 fp64 (2 MB)
    for (A, a, B, e) in ((3, 32, 12289, 4), (2, 16, 16000, 8),
                         (4, 8, 30000, 4)):
        assert L.bs_feasible(A, a, B, 1, e)
        src = O.random_bits(A * a * B, e, 1)
        d = to_dev(src)
        L.transpose_010_bs(d, A, a, B, elem_bytes=e)
        assert np.array_equal(from_dev(d, e), O.t010(src, A, a, B))


def test_bs_reports_capacity_error(L):
    # a 2 x 2^21 fp64 tile (32 MB) cannot be staged on chip
    from libmarshal_gb300.lm import LMError
    import torch
    d = torch.zeros(2 * (1 << 21) * 8, dtype=torch.uint8, device="cuda")
    with pytest.raises(LMError):
        L.transpose_010_bs(d, 1, 2, 1 << 21, elem_bytes=8)
    # the planner / PTTWAC path handles it
    src = O.random_bits(2 * (1 << 21), 8, 4)
    d = to_dev(src)
    L.transpose_0100(d, 1, 2, 1 << 21, 1, elem_bytes=8)
    assert np.array_equal(from_dev(d, 8), O.t010(src, 1, 2, 1 << 21))


# ---- padding -----------------------------------------------------------------

@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_padding_unpadding(L, e):
    import torch
    rng = np.random.default_rng(e)
    shapes = [(1000, 1001, 1003), (12289, 300, 12291), (5, 70000, 9),
              (3, 2, 3), (64, 64, 64), (1, 100000, 2)]
    for _ in range(6):
        x = int(rng.integers(1, 3000))
        y = int(rng.integers(1, 3000))
        shapes.append((x, y, x + int(rng.integers(0, 40))))
    for (x, y, pad) in shapes:
        buf = O.random_bits(y * pad, e, x + y)
        d = to_dev(buf)
        L.padding(d, x, y, pad, elem_bytes=e)
        got = from_dev(d, e)
        want = O.padding(buf, x, y, pad)
        assert np.array_equal(got, want), ("pad", x, y, pad, e)
        L.unpadding(d, x, y, pad, elem_bytes=e)
        assert np.array_equal(from_dev(d, e), O.unpadding(want, x, y, pad)), \
            ("unpad", x, y, pad, e)
    torch.cuda.synchronize()


def test_pad_transpose_unpad_flow(L):
    # The reference's `full` test flow (test/cl_unittest.cc:396-640): pad the
    # columns to a factorable width, transpose, unpad; 1000 x 1009 (prime).
    h, w = 1000, 1009
    A, a, B, b, ph, pw = O.alg5(h, w)
    H, W = h + ph, w + pw
    src = O.random_bits(h * w, 4, 77)
    buf = np.zeros(H * W, dtype=np.uint32)
    buf[:h * w] = src
    d = to_dev(buf)
    if pw:
        L.padding(d, w, h, W, elem_bytes=4)
    L.transpose(d, A, a, B, b, R=1, stages=O.alg3(A, a, B, b), elem_bytes=4)
    if ph:
        L.unpadding(d, h, w, H, elem_bytes=4)
    else:
        L.unpadding(d, h, w, H, elem_bytes=4)  # H == h: keeps first w rows
    got = from_dev(d, 4)[:h * w]
    assert np.array_equal(got, O.transpose(src, h, w))


# ---- failure detection without a GPU fault -----------------------------------

@pytest.mark.parametrize("unpad", [0, 1])
def test_bounded_wait_reports_timeout(L, unpad):
    import torch
    x, y, pad = 1000, 2000, 1010
    buf = O.random_bits(y * pad, 4, 1)
    d = to_dev(buf)
    failed = L.lib().lm_debug_pad_stall(None, d.data_ptr(), 4, x, y, pad,
                                        unpad, 3, 50_000_000)
    assert failed is True
    assert "timed out" in L.last_error()
    # the context is still usable
    d2 = to_dev(buf)
    L.padding(d2, x, y, pad, elem_bytes=4)
    assert np.array_equal(from_dev(d2, 4), O.padding(buf, x, y, pad))
    torch.cuda.synchronize()


# ---- Python API (src/py/transpose.py) ----------------------------------------

def test_python_array_api(L):
    import torch
    from libmarshal_gb300 import TransposeArrayInPlace, FullTranspose, T010_BS
    # transpose_unittest.py:82-94 shape
    A, a, B, b = 40, 16, 37, 10
    src = O.random_bits(A * a * B * b, 4, 3).reshape(A * a, B * b)
    t = torch.from_numpy(src.view(np.float32).copy()).cuda()
    out = TransposeArrayInPlace(t, a, b)
    assert tuple(out.shape) == (B * b, A * a)
    assert out.data_ptr() == t.data_ptr()
    assert np.array_equal(out.cpu().numpy().view(np.uint32), src.T)
    # transpose_unittest.py:39-57
    for a in (4, 8, 16, 32, 64):
        src = O.random_bits(40 * a * 37 * 30, 4, a)
        t = torch.from_numpy(src.view(np.float32).copy()).cuda()
        steps = FullTranspose(None, t, 40, a, 37, 30)
        torch.cuda.synchronize()
        assert np.array_equal(t.cpu().numpy().view(np.uint32),
                              O.transpose(src, 40 * a, 37 * 30))
        assert all(s.Throughput() > 0 for s in steps)
    # transpose_unittest.py:59-80
    for a in (4, 8, 16, 32, 64):
        src = O.random_bits(40 * a * 37, 4, a + 1)
        t = torch.from_numpy(src.view(np.float32).copy()).cuda()
        op = T010_BS(40, a, 37)
        assert op.IsFeasible(t)
        op.Transpose(None, t)
        assert op.Throughput() > 0
        assert np.array_equal(t.cpu().numpy().view(np.uint32),
                              O.t010(src, 40, a, 37))


def test_elapsed_time_accumulates(L):
    src = O.random_bits(1024 * 999, 4, 2)
    d = to_dev(src)
    et = ctypes.c_ulonglong(5)
    assert L.lib().lm_transpose_100(None, d.data_ptr(), 4, 1024, 999, 1,
                                    ctypes.byref(et)) is False
    assert et.value > 5


# ---- every plan of the 100 / 0100 planner ------------------------------------

@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_every_method_on_medium_100(L, e):
    # methods: 0 planner, 1 BS (may refuse), 2 PTTWAC, 3 stash, 4 two-pass,
    # 5 whole cycles (refuses long cycles), 6 through scratch
    from libmarshal_gb300.lm import LMError
    shapes = [(2048, 1031, 1), (1031, 2048, 1), (1500, 1200, 3),
              (4096, 600, 2), (700, 3000, 1), (3000, 700, 5), (3, 50000, 7),
              (40000, 37, 1)]
    for (A, B, b) in shapes:
        src = O.random_bits(A * B * b, e, A * 7 + B)
        want = O.t100(src, A, B, b)
        for method in (0, 1, 2, 3, 4, 5, 6):
            d = to_dev(src)
            try:
                L.transpose_0100(d, 1, A, B, b, method=method, elem_bytes=e)
            except LMError:
                assert method in (1, 3, 4, 5), (A, B, b, e, method)
                continue
            assert np.array_equal(from_dev(d, e), want), (A, B, b, e, method)
    assert L.lib().lm_device_status(None) == 0


@pytest.mark.parametrize("e", [4, 8])
def test_stash_plan_shapes(L, e):
    # shapes with a partial last column group, few and many rows per chunk
    rng = np.random.default_rng(e)
    for _ in range(8):
        A = int(rng.integers(300, 5000))
        B = int(rng.integers(300, 5000))
        b = int(rng.choice([1, 1, 2, 3, 7]))
        if A * B * b * e > (64 << 20):
            continue
        src = O.random_bits(A * B * b, e, A + B)
        d = to_dev(src)
        L.transpose_0100(d, 1, A, B, b, method=3, elem_bytes=e)
        assert np.array_equal(from_dev(d, e), O.t100(src, A, B, b)), (A, B, b)
    assert L.lib().lm_device_status(None) == 0


def _full_size_100(L, A, B, e, seed):
    import torch
    n = A * B
    src = O.random_bits(n, e, seed)
    want = np.empty_like(src)
    O.lib().lmo_soa_asta_mt(src.ctypes.data, want.ctypes.data, B, A, 1, e,
                            os.cpu_count() or 1)
    d = to_dev(src)
    L.transpose_100(d, A, B, 1, elem_bytes=e)
    got = from_dev(d, e)
    assert np.array_equal(got, want), (A, B, e)
    # and back: the size-independent round-trip property
    L.transpose_100(d, B, A, 1, elem_bytes=e)
    assert np.array_equal(from_dev(d, e), src)
    assert L.lib().lm_device_status(None) == 0
    del d
    torch.cuda.empty_cache()


def test_headline_full_size_fp32(L):
    # the headline workload: in-place 100 of the fp32 16384 x 12289 matrix
    _full_size_100(L, 16384, 12289, 4, 2024)


@pytest.mark.slow
def test_large_fp64_32768x16000(L):
    _full_size_100(L, 32768, 16000, 8, 2025)


@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_staged_method_shapes(L, e):
    """Method 6 (through scratch) on 0100s with several tiles, units of
    several elements, ragged block edges and a base that is only
    element-aligned."""
    import torch
    rng = np.random.default_rng(60 + e)
    for _ in range(6):
        T = int(rng.integers(1, 4))
        a = int(rng.integers(2, 700))
        B = int(rng.integers(2, 700))
        b = int(rng.choice([1, 2, 3, 8]))
        n = T * a * B * b
        src = O.random_bits(n, e, T + a + B + b)
        raw = torch.zeros(n * e + 64, dtype=torch.uint8, device="cuda")
        view = raw[e:e + n * e]
        view.copy_(torch.from_numpy(src.view(np.uint8).copy()).cuda())
        assert not L.lib().lm_transpose_0100_method(
            None, view.data_ptr(), e, T, a, B, b, 6, None), L.last_error()
        torch.cuda.synchronize()
        got = view.cpu().numpy().view(O.DTYPES[e])
        assert np.array_equal(got, O.t0100(src, T, a, B, b)), (T, a, B, b, e)
    assert L.lib().lm_device_status(None) == 0


TILE010_SHAPES = [
    # (T, a, B): a*e or B*e a multiple of 16 bytes selects the 16-byte
    # tile form (form A: output rows whole vectors; form B: input rows)
    (7, 32, 11), (5, 16, 3), (9, 11, 32), (3, 7, 16), (4, 16, 5),
    (3, 5, 2), (6, 2, 9), (40, 64, 3), (2, 3, 16), (1000, 16, 4),
    (1, 64, 200), (2049, 32, 7), (777, 13, 64), (3, 512, 16), (5, 16, 512),
    (4, 64, 700), (3, 700, 64), (2, 1000, 32), (3, 48, 1000),
    (3, 32, 1700), (2, 1700, 32), (3, 16, 7000),
    # output rows of whole 8- or 4-byte vectors only (chunks not 16-byte
    # aligned): form A with narrower vectors
    (1296, 100, 100), (7, 12, 5), (5, 24, 7), (9, 6, 13), (333, 20, 9),
]


@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_tile010_forms(L, e):
    """010 on 16-byte aligned buffers through the vector tile kernel (both
    forms, 16-, 8- and 4-byte output vectors, ragged last chunk, one-tile
    and many-tile cases) and with it switched off (the element-wise tile
    kernel), against the oracle."""
    import torch
    for (T, a, B) in TILE010_SHAPES:
        if a * B * e > 112 * 1024:
            continue
        n = T * a * B
        src = O.random_bits(n, e, T + a + B)
        want = O.t010(src, T, a, B)
        d = to_dev(src)
        assert d.data_ptr() % 16 == 0
        L.transpose_010_bs(d, T, a, B, elem_bytes=e)
        assert np.array_equal(from_dev(d, e), want), (T, a, B, e)
        # the same through the conversion entry points (AoS -> ASTA is
        # 010(h/t, t, w); ASTA -> AoS is 010(h/t, w, t))
        d = to_dev(src)
        L.aos_asta_bs(d, T * a, B, a, elem_bytes=e)
        assert np.array_equal(from_dev(d, e), want), ("aos", T, a, B, e)
        os.environ["LM_NO_TILE010"] = "1"
        try:
            d = to_dev(src)
            L.transpose_010_bs(d, T, a, B, elem_bytes=e)
            assert np.array_equal(from_dev(d, e), want), ("off", T, a, B, e)
        finally:
            del os.environ["LM_NO_TILE010"]
    assert L.lib().lm_device_status(None) == 0


@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_010_unaligned_buffers(L, e):
    """010 on a buffer that is only element-aligned: the 16-byte tile kernel
    declines it and the element-wise tile kernel (or its fallbacks) must
    give the oracle's result."""
    import torch
    for (T, a, B) in ((9, 32, 11), (5, 11, 32), (3, 64, 700), (2, 16, 3)):
        if a * B * e > 112 * 1024:
            continue
        n = T * a * B
        src = O.random_bits(n, e, T + a + B + 7)
        raw = torch.zeros(n * e + 64, dtype=torch.uint8, device="cuda")
        view = raw[e:e + n * e]
        view.copy_(torch.from_numpy(src.view(np.uint8).copy()).cuda())
        assert view.data_ptr() % 16 != 0
        assert not L.lib().lm_transpose_010_bs(None, view.data_ptr(), e, T, a,
                                               B, None), L.last_error()
        torch.cuda.synchronize()
        got = view.cpu().numpy().view(O.DTYPES[e])
        assert np.array_equal(got, O.t010(src, T, a, B)), (T, a, B, e)


@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_pttwac_walkers_racing_in_long_cycles(L, e):
    """Cycle following (method 2) where nearly every walker starts inside the
    same few long cycles at once: small A*B (one walker per position, all
    launched together), shapes with long cycles, units of one to many
    elements, several tiles; repeated, since the claim and start races are
    timing dependent.  Bit-exact against the oracle every time."""
    shapes = [(1, 3, 5, 1), (1, 7, 11, 1), (1, 13, 17, 3), (1, 61, 67, 1),
              (1, 127, 131, 2), (1, 255, 257, 1), (1, 1000, 999, 1),
              (1, 4, 1023, 8), (1, 1023, 4, 64), (8, 37, 41, 2),
              (3, 509, 521, 1)]
    for (T, a, B, b) in shapes:
        src = O.random_bits(T * a * B * b, e, T + a + B + b)
        want = O.t0100(src, T, a, B, b)
        for rep in range(8):
            d = to_dev(src)
            L.transpose_0100(d, T, a, B, b, method=2, elem_bytes=e)
            assert np.array_equal(from_dev(d, e), want), (T, a, B, b, e, rep)
    assert L.lib().lm_device_status(None) == 0


def test_full_transpose_reference_suite(L):
    """lm_full_transpose on the reference's `full` suite (15 seeded general
    matrices, h and w in [1000, 20000), single precision): the reference's
    flow -- Algorithm 5 padding, the Algorithm 3 staged transposition with
    BS 010 steps, unpadding -- and the direct form (one planned 100), and on
    the five smallest shapes the flow with PTTWAC 010 steps; each against the
    oracle's transpose (all host threads)."""
    import torch
    from tests.test_oracle import full_suite_shapes
    shapes = full_suite_shapes()
    small = sorted(shapes, key=lambda s: s[0] * s[1])[:5]
    for n, (M, N) in enumerate(shapes):
        src = O.random_bits(M * N, 4, 300 + n)
        want = np.empty_like(src)
        O.lib().lmo_soa_asta_mt(src.ctypes.data, want.ctypes.data, N, M, 1, 4,
                                os.cpu_count() or 1)
        (plan, need) = L.full_transpose_plan(M, N, 4)
        for variant in ((1, 2) if (M, N) in small else (1,)) + (0,):
            d = torch.empty(need if variant else M * N, dtype=torch.int32,
                            device="cuda")
            d[:M * N].copy_(torch.from_numpy(src.view(np.int32)))
            L.full_transpose(d, M, N, variant010=variant)
            torch.cuda.synchronize()
            got = d[:M * N].cpu().numpy().view(np.uint32)
            assert np.array_equal(got, want), (M, N, plan, variant)
            del d
        torch.cuda.empty_cache()
    assert L.lib().lm_device_status(None) == 0


@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_staged_narrow_vector_store(L, e):
    """The staged form (method 6) on one-element units: 1- and 2-byte shapes
    whose staged rows start on 32-bit words and whose output vectors land on
    16 bytes take the word-column vector store, shapes whose output rows
    allow 16-, 8- or 4-byte vectors (16 for 4- and 8-byte elements) the
    element-column vector store (rows on any boundary), the others the
    element-wise one; several tiles, ragged block edges; bit-exact against
    the oracle."""
    shapes = [(1, 7200, 1800), (1, 1024, 4000), (3, 256, 1000),
              (1, 4096, 500), (2, 48, 2000), (1, 7200, 1801),
              (1, 1000, 1000), (1, 336, 4004), (4, 160, 24),
              (1, 500, 1003), (2, 52, 777), (1, 4100, 999), (1, 500, 1001),
              (3, 6, 1000), (1, 4098, 333), (5, 1000, 37)]
    for (T, a, B) in shapes:
        src = O.random_bits(T * a * B, e, T + a + B)
        d = to_dev(src)
        L.transpose_0100(d, T, a, B, 1, method=6, elem_bytes=e)
        assert np.array_equal(from_dev(d, e), O.t0100(src, T, a, B, 1)), \
            (T, a, B, e)
    assert L.lib().lm_device_status(None) == 0


@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_resident_form(L, e):
    """The shared-memory-resident form (method 7: every CTA loads its blocks,
    grid barrier, blocks written transposed over the buffer): one- and
    many-tile shapes, units of one to many elements, ragged block edges,
    fewer blocks than SMs, a buffer that is only element-aligned; bit-exact
    against the oracle.  A payload beyond the shared memory of all SMs is
    refused with the buffer unchanged."""
    import torch
    shapes = [(1, 7200, 1800, 1), (1, 1000, 1000, 1), (3, 256, 1000, 1),
              (1, 4096, 500, 1), (1, 7200, 1801, 1), (5, 100, 90, 3),
              (1, 33, 65, 7), (2, 2000, 300, 2), (1, 3, 5, 1), (1, 1500, 1700, 1)]
    for (T, a, B, b) in shapes:
        n = T * a * B * b
        if n * e > 24 << 20:
            continue
        src = O.random_bits(n, e, T + a + B + b)
        want = O.t0100(src, T, a, B, b)
        d = to_dev(src)
        L.transpose_0100(d, T, a, B, b, method=7, elem_bytes=e)
        assert np.array_equal(from_dev(d, e), want), (T, a, B, b, e)
        # element-aligned only
        raw = torch.zeros(n * e + 64, dtype=torch.uint8, device="cuda")
        view = raw[e:e + n * e]
        view.copy_(torch.from_numpy(src.view(np.uint8).copy()).cuda())
        L.transpose_0100(view, T, a, B, b, method=7, elem_bytes=e)
        assert np.array_equal(from_dev(view, e), want), (T, a, B, b, e, "un")
    assert L.lib().lm_device_status(None) == 0
    # too large for shared memory: refused, buffer unchanged
    from libmarshal_gb300.lm import LMError
    n = (48 << 20) // e
    keep = torch.from_numpy(O.random_bits(n, e, 5).view(np.uint8).copy()).cuda()
    d = keep.clone()
    with pytest.raises(LMError):
        L.transpose_0100(d, 1, 8192, n // 8192, 1, method=7, elem_bytes=e)
    torch.cuda.synchronize()
    assert torch.equal(d, keep)


def test_resident_form_is_the_route_for_7200x1800(L):
    """The 7200 x 1800 transposition of bytes and half-words (13 and 26 MB)
    fits the shared memory of all SMs: the planner runs it as the resident
    form, one launch."""
    for e in (1, 2):
        src = O.random_bits(7200 * 1800, e, 11)
        d = to_dev(src)
        L.prof_collect()
        L.prof_enable(True)
        try:
            L.transpose_100(d, 7200, 1800, 1, elem_bytes=e)
            from_dev(d, e)
        finally:
            L.prof_enable(False)
        ran = L.prof_collect()
        assert list(ran) == ["resident"], ran
        assert ran["resident"][0] == 1
        assert np.array_equal(from_dev(d, e), O.t100(src, 7200, 1800, 1))


def test_resident_barrier_timeout_is_reported(L, cuda):
    """Failure detection for the resident form's grid barrier: a launch whose
    barrier waits for one CTA more than it has gives up after 50 ms in every
    CTA, reports the timeout, writes nothing, and the context stays
    usable."""
    import torch
    A, a, B, b, e = 1, 3000, 1000, 1, 1
    src = O.random_bits(a * B, e, 21)
    d = to_dev(src)
    keep = d.clone()
    failed = L.lib().lm_debug_resident_stall(None, d.data_ptr(), e, A, a, B,
                                             b, 50_000_000)
    assert failed is True
    assert "timed out" in L.last_error()
    torch.cuda.synchronize()
    assert torch.equal(d, keep)
    assert L.lib().lm_device_status(None) == 0
    # the next resident launches (and their barrier slots) work
    for _ in range(3):
        L.transpose_0100(d, A, a, B, b, method=7, elem_bytes=e)
        L.transpose_0100(d, A, B, a, b, method=7, elem_bytes=e)
    assert np.array_equal(from_dev(d, e), src)


def test_resident_concurrent_streams(L, cuda):
    """Resident launches from several host threads on their own streams at
    once: each launch gets its own barrier slot and target, so concurrent
    launches (which may share the SMs) never pass each other's barrier;
    every result bit-exact."""
    import threading
    import torch
    shapes = [(1, 2000, 1500, 1, 1), (1, 1200, 900, 1, 2), (3, 400, 500, 1, 4),
              (1, 777, 1333, 1, 8)]
    errors = []

    def work(k):
        try:
            T, a, B, b, e = shapes[k % len(shapes)]
            s = torch.cuda.Stream()
            src = O.random_bits(T * a * B * b, e, 100 + k)
            d = to_dev(src)
            torch.cuda.synchronize()
            with torch.cuda.stream(s):
                for _ in range(5):
                    L.transpose_0100(d, T, a, B, b, method=7, elem_bytes=e,
                                     stream=s)
                    L.transpose_0100(d, T, B, a, b, method=7, elem_bytes=e,
                                     stream=s)
                L.transpose_0100(d, T, a, B, b, method=7, elem_bytes=e,
                                 stream=s)
            s.synchronize()
            got = d.cpu().numpy().view(O.DTYPES[e])
            if not np.array_equal(got, O.t0100(src, T, a, B, b)):
                errors.append(k)
        except Exception as exc:  # reported below
            errors.append((k, repr(exc)))

    threads = [threading.Thread(target=work, args=(k,)) for k in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    assert L.lib().lm_device_status(None) == 0


@pytest.mark.parametrize("e", [1, 4])
def test_staged_l2_copy_back_sizes(L, e):
    """The staged form's copy back by cudaMemcpyAsync (up to 48 MB and from
    208 MB) and by the kernel that drops each scratch line from L2 once read
    (48-208 MB): one transposition on each side of the lower edge and one
    inside the range, bit-exact against the oracle."""
    for (A, B) in ((4000, 10000 // e), (4000, 16000 // e), (6000, 16000 // e)):
        src = O.random_bits(A * B, e, A + B)
        d = to_dev(src)
        L.transpose_0100(d, 1, A, B, 1, method=6, elem_bytes=e)
        assert np.array_equal(from_dev(d, e), O.t0100(src, 1, A, B, 1)), \
            (A, B, e)
        del d
    assert L.lib().lm_device_status(None) == 0
