"""Pins the CPU oracle (oracle/lm_oracle.c) -- no GPU needed.

1. Against golden vectors produced by the reference's OWN CPU code
   (tests/golden/golden.json, made by tests/golden/gen_golden.py from
   test/cl_unittest.cc:138-166, test/unittest.cu:68-82, include/plan.hpp).
2. Against the known answers of the reference's tests
   (test/cl_unittest.cc:705-709) and the shapes its planner picks.
3. Internal consistency: the in-place cycle follower equals the out-of-place
   layouts; round trips; numpy restatements.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import lm_oracle as O

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                     "golden.json")))


def sha(a):
    return hashlib.sha256(a.view(np.uint8).tobytes()).hexdigest()


def make(c, n):
    if c["fill"] == "index":
        return O.index_fill(n, c["e"])
    return O.random_bits(n, c["e"], c["seed"])


@pytest.mark.parametrize("c", GOLDEN["aos_asta"],
                         ids=lambda c: "%s-%dx%d-t%d-e%d" % (
                             c["tag"], c["h"], c["w"], c["t"], c["e"]))
def test_aos_asta_matches_reference(c):
    src = make(c, c["h"] * c["w"])
    assert sha(O.aos_asta(src, c["h"], c["w"], c["t"])) == c["sha256"]


@pytest.mark.parametrize("c", GOLDEN["soa_asta"],
                         ids=lambda c: "%s-%dx%d-t%d-e%d" % (
                             c["tag"], c["h"], c["w"], c["t"], c["e"]))
def test_soa_asta_matches_reference(c):
    src = make(c, c["h"] * c["w"])
    assert sha(O.soa_asta(src, c["h"], c["w"], c["t"])) == c["sha256"]


@pytest.mark.parametrize("c", GOLDEN["full"],
                         ids=lambda c: "%s-%dx%d-e%d" % (c["tag"], c["M"],
                                                         c["N"], c["e"]))
def test_full_transpose_matches_reference(c):
    src = make(c, c["M"] * c["N"])
    got = O.transpose(src, c["M"], c["N"])
    assert sha(got) == c["sha256"]
    # and it is the matrix transpose
    assert np.array_equal(got.reshape(c["N"], c["M"]),
                          src.reshape(c["M"], c["N"]).T)


def test_num_cycles_matches_reference():
    for m, n, want in GOLDEN["num_cycles"]:
        assert O.num_cycles(m, n) == want, (m, n)
        assert O.num_cycles_fast(m, n) == want, (m, n)


def test_known_cycle_counts():
    # test/cl_unittest.cc:705-709
    assert O.num_cycles(2, 3) == 1
    assert O.num_cycles(3, 5) == 2


def test_next_matches_reference_with_wraparound():
    for i, m, n, want in GOLDEN["next"]:
        assert O.next_index(i, m, n) == want, (i, m, n)


def test_factorize_and_tile_options_match_reference():
    for n, want in GOLDEN["tile_options"]:
        assert O.tile_options(n) == want, n
    for n, want in GOLDEN["factors"]:
        assert [list(p) for p in O.factorize(n)] == want, n


def test_alg5_alg3_baseline_shapes():
    # the 7200x1800 staged transposition: a=100, A=72, b=100, B=18, no padding, stage 3
    assert O.alg5(7200, 1800) == (72, 100, 18, 100, 0, 0)
    assert O.alg3(72, 100, 18, 100) == 3
    # 16384x12289 (12289 prime): pads w to 12291 = 3*17*241 -> b=51, stage 32
    assert O.alg5(16384, 12289) == (256, 64, 241, 51, 0, 2)
    assert O.alg3(256, 64, 241, 51) == 32
    # 32768x16000: a=64, b=100, stage 3
    assert O.alg5(32768, 16000) == (512, 64, 160, 100, 0, 0)
    assert O.alg3(512, 64, 160, 100) == 3


@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_inplace_cycle_follower_equals_layouts(e):
    rng = np.random.default_rng(e)
    for _ in range(40):
        A, B, b = (int(v) for v in rng.integers(1, 40, size=3))
        src = O.random_bits(A * B * b, e, int(rng.integers(1 << 30)))
        buf = src.copy()
        O.inplace_100(buf, A, B, b)
        assert np.array_equal(buf, O.t100(src, A, B, b)), (A, B, b)


@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_elementary_ops_against_numpy(e):
    rng = np.random.default_rng(10 + e)
    for _ in range(30):
        A, a, B, b = (int(v) for v in rng.integers(1, 13, size=4))
        src = O.random_bits(A * a * B * b, e, 7)
        x = src.reshape(A, a, B, b)
        assert np.array_equal(O.t0100(src, A, a, B, b),
                              x.transpose(0, 2, 1, 3).reshape(-1))
        y = src[:A * a * B].reshape(A, a, B)
        assert np.array_equal(O.t010(np.ascontiguousarray(src[:A * a * B]),
                                     A, a, B),
                              y.transpose(0, 2, 1).reshape(-1))
        z = src[:A * B * b].reshape(A, B, b)
        assert np.array_equal(O.t100(np.ascontiguousarray(src[:A * B * b]),
                                     A, B, b),
                              z.transpose(1, 0, 2).reshape(-1))


def test_cfg1_round_trip():
    src = O.random_bits(65536 * 7, 4, 0)
    asta = O.aos_asta(src, 65536, 7, 32)
    assert np.array_equal(O.t010(asta, 2048, 7, 32), src)


@pytest.mark.parametrize("e", [1, 2, 4, 8])
def test_padding_semantics(e):
    rng = np.random.default_rng(20 + e)
    for _ in range(20):
        x, y = (int(v) for v in rng.integers(1, 50, size=2))
        pad = x + int(rng.integers(0, 9))
        buf = O.random_bits(y * pad, e, 3)
        out = O.padding(buf, x, y, pad)
        want = np.zeros((y, pad), dtype=buf.dtype)
        want[:, :x] = buf[:y * x].reshape(y, x)
        assert np.array_equal(out, want.reshape(-1))
        back = O.unpadding(out, x, y, pad)
        want2 = np.zeros(y * pad, dtype=buf.dtype)
        want2[:y * x] = buf[:y * x]
        assert np.array_equal(back, want2)


def test_oracle_rejects_bad_tiles():
    src = O.random_bits(10 * 3, 4, 0)
    with pytest.raises(ValueError):
        O.aos_asta(src, 10, 3, 4)  # 4 does not divide 10


def full_suite_shapes():
    """The reference's `full` test shapes (test/cl_unittest.cc:344-389,
    single precision, general matrices): srand(n + 1), h = rand() % 19000 +
    1000, w = rand() % 19000 + 1000, n = 0..14, with the C library's rand()."""
    import ctypes
    libc = ctypes.CDLL("libc.so.6")
    out = []
    for n in range(15):
        libc.srand(n + 1)
        h = libc.rand() % 19000 + 1000
        w = libc.rand() % 19000 + 1000
        out.append((h, w))
    return out


def test_library_full_transpose_plan_matches_oracle(built):
    """lm_full_transpose_plan (the library's Algorithm 5 / Algorithm 3) gives
    the oracle's super-element sizes, padding and stage code: for the
    reference's full suite, the PPoPP'14 sizes and seeded shapes, with the
    single- (12288) and double-precision (6144) local-memory limits."""
    from libmarshal_gb300 import lm
    rng = np.random.default_rng(5)
    shapes = full_suite_shapes() + [(7200, 1800), (1800, 7200), (5100, 2500),
                                    (16384, 12289), (23, 5), (97, 101)]
    shapes += [tuple(int(x) for x in rng.integers(1, 30000, 2))
               for _ in range(40)]
    for (h, w) in shapes:
        for e, mm in ((4, 12288), (8, 6144)):
            A, a, B, b, ph, pw = O.alg5(h, w, mm)
            plan, need = lm.full_transpose_plan(h, w, e)
            assert plan == (A, a, B, b, ph, pw, O.alg3(A, a, B, b, mm)), \
                (h, w, e)
            assert need == (h + ph) * (w + pw)
