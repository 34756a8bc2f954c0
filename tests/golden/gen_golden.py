"""Generate tests/golden/golden.json from the reference's OWN CPU code.

Run in a container that has the reference checkout, naming its root:

    python tests/golden/gen_golden.py <reference-root>   (or LM_REFERENCE=...)

It builds oracle/_ref/libref_cpu.so with oracle/build_ref.sh (the reference's
cpu_aos_asta / cpu_soa_asta from test/cl_unittest.cc:138-166, the templated
cpu_aos_asta from test/unittest.cu:68-82, and include/plan.hpp), runs them on
seeded inputs and records SHA-256 digests of the outputs plus the planner
answers.  The fixture therefore holds only digests and small integers -- no
reference code and no bulk data.

Inputs are regenerated identically in the tests: splitmix64(seed) bytes
(oracle.lm_oracle.random_bits) or the linear-index fill (index_fill).

Shapes follow the reference's own suites (test/cl_unittest.cc:170-387,
test/unittest.cu:101-246), scaled where noted so the CPU suite stays fast.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import lm_oracle as O  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden", "golden.json")
SUF = {1: "u8", 2: "u16", 4: "u32", 8: "u64"}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(a.view(np.uint8).tobytes()).hexdigest()


def make_input(kind: str, n: int, e: int, seed: int) -> np.ndarray:
    if kind == "index":
        return O.index_fill(n, e)
    return O.random_bits(n, e, seed)


def aos_cases():
    c = []
    # AoS [65536][7] fp32 to ASTA with tile 32, and the inverse.
    c.append(dict(h=65536, w=7, t=32, e=4, fill="random", seed=0, tag="cfg1"))
    c.append(dict(h=2048 * 7, w=32, t=7, e=4, fill="random", seed=0,
                  tag="cfg1-inverse-on-random"))
    # bug524 / bug525 (unittest.cu:147-196): h=16384, t=16, w in 1..99 (subset).
    for w in (1, 2, 3, 5, 6, 7, 16, 31, 33, 64, 66, 97, 99):
        c.append(dict(h=16384, w=w, t=16, e=4, fill="random", seed=5432,
                      tag="bug525"))
    # bug533 (cl_unittest.cc:294-325): w=3*2^k<=384, t=1..8,
    # h=(500/w+1)*(13000+t-1)/t*t; h scaled by 1/8 to keep the suite fast.
    for w in (3, 6, 12, 24, 48, 96, 192, 384):
        for t in (1, 2, 3, 5, 7, 8):
            h = ((500 // w + 1) * (13000 + t - 1) // t * t) // 8 // t * t
            c.append(dict(h=h, w=w, t=t, e=4, fill="random", seed=w * 16 + t,
                          tag="bug533"))
    # bug536 (cl_unittest.cc:225-292): w in {197,215}, t in {16,32,64}.
    for w, hs in ((197, 35588), (215, 44609)):
        for t in (16, 32, 64):
            h = (hs + t - 1) // t * t
            c.append(dict(h=h, w=w, t=t, e=4, fill="random", seed=7,
                          tag="bug536"))
    # every element width
    for e in (1, 2, 4, 8):
        for (h, w, t) in ((4096, 7, 32), (1000, 13, 8), (96, 100, 96),
                          (64 * 3, 37, 64)):
            c.append(dict(h=h, w=w, t=t, e=e, fill="random", seed=100 + e,
                          tag="widths"))
    return c


def soa_cases():
    c = []
    # bug538 (unittest.cu:101-121)
    c.append(dict(h=65538, w=2, t=2, e=4, fill="random", seed=5432,
                  tag="bug538"))
    # bug528 (unittest.cu:123-145): h=1024, t=64, w=1..99 (subset)
    for w in (1, 2, 3, 7, 16, 50, 64, 99):
        c.append(dict(h=1024, w=w, t=64, e=4, fill="random", seed=5432,
                      tag="bug528"))
    # bug537 (cl_unittest.cc:170-223): w in {197,215}, t=1..1024 (powers of 2)
    for w, hs in ((197, 35588), (215, 44609)):
        for t in (1, 2, 4, 8, 16, 32, 64, 128, 256, 512, 1024):
            h = (hs + t - 1) // t * t
            c.append(dict(h=h, w=w, t=t, e=4, fill="random", seed=11,
                          tag="bug537"))
    for e in (1, 2, 4, 8):
        for (h, w, t) in ((4096, 4, 32), (1000, 13, 8), (640, 9, 64)):
            c.append(dict(h=h, w=w, t=t, e=e, fill="random", seed=200 + e,
                          tag="widths"))
    return c


def full_cases():
    c = []
    # the 7200x1800 staged transposition and the PPoPP'14 sizes (cl_unittest.cc:386-387).
    for e in (1, 2, 4, 8):
        c.append(dict(M=7200, N=1800, e=e, fill="index", seed=0, tag="cfg2"))
    for (M, N) in ((5100, 2500), (4000, 3200), (3300, 3900), (2500, 5100),
                   (1800, 7200)):
        c.append(dict(M=M, N=N, e=4, fill="random", seed=M + N, tag="ppopp14"))
    # Python suite shapes (transpose_unittest.py:39-57, 82-94): A=40, B=37
    for a in (4, 8, 16, 32, 64):
        c.append(dict(M=40 * a, N=37 * 30, e=4, fill="random", seed=a,
                      tag="py-full"))
    c.append(dict(M=40 * 16, N=37 * 10, e=4, fill="random", seed=9,
                  tag="py-array"))
    return c


def main() -> None:
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LM_REFERENCE")
    if not ref:
        sys.exit("usage: gen_golden.py <reference-root> (or set LM_REFERENCE)")
    subprocess.check_call(["sh", os.path.join(ROOT, "oracle", "build_ref.sh"),
                           ref])
    R = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_cpu.so"))
    vp, ci = ctypes.c_void_p, ctypes.c_int
    for e, s in SUF.items():
        for pre in ("ref_cl_aos_asta_", "ref_cl_soa_asta_", "ref_cu_aos_asta_"):
            getattr(R, pre + s).argtypes = [vp, vp, ci, ci, ci]
            getattr(R, pre + s).restype = None
    R.ref_next.argtypes = [ctypes.c_uint, ci, ci]
    R.ref_next.restype = ctypes.c_uint
    R.ref_num_cycles.argtypes = [ci, ci]
    R.ref_num_cycles.restype = ctypes.c_longlong
    R.ref_tile_options.argtypes = [ci, ctypes.POINTER(ci), ci]
    R.ref_factors.argtypes = [ci, ctypes.POINTER(ci), ctypes.POINTER(ci), ci]

    out = {"source": "reference CPU code via oracle/build_ref.sh",
           "aos_asta": [], "soa_asta": [], "full": [], "num_cycles": [],
           "next": [], "tile_options": [], "factors": []}

    for c in aos_cases():
        n = c["h"] * c["w"]
        src = make_input(c["fill"], n, c["e"], c["seed"])
        dst = np.zeros_like(src)
        getattr(R, "ref_cl_aos_asta_" + SUF[c["e"]])(src.ctypes.data,
                                                     dst.ctypes.data,
                                                     c["h"], c["w"], c["t"])
        dst2 = np.zeros_like(src)
        getattr(R, "ref_cu_aos_asta_" + SUF[c["e"]])(src.ctypes.data,
                                                     dst2.ctypes.data,
                                                     c["h"], c["w"], c["t"])
        assert (dst == dst2).all(), "the two reference aos_asta disagree"
        c["sha256"] = digest(dst)
        out["aos_asta"].append(c)

    for c in soa_cases():
        n = c["h"] * c["w"]
        src = make_input(c["fill"], n, c["e"], c["seed"])
        dst = np.zeros_like(src)
        getattr(R, "ref_cl_soa_asta_" + SUF[c["e"]])(src.ctypes.data,
                                                     dst.ctypes.data,
                                                     c["h"], c["w"], c["t"])
        c["sha256"] = digest(dst)
        out["soa_asta"].append(c)

    for c in full_cases():
        M, N, e = c["M"], c["N"], c["e"]
        src = make_input(c["fill"], M * N, e, c["seed"])
        tmp = np.zeros_like(src)
        dst = np.zeros_like(src)
        # golden of the reference's full test (cl_unittest.cc:549-552)
        getattr(R, "ref_cl_aos_asta_" + SUF[e])(src.ctypes.data,
                                                tmp.ctypes.data, M, N, 1)
        getattr(R, "ref_cl_soa_asta_" + SUF[e])(tmp.ctypes.data,
                                                dst.ctypes.data, N, M, 1)
        c["sha256"] = digest(dst)
        out["full"].append(c)

    pairs = [(m, n) for m in range(1, 13) for n in range(1, 13)]
    pairs += [(2, 3), (3, 5), (37, 40), (64, 27), (100, 72), (197, 35),
              (512, 241), (1024, 33)]
    for m, n in pairs:
        out["num_cycles"].append([m, n, int(R.ref_num_cycles(m, n))])
    # Next with 32-bit wrap-around (i*m overflows for large shapes).
    rng = np.random.default_rng(1)
    for (m, n) in ((16384, 12289), (32768, 16000), (4, 1 << 22), (7, 65536),
                   (65536, 7), (12289, 16384)):
        for i in rng.integers(0, m * n, size=16).tolist() + [0, m * n - 1, 1]:
            out["next"].append([int(i), m, n, int(R.ref_next(int(i), m, n))])
    ns = list(range(1, 130)) + [360, 1000, 1800, 7200, 12289, 12290, 12291,
                                16000, 16384, 32768, 65536, 44609, 35588,
                                5100, 2500, 3300, 3900]
    buf = (ctypes.c_int * 8192)()
    P = (ctypes.c_int * 64)()
    E = (ctypes.c_int * 64)()
    for n in ns:
        k = R.ref_tile_options(n, buf, 8192)
        out["tile_options"].append([n, [buf[i] for i in range(k)]])
        k = R.ref_factors(n, P, E, 64)
        out["factors"].append([n, [[P[i], E[i]] for i in range(k)]])

    with open(OUT, "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print("wrote", OUT, "aos", len(out["aos_asta"]), "soa",
          len(out["soa_asta"]), "full", len(out["full"]))


if __name__ == "__main__":
    main()
