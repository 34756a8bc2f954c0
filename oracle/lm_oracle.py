"""ctypes loader for the CPU oracle (oracle/lm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
as the checker, and by bench.py's CPU-baseline / reference leg.  The product
package ``libmarshal_gb300`` never imports this module.

``build()`` compiles the C restatement with gcc into ``oracle/_build``; it is
plain C (no intrinsics) so the same source builds on x86_64 and aarch64.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liblm_oracle.so")
SRC = os.path.join(HERE, "lm_oracle.c")

_lib = None


def build(force: bool = False) -> str:
    """Compile liblm_oracle.so (seconds)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(
                os.path.join(HERE, "lm_oracle.h"))):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-fPIC", "-shared", "-pthread",
                           "-std=c11", "-o", tmp, SRC, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        i64, vp, c_int = ctypes.c_int64, ctypes.c_void_p, ctypes.c_int
        for name in ("lmo_aos_asta", "lmo_soa_asta"):
            getattr(L, name).argtypes = [vp, vp, i64, i64, i64, c_int]
            getattr(L, name).restype = c_int
        for name in ("lmo_aos_asta_mt", "lmo_soa_asta_mt"):
            getattr(L, name).argtypes = [vp, vp, i64, i64, i64, c_int, c_int]
            getattr(L, name).restype = c_int
        L.lmo_010.argtypes = [vp, vp, i64, i64, i64, c_int]
        L.lmo_100.argtypes = [vp, vp, i64, i64, i64, c_int]
        L.lmo_0100.argtypes = [vp, vp, i64, i64, i64, i64, c_int]
        L.lmo_transpose.argtypes = [vp, vp, i64, i64, c_int]
        L.lmo_inplace_100.argtypes = [vp, i64, i64, i64, c_int]
        L.lmo_inplace_100.restype = i64
        L.lmo_padding.argtypes = [vp, i64, i64, i64, c_int]
        L.lmo_unpadding.argtypes = [vp, i64, i64, i64, c_int]
        L.lmo_next.argtypes = [ctypes.c_uint32, c_int, c_int]
        L.lmo_next.restype = ctypes.c_uint32
        L.lmo_num_cycles.argtypes = [c_int, c_int]
        L.lmo_num_cycles.restype = i64
        L.lmo_num_cycles_fast.argtypes = [i64, i64]
        L.lmo_num_cycles_fast.restype = i64
        ip = ctypes.POINTER(c_int)
        L.lmo_factorize.argtypes = [c_int, ip, ip, c_int]
        L.lmo_tile_options.argtypes = [c_int, ip, c_int]
        L.lmo_alg5.argtypes = [c_int, c_int, c_int, ip]
        L.lmo_alg3.argtypes = [c_int, c_int, c_int, c_int, c_int]
        L.lmo_fill_splitmix64.argtypes = [vp, i64, ctypes.c_uint64]
        L.lmo_fill_splitmix64.restype = None
        L.lmo_fill_index.argtypes = [vp, i64, c_int]
        L.lmo_fill_index.restype = None
        _lib = L
    return _lib


DTYPES = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise ValueError("oracle %s rejected its arguments" % what)


def random_bits(n_elems: int, e: int, seed: int) -> np.ndarray:
    """n_elems elements of width e filled by splitmix64(seed)."""
    a = np.empty(n_elems, dtype=DTYPES[e])
    lib().lmo_fill_splitmix64(_ptr(a), a.nbytes, seed)
    return a


def index_fill(n_elems: int, e: int) -> np.ndarray:
    """Element i holds i mod 2^(8e)."""
    a = np.empty(n_elems, dtype=DTYPES[e])
    lib().lmo_fill_index(_ptr(a), n_elems, e)
    return a


def aos_asta(src: np.ndarray, height: int, width: int, tile: int) -> np.ndarray:
    dst = np.empty_like(src)
    _check(lib().lmo_aos_asta(_ptr(src), _ptr(dst), height, width, tile,
                              src.itemsize), "aos_asta")
    return dst


def soa_asta(src: np.ndarray, height: int, width: int, tile: int) -> np.ndarray:
    dst = np.empty_like(src)
    _check(lib().lmo_soa_asta(_ptr(src), _ptr(dst), height, width, tile,
                              src.itemsize), "soa_asta")
    return dst


def t010(src: np.ndarray, A: int, a: int, B: int) -> np.ndarray:
    dst = np.empty_like(src)
    _check(lib().lmo_010(_ptr(src), _ptr(dst), A, a, B, src.itemsize), "010")
    return dst


def t100(src: np.ndarray, A: int, B: int, b: int) -> np.ndarray:
    dst = np.empty_like(src)
    _check(lib().lmo_100(_ptr(src), _ptr(dst), A, B, b, src.itemsize), "100")
    return dst


def t0100(src: np.ndarray, A: int, a: int, B: int, b: int) -> np.ndarray:
    dst = np.empty_like(src)
    _check(lib().lmo_0100(_ptr(src), _ptr(dst), A, a, B, b, src.itemsize),
           "0100")
    return dst


def transpose(src: np.ndarray, M: int, N: int) -> np.ndarray:
    dst = np.empty_like(src)
    _check(lib().lmo_transpose(_ptr(src), _ptr(dst), M, N, src.itemsize),
           "transpose")
    return dst


def inplace_100(buf: np.ndarray, A: int, B: int, b: int) -> int:
    r = lib().lmo_inplace_100(_ptr(buf), A, B, b, buf.itemsize)
    if r < 0:
        raise ValueError("oracle inplace_100 rejected its arguments")
    return r


def padding(buf: np.ndarray, x: int, y: int, pad: int) -> np.ndarray:
    out = buf.copy()
    _check(lib().lmo_padding(_ptr(out), x, y, pad, out.itemsize), "padding")
    return out


def unpadding(buf: np.ndarray, x: int, y: int, pad: int) -> np.ndarray:
    out = buf.copy()
    _check(lib().lmo_unpadding(_ptr(out), x, y, pad, out.itemsize),
           "unpadding")
    return out


def next_index(i: int, m: int, n: int) -> int:
    return lib().lmo_next(i, m, n)


def num_cycles(m: int, n: int) -> int:
    return lib().lmo_num_cycles(m, n)


def num_cycles_fast(m: int, n: int) -> int:
    return lib().lmo_num_cycles_fast(m, n)


def factorize(n: int):
    P = (ctypes.c_int * 64)()
    E = (ctypes.c_int * 64)()
    k = lib().lmo_factorize(n, P, E, 64)
    return [(P[i], E[i]) for i in range(min(k, 64))]


def tile_options(n: int):
    cap = 8192
    out = (ctypes.c_int * cap)()
    k = lib().lmo_tile_options(n, out, cap)
    return [out[i] for i in range(min(k, cap))]


def alg5(h: int, w: int, max_mem: int = 12288):
    out = (ctypes.c_int * 6)()
    if lib().lmo_alg5(h, w, max_mem, out) != 0:
        raise ValueError("alg5 did not converge")
    return tuple(out[i] for i in range(6))


def alg3(A: int, a: int, B: int, b: int, max_mem: int = 12288) -> int:
    return lib().lmo_alg3(A, a, B, b, max_mem)
