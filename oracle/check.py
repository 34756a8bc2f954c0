"""Threaded per-job checking against the oracle for mixed job lists.

TEST INFRASTRUCTURE ONLY: the checker behind tests/ and behind bench.py's
verification passes (which run outside every timed region).  The product
package ``libmarshal_gb300`` never imports this module.

Each job is one layout conversion of the library's op table
(include/lm_marshal.h, LM_OP_*) on a contiguous region of elem_bytes-wide
elements.  ``expected`` maps it onto the oracle's restatements of the
reference's CPU layouts:

  AoS -> ASTA  [h][w] -> [h/t][w][t]     cpu_aos_asta (test/cl_unittest.cc:138-151)
  SoA -> ASTA  [w][h] -> [h/t][w][t]     cpu_soa_asta (test/cl_unittest.cc:153-166)
  ASTA -> AoS  = 010(h/t, w, t)          cpu_aos_asta with h = h/t*w, w = t, t = w
  ASTA -> SoA  = 100(h/t, w, t)          cpu_soa_asta with h = w*t, w = h/t, t = t
  transpose    [M][N] -> [N][M]          the full-transpose golden (:549-552)
  010 / 100 / 0100                       oracle/lm_oracle.h

Inputs are splitmix64 bytes seeded per job, so a job's input can be
regenerated anywhere without keeping a copy.  ctypes calls release the GIL,
so a thread pool spreads the oracle over the host cores.
"""
from __future__ import annotations

import concurrent.futures as cf
import os

import numpy as np

from oracle import lm_oracle as O

OP_0100, OP_010, OP_100, OP_AOS_ASTA, OP_ASTA_AOS, OP_SOA_ASTA, \
    OP_ASTA_SOA, OP_TRANSPOSE = range(8)


def n_elems(op: int, dims) -> int:
    d = list(dims) + [0] * (4 - len(dims))
    if op == OP_0100:
        return d[0] * d[1] * d[2] * d[3]
    if op in (OP_010, OP_100):
        return d[0] * d[1] * d[2]
    if op == OP_TRANSPOSE:
        return d[0] * d[1]
    return d[0] * d[1]  # height x width


def expected(op: int, dims, src: np.ndarray) -> np.ndarray:
    """The oracle's output for one job; src is the job's input elements."""
    d = list(dims) + [0] * (4 - len(dims))
    if op == OP_AOS_ASTA:
        return O.aos_asta(src, d[0], d[1], d[2])
    if op == OP_SOA_ASTA:
        return O.soa_asta(src, d[0], d[1], d[2])
    if op == OP_ASTA_AOS:
        return O.t010(src, d[0] // d[2], d[1], d[2])
    if op == OP_ASTA_SOA:
        return O.t100(src, d[0] // d[2], d[1], d[2])
    if op == OP_TRANSPOSE:
        return O.transpose(src, d[0], d[1])
    if op == OP_010:
        return O.t010(src, d[0], d[1], d[2])
    if op == OP_100:
        return O.t100(src, d[0], d[1], d[2])
    if op == OP_0100:
        return O.t0100(src, d[0], d[1], d[2], d[3])
    raise ValueError("unknown op %d" % op)


def job_input(nelem: int, e: int, seed: int) -> np.ndarray:
    return O.random_bits(nelem, e, seed)


def threads() -> int:
    return max(1, os.cpu_count() or 1)


def pool() -> cf.ThreadPoolExecutor:
    return cf.ThreadPoolExecutor(max_workers=threads())


def fill_host(host: np.ndarray, jobs, seed0: int) -> None:
    """Writes every job's input into its byte range of `host` (uint8), job k
    seeded seed0 + k.  jobs: (offset_bytes, op, dims, elem_bytes)."""
    def one(k):
        off, op, dims, e = jobs[k]
        n = n_elems(op, dims)
        view = host[off:off + n * e]
        O.lib().lmo_fill_splitmix64(view.ctypes.data, view.nbytes, seed0 + k)
    with pool() as ex:
        list(ex.map(one, range(len(jobs))))


def check_host(host: np.ndarray, jobs, seed0: int):
    """Compares every job's bytes in `host` (uint8, after the conversion)
    with the oracle applied to its regenerated input.  Returns the list of
    indices that differ."""
    def one(k):
        off, op, dims, e = jobs[k]
        n = n_elems(op, dims)
        src = job_input(n, e, seed0 + k)
        want = expected(op, dims, src)
        got = host[off:off + n * e].view(O.DTYPES[e])
        return None if np.array_equal(got, want) else k
    with pool() as ex:
        return [k for k in ex.map(one, range(len(jobs))) if k is not None]
