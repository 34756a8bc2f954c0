"""Python API of libmarshal (src/py/transpose.py of the reference) on PyTorch.

Same classes and functions with the same meaning:

  Transposition(m, n)          .Next(i), .GetNumCycles()     (transpose.py:4-29)
  T010_BS(A, a, B)             .IsFeasible(buf), .Transpose(stream, buf),
  T100(A, B, b)                .Throughput()                  (transpose.py:31-87)
  T0100(A, a, B, b)
  FullTranspose(stream, buf, A, a, B, b)                      (transpose.py:89-105)
  TransposeArrayInPlace(arr, a=1, b=1)                        (transpose.py:108-116)

The reference's first argument is a PyOpenCL queue and buffers are cl.Buffer /
pyopencl.array; here the queue is a ``torch.cuda.Stream`` (or None for the
current stream) and buffers / arrays are contiguous CUDA tensors.  The work
runs through liblmarshal.so's C ABI; the reference's binding loaded its
OpenCL kernels directly (src/py/basic.py) and no longer matches them.

Throughput() reports GB/s as 2 x bytes / kernel time, the reference's measure,
with the real element size (the reference hard-codes 4 bytes).
"""
from __future__ import annotations

from . import lm


class Transposition:
    """Transposition of an m x n row-major matrix (include/plan.hpp:48-92)."""

    def __init__(self, mm, nn):
        self.m = mm
        self.n = nn
        self.nr_cycles = -1  # number of non-trivial cycles

    def Next(self, i):
        # Successor of position i (integer division, as the Python 2 original)
        return i * self.m - (self.m * self.n - 1) * (i // self.n)

    def GetNumCycles(self):
        if self.nr_cycles >= 0:
            return self.nr_cycles
        self.nr_cycles = 0
        for i in range(1, self.m * self.n):
            j = self.Next(i)
            if j == i:
                continue
            while j > i:
                j = self.Next(j)
            if j != i:
                continue
            self.nr_cycles += 1
        return self.nr_cycles

    def IsFeasible(self, buf=None):
        return False


class _Timed:
    def _record(self, stream, fn):
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        self._start = torch.cuda.Event(enable_timing=True)
        self._end = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(s):
            self._start.record(s)
            fn(s)
            self._end.record(s)
        return self

    def Throughput(self):
        """GB/s = 2 x payload bytes / elapsed ns (waits for the kernel)."""
        self._end.synchronize()
        ns = self._start.elapsed_time(self._end) * 1.0e6
        return float(self._bytes * 2) / ns if ns > 0 else float("inf")


class T010_BS(Transposition, _Timed):
    """[A][a][B] -> [A][B][a] by on-chip tiles (transpose.py:31-48)."""

    def __init__(self, AA, aa, BB):
        Transposition.__init__(self, aa, BB)
        self.A, self.a, self.B = AA, aa, BB

    def IsFeasible(self, buf):
        return lm.bs_feasible(self.A, self.a, self.B, 1, buf.element_size())

    def Transpose(self, stream, buf):
        self._bytes = self.A * self.a * self.B * buf.element_size()
        return self._record(stream, lambda s: lm.transpose_010_bs(
            buf, self.A, self.a, self.B, stream=s))


class T100(Transposition, _Timed):
    """[A][B][b] -> [B][A][b] (transpose.py:50-67)."""

    def __init__(self, AA, BB, bb):
        Transposition.__init__(self, AA, BB)
        self.A, self.B, self.b = AA, BB, bb

    def IsFeasible(self, buf):
        # Any super-element size works here (large ones are sliced).
        return self.A > 0 and self.B > 0 and self.b > 0

    def Transpose(self, stream, buf):
        self._bytes = self.A * self.B * self.b * buf.element_size()
        return self._record(stream, lambda s: lm.transpose_100(
            buf, self.A, self.B, self.b, stream=s))


class T0100(Transposition, _Timed):
    """[A][a][B][b] -> [A][B][a][b] (transpose.py:69-87)."""

    def __init__(self, AA, aa, BB, bb):
        Transposition.__init__(self, aa, BB)
        self.A, self.a, self.B, self.b = AA, aa, BB, bb

    def IsFeasible(self, buf):
        return self.A > 0 and self.a > 0 and self.B > 0 and self.b > 0

    def Transpose(self, stream, buf):
        self._bytes = self.A * self.a * self.B * self.b * buf.element_size()
        return self._record(stream, lambda s: lm.transpose_0100(
            buf, self.A, self.a, self.B, self.b, stream=s))


def FullTranspose(stream, buf, A, a, B, b):
    """In-place [A*a][B*b] -> [B*b][A*a]: the three-step plan
    100 -> 010 -> 0100 when feasible, else the element-wise fallback
    (transpose.py:89-105)."""
    method2a = T100(A * a, B, b)       # AaBb -> BAab
    method2b = T010_BS(B * A, a, b)    # BAab -> BAba
    method2c = T0100(B, A, b, a)       # BAba -> BbAa
    if (method2a.IsFeasible(buf) and method2b.IsFeasible(buf)
            and method2c.IsFeasible(buf)):
        method2a.Transpose(stream, buf)
        method2b.Transpose(stream, buf)
        method2c.Transpose(stream, buf)
        return [method2a, method2b, method2c]
    fallback = T0100(1, A * a, B * b, 1)
    fallback.Transpose(stream, buf)
    return [fallback]


def TransposeArrayInPlace(arr, a=1, b=1):
    """Transpose a 2-D CUDA tensor in place; returns the (N, M) view of the
    same storage (transpose.py:108-116)."""
    if arr.dim() != 2:
        raise TypeError("only allows transposing 2D arrays")
    if arr.shape[0] % a != 0 or arr.shape[1] % b != 0:
        raise TypeError("tile size must evenly divide array dimensions")
    if not arr.is_contiguous():
        raise TypeError("array must be contiguous")
    FullTranspose(None, arr, arr.shape[0] // a, a, arr.shape[1] // b, b)
    return arr.view(arr.shape[1], arr.shape[0])
