"""ctypes binding of liblmarshal.so (the C ABI declared in include/*.h).

Buffers are PyTorch CUDA tensors (any dtype; the element width is the
tensor's element size unless ``elem_bytes`` is given) or raw device pointers
(ints, with ``elem_bytes`` required).  Streams are ``torch.cuda.Stream``,
raw ``cudaStream_t`` ints, or None for torch's current stream.

The library must have been built (``libmarshal_gb300.build.build()``); there
is no fallback of any kind: if the CUDA library is missing, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "liblmarshal.so")

_lib = None
_lock = threading.Lock()


class LMError(RuntimeError):
    """A libmarshal_gb300 call returned its error flag."""


# name -> (restype, argtypes)
_B = ctypes.c_bool
_I = ctypes.c_int
_LL = ctypes.c_longlong
_ULLP = ctypes.POINTER(ctypes.c_ulonglong)
_VP = ctypes.c_void_p
_SIGS = {
    "lm_last_error": (ctypes.c_char_p, []),
    "lm_version": (ctypes.c_char_p, []),
    "lm_marshal_finalize": (None, []),
    "cl_marshal_finalize": (None, []),
    "lm_aos_asta_bs": (_B, [_VP, _VP, _I, _I, _I, _I]),
    "lm_aos_asta_pttwac": (_B, [_VP, _VP, _I, _I, _I, _I, _I, _I]),
    "lm_aos_asta": (_B, [_VP, _VP, _I, _I, _I, _I, _I]),
    "lm_transpose": (_B, [_VP, _VP, _I, _I, _I, _I, _I, _I, _I, _ULLP]),
    "lm_transpose_ex": (_B, [_VP, _VP, _I, _I, _I, _I, _I, _I, _I, _I, _ULLP]),
    "lm_full_transpose_plan": (_B, [_I, _I, _I, _VP, _VP]),
    "lm_full_transpose": (_B, [_VP, _VP, _I, _I, _I, _LL, _I, _ULLP]),
    "lm_transpose_010_bs": (_B, [_VP, _VP, _I, _I, _I, _I, _ULLP]),
    "lm_transpose_010_pttwac": (_B, [_VP, _VP, _I, _I, _I, _I, _ULLP, _I, _I]),
    "lm_transpose_100": (_B, [_VP, _VP, _I, _I, _I, _I, _ULLP]),
    "lm_transpose_100_noalloc": (_B, [_VP, _VP, _I, _I, _I, _I]),
    "lm_transpose_0100": (_B, [_VP, _VP, _I, _I, _I, _I, _I, _ULLP]),
    "lm_transpose_0100_method": (_B, [_VP, _VP, _I, _I, _I, _I, _I, _I, _ULLP]),
    "lm_padding": (_B, [_VP, _VP, _I, _I, _I, _I, _ULLP]),
    "lm_unpadding": (_B, [_VP, _VP, _I, _I, _I, _I, _ULLP]),
    "lm_bs_feasible": (_I, [_LL, _I, _I, _I, _I]),
    "lm_debug_pad_stall": (_B, [_VP, _VP, _I, _I, _I, _I, _I, _LL,
                                ctypes.c_ulonglong]),
    "lm_debug_resident_stall": (_B, [_VP, _VP, _I, _I, _I, _I, _I,
                                     ctypes.c_ulonglong]),
    "lm_batch_create": (_B, [_VP]),
    "lm_batch_destroy": (None, [_VP]),
    "lm_batch_run": (_B, [_VP, _VP, _VP, _I, ctypes.c_uint]),
    "lm_batch_stats_get": (_B, [_VP, _VP]),
    "lm_batch_set_arena": (_B, [_VP, ctypes.c_ulonglong]),
    "lm_tune_entries": (_I, []),
    "lm_serve_create": (_B, [_VP, ctypes.c_ulonglong]),
    "lm_serve_submit": (_B, [_VP, _VP, _ULLP]),
    "lm_serve_poll": (_I, [_VP, _VP, _I]),
    "lm_serve_drain": (_B, [_VP, _LL]),
    "lm_serve_stats_get": (_B, [_VP, _VP]),
    "lm_serve_destroy": (None, [_VP]),
    "lm_serve_replay": (_B, [_VP, _VP, _VP, _VP, _I, ctypes.c_uint, _VP]),
    "lm_launch_count": (ctypes.c_ulonglong, []),
    "lm_device_status": (ctypes.c_uint, [_VP]),
    "lm_prof_enable": (None, [_I]),
    "lm_prof_collect": (_I, [_VP, _I]),
    "lm_prof_timeline": (_I, [_VP, _I]),
    "lm_tune_variant": (_I, [_I, _LL, _LL, _LL, _LL, _I]),
    "gpu_aos_asta_bs_float": (_B, [_VP, _I, _I, _I, _VP]),
    "gpu_aos_asta_bs_double": (_B, [_VP, _I, _I, _I, _VP]),
    "gpu_aos_asta_pttwac": (_B, [_VP, _I, _I, _I, _VP]),
    "gpu_soa_asta_pttwac": (_B, [_VP, _I, _I, _I, _VP]),
}


def lib():
    """Load liblmarshal.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise LMError(
                        "liblmarshal.so is not built (%s); run "
                        "libmarshal_gb300.build.build()" % LIB_PATH)
                L = ctypes.CDLL(LIB_PATH)
                for name, (res, args) in _SIGS.items():
                    fn = getattr(L, name)
                    fn.restype = res
                    fn.argtypes = args
                _lib = L
    return _lib


def exported_symbols():
    return sorted(_SIGS)


def last_error() -> str:
    v = lib().lm_last_error()
    return v.decode() if v else ""


def _check(failed: bool, what: str) -> None:
    if failed:
        raise LMError("%s failed: %s" % (what, last_error()))


def buf_ptr(buf, elem_bytes=None):
    """(device pointer, element bytes) of a CUDA tensor or a raw pointer."""
    if isinstance(buf, int):
        if elem_bytes is None:
            raise ValueError("elem_bytes is required with a raw pointer")
        return buf, int(elem_bytes)
    if not buf.is_cuda:
        raise ValueError("buffer must be a CUDA tensor")
    if not buf.is_contiguous():
        raise ValueError("buffer must be contiguous")
    return buf.data_ptr(), int(elem_bytes or buf.element_size())


def stream_ptr(stream=None) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class _Timer:
    def __init__(self, timed):
        self.v = ctypes.c_ulonglong(0) if timed else None

    def arg(self):
        return ctypes.byref(self.v) if self.v is not None else None

    def ns(self):
        return self.v.value if self.v is not None else None


def aos_asta_bs(buf, height, width, tile_size, stream=None, elem_bytes=None):
    p, e = buf_ptr(buf, elem_bytes)
    _check(lib().lm_aos_asta_bs(stream_ptr(stream), p, e, height, width,
                                tile_size), "lm_aos_asta_bs")


def aos_asta_pttwac(buf, height, width, tile_size, R=1, P=1, stream=None,
                    elem_bytes=None):
    p, e = buf_ptr(buf, elem_bytes)
    _check(lib().lm_aos_asta_pttwac(stream_ptr(stream), p, e, height, width,
                                    tile_size, R, P), "lm_aos_asta_pttwac")


def aos_asta(buf, height, width, tile_size, R=1, stream=None, elem_bytes=None):
    p, e = buf_ptr(buf, elem_bytes)
    _check(lib().lm_aos_asta(stream_ptr(stream), p, e, height, width,
                             tile_size, R), "lm_aos_asta")


def full_transpose_plan(M, N, elem_bytes):
    """The reference's Algorithm 5 / Algorithm 3 choice for an M x N matrix:
    ((A, a, B, b, pad_h, pad_w, stages), elements the padded flow needs)."""
    plan = (ctypes.c_int * 7)()
    need = ctypes.c_longlong()
    _check(lib().lm_full_transpose_plan(M, N, elem_bytes,
                                        ctypes.cast(plan, ctypes.c_void_p),
                                        ctypes.byref(need)),
           "lm_full_transpose_plan")
    return tuple(plan), need.value


def full_transpose(buf, M, N, variant010=0, stream=None, elem_bytes=None,
                   timed=False):
    """[M][N] -> [N][M] in place for any M, N (lm_full_transpose); buf may
    be longer than M*N (the padded flow of variant010 1 or 2 needs
    full_transpose_plan's element count)."""
    p, e = buf_ptr(buf, elem_bytes)
    cap = buf.numel() * buf.element_size() // e if hasattr(buf, "numel") \
        else M * N
    t = _Timer(timed)
    _check(lib().lm_full_transpose(stream_ptr(stream), p, e, M, N, cap,
                                   variant010, t.arg()), "lm_full_transpose")
    return t.ns()


def transpose(buf, A, a, B, b, R=1, stages=3, variant010=0, stream=None,
              elem_bytes=None, timed=False):
    p, e = buf_ptr(buf, elem_bytes)
    t = _Timer(timed)
    if variant010:
        _check(lib().lm_transpose_ex(stream_ptr(stream), p, e, A, a, B, b, R,
                                     stages, variant010, t.arg()),
               "lm_transpose_ex")
    else:
        _check(lib().lm_transpose(stream_ptr(stream), p, e, A, a, B, b, R,
                                  stages, t.arg()), "lm_transpose")
    return t.ns()


def transpose_010_bs(buf, A, a, B, stream=None, elem_bytes=None, timed=False):
    p, e = buf_ptr(buf, elem_bytes)
    t = _Timer(timed)
    _check(lib().lm_transpose_010_bs(stream_ptr(stream), p, e, A, a, B,
                                     t.arg()), "lm_transpose_010_bs")
    return t.ns()


def transpose_010_pttwac(buf, A, a, B, R=1, P=1, stream=None,
                         elem_bytes=None, timed=False):
    p, e = buf_ptr(buf, elem_bytes)
    t = _Timer(timed)
    _check(lib().lm_transpose_010_pttwac(stream_ptr(stream), p, e, A, a, B,
                                         t.arg(), R, P),
           "lm_transpose_010_pttwac")
    return t.ns()


def transpose_100(buf, A, B, b, stream=None, elem_bytes=None, timed=False):
    p, e = buf_ptr(buf, elem_bytes)
    t = _Timer(timed)
    _check(lib().lm_transpose_100(stream_ptr(stream), p, e, A, B, b, t.arg()),
           "lm_transpose_100")
    return t.ns()


def transpose_0100(buf, A, a, B, b, method=0, stream=None, elem_bytes=None,
                   timed=False):
    p, e = buf_ptr(buf, elem_bytes)
    t = _Timer(timed)
    if method:
        _check(lib().lm_transpose_0100_method(stream_ptr(stream), p, e, A, a,
                                              B, b, method, t.arg()),
               "lm_transpose_0100_method")
    else:
        _check(lib().lm_transpose_0100(stream_ptr(stream), p, e, A, a, B, b,
                                       t.arg()), "lm_transpose_0100")
    return t.ns()


def padding(buf, x_size, y_size, pad_size, stream=None, elem_bytes=None,
            timed=False):
    p, e = buf_ptr(buf, elem_bytes)
    t = _Timer(timed)
    _check(lib().lm_padding(stream_ptr(stream), p, e, x_size, y_size, pad_size,
                            t.arg()), "lm_padding")
    return t.ns()


def unpadding(buf, x_size, y_size, pad_size, stream=None, elem_bytes=None,
              timed=False):
    p, e = buf_ptr(buf, elem_bytes)
    t = _Timer(timed)
    _check(lib().lm_unpadding(stream_ptr(stream), p, e, x_size, y_size,
                              pad_size, t.arg()), "lm_unpadding")
    return t.ns()


def bs_feasible(T, a, B, b, elem_bytes) -> bool:
    return bool(lib().lm_bs_feasible(T, a, B, b, elem_bytes))


class ProfEntry(ctypes.Structure):
    """lm_prof_entry of include/lm_marshal.h."""
    _fields_ = [("name", ctypes.c_char * 48), ("launches", ctypes.c_longlong),
                ("total_ms", ctypes.c_double)]


def launch_count() -> int:
    """Kernels launched by the library since it was loaded."""
    return int(lib().lm_launch_count())


class ProfSpan(ctypes.Structure):
    """lm_prof_span of include/lm_marshal.h."""
    _fields_ = [("name", ctypes.c_char * 48), ("start_ms", ctypes.c_double),
                ("end_ms", ctypes.c_double)]


def prof_timeline():
    """[(kernel, start_ms, end_ms)] of the launches recorded since profiling
    was enabled (lm_prof_timeline), in launch order."""
    cap = 1 << 16
    arr = (ProfSpan * cap)()
    n = lib().lm_prof_timeline(ctypes.cast(arr, ctypes.c_void_p), cap)
    return [(arr[i].name.decode(), arr[i].start_ms, arr[i].end_ms)
            for i in range(min(n, cap))]


def prof_enable(on: bool = True) -> None:
    lib().lm_prof_enable(1 if on else 0)


def prof_collect():
    """{kernel name: (launches, summed device ms)} since the last collect."""
    cap = 64
    arr = (ProfEntry * cap)()
    n = lib().lm_prof_collect(ctypes.cast(arr, ctypes.c_void_p), cap)
    return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms))
            for i in range(min(n, cap))}


# ---- batched conversion ------------------------------------------------------

OP_0100, OP_010, OP_100, OP_AOS_ASTA, OP_ASTA_AOS, OP_SOA_ASTA, OP_ASTA_SOA, \
    OP_TRANSPOSE = range(8)
BATCH_GRAPH, BATCH_NO_TUNE, BATCH_NO_CLUSTER, BATCH_NO_SCRATCH = 1, 2, 4, 8


class Job(ctypes.Structure):
    """lm_job of include/lm_marshal.h."""
    _fields_ = [("buf", ctypes.c_void_p), ("elem_bytes", ctypes.c_int),
                ("op", ctypes.c_int), ("d0", ctypes.c_longlong),
                ("d1", ctypes.c_longlong), ("d2", ctypes.c_longlong),
                ("d3", ctypes.c_longlong)]


class BatchStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_ulonglong) for n in (
        "bytes", "small_bytes", "big_bytes", "large_bytes", "small_jobs",
        "big_jobs", "large_jobs", "identity", "small_items", "big_items",
        "band_bytes", "band_jobs", "band_items", "staged_bytes",
        "staged_jobs", "staged_waves")]


class Batch:
    """Owner of an lm_batch_t: run(jobs) converts every job in place."""

    def __init__(self):
        self.h = ctypes.c_void_p()
        _check(lib().lm_batch_create(ctypes.byref(self.h)), "lm_batch_create")

    def run(self, jobs, stream=None, graph=False, tune=True, cluster=True,
            scratch=True):
        arr = (Job * len(jobs))()
        for i, j in enumerate(jobs):
            arr[i] = j
        flags = ((BATCH_GRAPH if graph else 0) | (0 if tune else BATCH_NO_TUNE)
                 | (0 if cluster else BATCH_NO_CLUSTER)
                 | (0 if scratch else BATCH_NO_SCRATCH))
        _check(lib().lm_batch_run(self.h, stream_ptr(stream),
                                  ctypes.cast(arr, ctypes.c_void_p),
                                  len(jobs), flags), "lm_batch_run")

    def stats(self):
        st = BatchStats()
        _check(lib().lm_batch_stats_get(self.h, ctypes.byref(st)),
               "lm_batch_stats_get")
        return {n: getattr(st, n) for n, _ in BatchStats._fields_}

    def close(self):
        if self.h:
            lib().lm_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def job(buf, op, dims, elem_bytes=None):
    """lm_job for a CUDA tensor (or raw pointer) and up to four dims."""
    p, e = buf_ptr(buf, elem_bytes)
    d = list(dims) + [0] * (4 - len(dims))
    return Job(p, e, op, *d)


class Request(ctypes.Structure):
    """lm_request of include/lm_marshal.h."""
    _fields_ = [("elem_bytes", ctypes.c_int), ("op", ctypes.c_int),
                ("d0", ctypes.c_longlong), ("d1", ctypes.c_longlong),
                ("d2", ctypes.c_longlong), ("d3", ctypes.c_longlong),
                ("buf", ctypes.c_void_p), ("src", ctypes.c_void_p),
                ("dst", ctypes.c_void_p)]


class ServeDone(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_ulonglong), ("status", ctypes.c_int),
                ("latency_ns", ctypes.c_longlong),
                ("queue_ns", ctypes.c_longlong), ("done_ns", ctypes.c_longlong)]


SERVE_PLAIN = 1


def serve_replay(server, reqs, arrival_ns, after=None, plain=False):
    """Replays a trace (list of Request, arrival offsets in ns, optional
    dependency indices) through `server` (or alone per request with
    plain=True); returns [(status, latency_ns, queue_ns)] per request."""
    n = len(reqs)
    arr = (Request * n)(*reqs)
    t = (ctypes.c_longlong * n)(*[int(x) for x in arrival_ns])
    a = (ctypes.c_int * n)(*([-1] * n if after is None else after))
    out = (ServeDone * n)()
    h = server.h if server is not None else None
    _check(lib().lm_serve_replay(h, ctypes.cast(arr, ctypes.c_void_p),
                                 ctypes.cast(t, ctypes.c_void_p),
                                 ctypes.cast(a, ctypes.c_void_p), n,
                                 SERVE_PLAIN if plain else 0,
                                 ctypes.cast(out, ctypes.c_void_p)),
           "lm_serve_replay")
    return [(out[i].status, out[i].latency_ns, out[i].queue_ns)
            for i in range(n)]


class ServeStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_ulonglong) for n in (
        "submitted", "completed", "batches", "bytes", "peak_inflight_bytes")]


class Server:
    """Owner of an lm_serve_t (a worker thread converting submitted
    requests under an HBM budget, continuously batched)."""

    def __init__(self, budget_bytes):
        self.h = ctypes.c_void_p()
        _check(lib().lm_serve_create(ctypes.byref(self.h), int(budget_bytes)),
               "lm_serve_create")

    def submit(self, op, dims, elem_bytes=None, buf=None, src=None, dst=None):
        """In place on a device buffer (`buf`: CUDA tensor or pointer), or
        host arrays `src` -> `dst` (pinned tensors or pointers) staged through
        the server's pool.  Returns the ticket."""
        d = list(dims) + [0] * (4 - len(dims))
        r = Request()
        if buf is not None:
            p, e = buf_ptr(buf, elem_bytes)
            r.buf = p
        else:
            e = int(elem_bytes or src.element_size())
            r.src = src if isinstance(src, int) else src.data_ptr()
            r.dst = dst if isinstance(dst, int) else dst.data_ptr()
        r.elem_bytes, r.op = e, op
        r.d0, r.d1, r.d2, r.d3 = d
        t = ctypes.c_ulonglong(0)
        _check(lib().lm_serve_submit(self.h, ctypes.byref(r), ctypes.byref(t)),
               "lm_serve_submit")
        return t.value

    def poll(self, cap=4096):
        """Completed requests: [(ticket, status, latency_ns, queue_ns)]."""
        arr = (ServeDone * cap)()
        n = lib().lm_serve_poll(self.h, ctypes.cast(arr, ctypes.c_void_p), cap)
        if n < 0:
            raise LMError("lm_serve_poll: bad arguments")
        return [(arr[i].ticket, arr[i].status, arr[i].latency_ns,
                 arr[i].queue_ns) for i in range(n)]

    def drain(self, timeout_ms=-1):
        _check(lib().lm_serve_drain(self.h, int(timeout_ms)), "lm_serve_drain")

    def stats(self):
        st = ServeStats()
        _check(lib().lm_serve_stats_get(self.h, ctypes.byref(st)),
               "lm_serve_stats_get")
        return {n: getattr(st, n) for n, _ in ServeStats._fields_}

    def close(self):
        if self.h:
            lib().lm_serve_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def finalize() -> None:
    lib().lm_marshal_finalize()
