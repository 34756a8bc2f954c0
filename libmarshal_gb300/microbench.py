"""Time one layout conversion on the current GPU (the reference's tests print
the same measure: GB/s = 2 x payload bytes / kernel time,
test/cl_unittest.cc:215,279,650-657).

    python -m libmarshal_gb300.microbench OP DIMS... [--elem E] [--reps N]
                                          [--warmup W] [--method M]

OP and DIMS:
    010   A a B       lm_transpose_010_bs            (BS on-chip tiles)
    010p  A a B       lm_transpose_010_pttwac        (R=1, P=1)
    100   A B b       lm_transpose_100               (planner)
    0100  A a B b     lm_transpose_0100_method       (--method 0/1/2)
    full  A a B b S   lm_transpose, stages S

Prints one line with the average time, GB/s and the per-kernel breakdown
(launches, average ms) from the library's event profiler.  Inputs are random
bytes on the device; the op runs in place on the same buffer every rep.
"""
from __future__ import annotations

import argparse
import json
import os
import sys


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("op", choices=["010", "010p", "100", "0100", "full"])
    ap.add_argument("dims", type=int, nargs="+")
    ap.add_argument("--elem", type=int, default=4)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--method", type=int, default=0)
    args = ap.parse_args(argv)

    import torch
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    from libmarshal_gb300 import build, lm
    build.build()

    e = args.elem
    d = args.dims
    n = 1
    for v in d[:4] if args.op in ("0100", "full") else d[:3]:
        n *= v
    nbytes = n * e
    dev = torch.device("cuda:0")
    buf = torch.randint(0, 256, (max(nbytes, 1),), dtype=torch.uint8,
                        device=dev)

    def run():
        if args.op == "010":
            lm.transpose_010_bs(buf, d[0], d[1], d[2], elem_bytes=e)
        elif args.op == "010p":
            lm.transpose_010_pttwac(buf, d[0], d[1], d[2], R=1, P=1,
                                    elem_bytes=e)
        elif args.op == "100":
            lm.transpose_100(buf, d[0], d[1], d[2], elem_bytes=e)
        elif args.op == "0100":
            lm.transpose_0100(buf, d[0], d[1], d[2], d[3],
                              method=args.method, elem_bytes=e)
        else:
            lm.transpose(buf, d[0], d[1], d[2], d[3], R=1, stages=d[4],
                         elem_bytes=e)

    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    lm.prof_collect()
    lm.prof_enable(True)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.reps):
        run()
    e1.record()
    torch.cuda.synchronize()
    lm.prof_enable(False)
    ms = e0.elapsed_time(e1) / max(args.reps, 1)
    prof = lm.prof_collect()
    status = int(lm.lib().lm_device_status(None))  # non-zero: a wait timed out
    print(json.dumps({
        "op": args.op, "dims": d, "elem_bytes": e, "payload_bytes": nbytes,
        "ms": round(ms, 4), "GBps_2x": round(2 * nbytes / ms / 1e6, 1),
        "status": status,
        "kernels": {k: {"launches": v[0], "avg_ms": round(v[1] / v[0], 4)}
                    for k, v in prof.items()}}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
