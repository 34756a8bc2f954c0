"""Build liblmarshal.so (the CUDA library behind the C ABI) in-tree.

    python -m libmarshal_gb300.build            # or __graft_entry__.build()

Compiles every csrc/*.cu for sm_103a only (one -gencode, no PTX for other
architectures), in parallel, and links libmarshal_gb300/_lib/liblmarshal.so
with the static CUDA runtime.  No cmake; a minute or less on either host.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB_PATH = os.path.join(LIB_DIR, "liblmarshal.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-Wall", "-I", os.path.join(HERE, "..",
                                                             "include")]


def _deps_newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = (glob.glob(os.path.join(CSRC, "*.cuh")) +
               glob.glob(os.path.join(CSRC, "*.h")) +
               glob.glob(os.path.join(HERE, "..", "include", "*.h")))
    cc = nvcc()
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _deps_newer(obj, [src] + headers):
            jobs.append([cc] + _flags() + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs),
                                                   os.cpu_count() or 4)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True,
                              text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose or r.returncode:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode:
                    raise RuntimeError("nvcc failed: " + " ".join(j))
    if force or jobs or _deps_newer(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        r = subprocess.run([cc] + ARCH + ["-shared", "-o", tmp] + objs +
                           ["-lcudart_static", "-lrt", "-lpthread", "-ldl"],
                           capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
