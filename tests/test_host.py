"""Host-side checks that need no GPU: the C ABI library builds, loads and
exports every symbol include/*.h declares; the division helper used by every
kernel; the Python API's host logic."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = set()
    for h in ("marshal.h", "lm_marshal.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\**\s*(\w+)\s*\(",
                             text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_reference_surface():
    names = header_functions()
    # include/marshal.h:26-31 of the reference
    for n in ("gpu_aos_asta_bs_float", "gpu_aos_asta_bs_double",
              "gpu_aos_asta_pttwac", "gpu_soa_asta_pttwac"):
        assert n in names
    # include/cl_marshal.h:26-49 of the reference, lm_ prefix
    for n in ("aos_asta_bs", "aos_asta_pttwac", "aos_asta", "transpose",
              "transpose_010_bs", "transpose_010_pttwac", "transpose_100",
              "transpose_0100", "padding", "unpadding"):
        assert "lm_" + n in names
    assert "cl_marshal_finalize" in names


def test_library_exports_every_declared_symbol(built):
    from libmarshal_gb300 import lm
    L = lm.lib()
    for name in header_functions():
        assert hasattr(L, name), name
    assert set(header_functions()) <= set(lm.exported_symbols())
    assert b"sm_103a" in L.lm_version()


def test_library_reports_errors_without_a_gpu_call(built):
    # argument validation happens before any CUDA call
    from libmarshal_gb300 import lm
    L = lm.lib()
    assert L.lm_aos_asta_bs(None, None, 4, 10, 3, 4) is True
    assert "multiple" in lm.last_error()
    assert L.lm_transpose_100(None, None, 3, 4, 5, 1, None) is True
    assert "element size" in lm.last_error()
    # a 4-byte element at an odd address is refused before any launch
    assert L.lm_transpose_100(None, 0x1002, 4, 4, 5, 1, None) is True
    assert "aligned" in lm.last_error()
    assert L.lm_transpose_100_noalloc(None, 0x1004, 8, 4, 5, 1) is True
    assert "aligned" in lm.last_error()
    assert L.lm_padding(None, 0x1001, 2, 3, 4, 5, None) is True
    assert "aligned" in lm.last_error()
    # method codes 0..7 (7: held in shared memory); others refused
    assert L.lm_transpose_0100_method(None, 0x1000, 4, 1, 4, 5, 1, 8,
                                      None) is True
    assert "0..7" in lm.last_error()
    assert L.lm_debug_resident_stall(None, 0x1002, 4, 1, 4, 5, 1, 1000) is True
    assert "aligned" in lm.last_error()
    assert L.lm_debug_resident_stall(None, 0x1000, 4, 1, 1, 5, 1, 1000) is True
    assert "dimensions" in lm.last_error()


def _fastdiv(d):
    l = 0
    while l < 32 and (1 << l) < d:
        l += 1
    m = ((1 << 32) * ((1 << l) - d)) // d + 1
    return m & 0xffffffff, l


def test_fastdiv_formula():
    # Python restatement of lm::make_fastdiv / lm::fdiv (lm_core.cuh)
    rng = np.random.default_rng(0)
    ds = [1, 2, 3, 5, 7, 31, 32, 33, 100, 12289, 16384, 65537, 2**31 - 1,
          2**31, 2**31 + 1, 2**32 - 1] + [int(v) for v in
                                          rng.integers(1, 2**32, size=200)]
    ns = [0, 1, 2**31 - 1, 2**31, 2**32 - 1] + [int(v) for v in
                                                rng.integers(0, 2**32,
                                                             size=300)]
    for d in ds:
        m, s = _fastdiv(d)
        assert m < 2**32
        for n in ns + [d - 1, d, d + 1, (2**32 - 1) // d * d]:
            if not 0 <= n < 2**32:
                continue
            hi = (n * m) >> 32
            assert (hi + n) >> s == n // d, (n, d)


def test_python_api_host_logic():
    from libmarshal_gb300 import Transposition, TransposeArrayInPlace
    from oracle import lm_oracle as O
    for m, n in ((2, 3), (3, 5), (7, 4), (12, 9)):
        t = Transposition(m, n)
        assert t.GetNumCycles() == O.num_cycles(m, n)
        for i in range(m * n):
            assert t.Next(i) == O.next_index(i, m, n)
    torch = pytest.importorskip("torch")
    with pytest.raises(TypeError):
        TransposeArrayInPlace(torch.zeros(2, 3, 4))
    with pytest.raises(TypeError):
        TransposeArrayInPlace(torch.zeros(10, 9), a=3, b=1)


def test_cl_compat_header_compiles_and_links(built, tmp_path):
    """A C program written against the reference's cl_* names builds with
    include/cl_marshal_compat.h and links against the library; it only
    exercises argument checks (no device needed)."""
    import shutil
    import subprocess
    from libmarshal_gb300 import lm
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "uses_cl.c"
    src.write_text(r"""
#include <stdio.h>
#include "cl_marshal_compat.h"
int main(void) {
  cl_ulong et = 0;
  /* element size and divisibility are checked before any device work */
  int e1 = cl_aos_asta_bs(NULL, NULL, 10, 3, 4);           /* 10 % 4 != 0 */
  int e2 = cl_transpose_100(NULL, (cl_mem)0x1002, 4, 5, 1, NULL); /* misaligned */
  (void)et;
  printf("%d %d %s\n", e1, e2, lm_last_error());
  cl_marshal_finalize();
  return (e1 && e2) ? 0 : 1;
}
""")
    exe = tmp_path / "uses_cl"
    libdir = os.path.dirname(lm.LIB_PATH)
    subprocess.check_call([cc, "-std=c99", str(src), "-I",
                           os.path.join(root, "include"), "-L", libdir,
                           "-llmarshal", "-Wl,-rpath," + libdir, "-o",
                           str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "aligned" in out.stdout
