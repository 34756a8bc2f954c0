"""libmarshal_gb300 -- in-place data-layout conversion on one GB300 (sm_103a).

The product is liblmarshal.so (hand-written CUDA kernels behind a C ABI,
declared in include/marshal.h and include/lm_marshal.h).  This package holds
its sources (csrc/), its build step (build.py), the ctypes binding (lm.py)
and the Python API of the reference's binding (transpose.py).
"""
from . import lm  # noqa: F401
from .lm import LMError  # noqa: F401
from .transpose import (FullTranspose, T010_BS, T0100, T100,  # noqa: F401
                        Transposition, TransposeArrayInPlace)

__all__ = ["lm", "LMError", "Transposition", "T010_BS", "T100", "T0100",
           "FullTranspose", "TransposeArrayInPlace"]
