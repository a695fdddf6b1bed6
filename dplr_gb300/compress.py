"""Dense -> PLR compression on the GPU (dplrd2gep, src/dplrd2p.c:186).

``d2gep`` compresses a dense float64 matrix into a host PLR tree through
the library's ``dplr_gpu_d2gep``: one truncated SVD (cuSOLVER gesvd) per
off-diagonal block, the blocks spread over ``workers`` streams.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native, tree


def d2gep(a: np.ndarray, eps: float, nlvl: int, workers: int = 0):
    """PLR tree of the square matrix ``a`` with ``nlvl`` levels and absolute
    accuracy ``eps`` (the thresholds of dplrd2gep)."""
    a = np.asfortranarray(a, dtype=np.float64)
    m = a.shape[0]
    if a.ndim != 2 or a.shape[1] != m:
        raise ValueError("square matrix required")
    lib = _native.lib()
    b = tree.new_empty()
    info = ctypes.c_int(-12345)
    try:
        rc = lib.dplr_gpu_d2gep(m, a.ctypes.data, m, b, eps, nlvl, workers, ctypes.byref(info))
        _native.check(rc, "dplr_gpu_d2gep")
        if info.value != 0:
            raise _native.NativeError(f"dplrd2gep: info = {info.value}")
        return tree.from_c(b)
    finally:
        tree.free_c(b)
