"""Compression on the GPU.

* ``d2gep`` compresses a dense float64 matrix into a host PLR tree through
  the library's ``dplr_gpu_d2gep`` (dplrd2gep, src/dplrd2p.c:186): one
  truncated SVD per off-diagonal block (a verified sketch for large blocks,
  else cuSOLVER gesvd), the blocks spread over ``workers`` streams.
* ``reduce_svd`` recompresses a PLR tree's low-rank blocks by truncated
  SVDs (``dplr_gpu_reduce_svd``), the alternative to dplrreduce's
  Gram-Schmidt, with dplrreduce's thresholds (eps/4 per level).
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


def reduce_svd(t, eps: float, workers: int = 0):
    """The tree ``t`` with every low-rank block replaced by its SVD truncated
    below the block's threshold (eps/4 per level); a new tree."""
    lib = _native.lib()
    c = tree.to_c(t)
    try:
        _native.check(lib.dplr_gpu_reduce_svd(t.size, c, eps, workers), "dplr_gpu_reduce_svd")
        return tree.from_c(c)
    finally:
        tree.free_c(c)
