"""Python handle on the CPU oracle (test infrastructure only).

Loads ``oracle/_build/liboracle.so`` (the C restatement linked to an
optimised BLAS) or ``liboracle_loops.so`` (plain loops), and, where it was
built, ``oracle/_ref/libdplr_ref.so`` (the reference's own C sources).
Only tests, the smoke check and the benchmark's CPU leg import this.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from dplr_gb300.capi import PlrApi  # noqa: E402
from dplr_gb300.tree import c_double_p  # noqa: E402

_cache: dict = {}


def _build_if_missing(path: str) -> None:
    if not os.path.exists(path):
        from oracle.build_oracle import build_oracle
        build_oracle()


def oracle(kind: str = "best") -> PlrApi:
    """The C restatement; kind = 'best' (BLAS if available), 'blas', 'loops'."""
    blas = os.path.join(HERE, "_build", "liboracle.so")
    loops = os.path.join(HERE, "_build", "liboracle_loops.so")
    _build_if_missing(loops)
    if kind == "best":
        path = blas if os.path.exists(blas) else loops
    else:
        path = blas if kind == "blas" else loops
    if path not in _cache:
        lib = ctypes.CDLL(path)
        api = PlrApi(lib, "orc_")
        f = lib.orc_dortlr
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int, ctypes.c_int, c_double_p, c_double_p, ctypes.c_int,
                      c_double_p, ctypes.c_double, ctypes.c_int]
        lib.orc_error_count.restype = ctypes.c_long
        lib.orc_set_threads.argtypes = [ctypes.c_int]
        lib.orc_blas_optimised.restype = ctypes.c_int
        lib.orc_inverse_shape.restype = ctypes.c_int
        lib.orc_inverse_shape.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double]
        lib.orc_resid_dd.restype = ctypes.c_int
        lib.orc_resid_dd.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, c_double_p,
                                     ctypes.c_int, c_double_p, ctypes.c_int, c_double_p,
                                     c_double_p, ctypes.c_int]
        api.path = path
        _cache[path] = api
    return _cache[path]


def dortlr(api: PlrApi, u: np.ndarray, v: np.ndarray, sval: np.ndarray, eps: float,
           niter: int = 1) -> int:
    """In-place Gram-Schmidt recompression of u diag(sval) v^T; returns rank."""
    for a in (u, v, sval):
        if a.dtype != np.float64 or not a.flags.f_contiguous:
            raise ValueError("float64 Fortran-ordered arrays required")
    return api.lib.orc_dortlr(u.shape[0], v.shape[0], u.ctypes.data_as(c_double_p),
                              v.ctypes.data_as(c_double_p), u.shape[1],
                              sval.ctypes.data_as(c_double_p), eps, niter)


def resid_dd(api: PlrApi, cptr, x: np.ndarray, b: np.ndarray, threads: int | None = None):
    """Per column j of x, b (arrays of shape (ncols, m), row j = column j):
    (||b_j - A x_j||, || |A||x_j| ||) with A x_j evaluated in double-double
    arithmetic on the tree `cptr` (a DPlrMtx pointer)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    if x.shape != b.shape or x.ndim != 2:
        raise ValueError("x and b must be (ncols, m) arrays of the same shape")
    nc, m = x.shape
    rn, an = np.zeros(nc), np.zeros(nc)
    rc = api.lib.orc_resid_dd(m, ctypes.cast(cptr, ctypes.c_void_p), nc, x.ctypes.data_as(c_double_p), m,
                              b.ctypes.data_as(c_double_p), m, rn.ctypes.data_as(c_double_p),
                              an.ctypes.data_as(c_double_p), int(threads or os.cpu_count() or 1))
    if rc != 0:
        raise RuntimeError("orc_resid_dd failed")
    return rn, an


def error_count(api: PlrApi) -> int:
    return int(api.lib.orc_error_count())


def set_threads(api: PlrApi, n: int) -> None:
    api.lib.orc_set_threads(int(n))


def reference() -> PlrApi | None:
    """The reference's own C sources (built only where they are present)."""
    path = os.path.join(HERE, "_ref", "libdplr_ref.so")
    if not os.path.exists(path):
        return None
    if path not in _cache:
        try:
            lib = ctypes.CDLL(path)
        except OSError:
            return None
        api = PlrApi(lib, "dplr")
        api.path = path
        _cache[path] = api
    return _cache[path]
