"""ctypes signatures of the DPLR C interface (include/dplr.h).

``bind_plr_api(lib, prefix)`` attaches argument/return types to a loaded
shared library that exports the DPLR entry points under ``prefix`` +
name: ``"dplr"`` for libdplr_gb300.so (and for DPLR's own objects built
as a shared library), ``"orc_"`` for the CPU oracle.  The returned
``PlrApi`` converts numpy arguments to the raw pointers the C functions
take and keeps DPLR's calling convention (scalars by pointer, column-major
arrays, leading dimensions and increments).
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char, c_double, c_int, c_long

import numpy as np

from .tree import PDPlrMtx, c_double_p

_SIGNATURES = {
    "ini": (None, [PDPlrMtx]),
    "clr": (None, [PDPlrMtx]),
    "inid": (None, [c_int, PDPlrMtx]),
    "inilr": (None, [c_int, PDPlrMtx, c_int]),
    "inih": (None, [c_int, PDPlrMtx]),
    "resizelr": (None, [PDPlrMtx, c_int]),
    "nz": (c_long, [c_int, PDPlrMtx]),
    "rnk": (None, [c_int, PDPlrMtx, POINTER(c_int)]),
    "gep2d": (None, [c_int, PDPlrMtx, c_double_p, c_int]),
    "gepmv": (None, [c_char, c_int, POINTER(c_double), PDPlrMtx, c_double_p, c_int,
                     POINTER(c_double), c_double_p, c_int]),
    "gepdmm": (None, [c_char, c_char, c_int, c_int, POINTER(c_double), PDPlrMtx, c_double_p,
                      c_int, POINTER(c_double), c_double_p, c_int]),
    "geprk": (None, [c_int, c_int, POINTER(c_double), c_double_p, c_int, c_double_p, c_int,
                     c_double_p, c_int, PDPlrMtx, c_double]),
    "geinv": (None, [c_int, PDPlrMtx, PDPlrMtx, c_double, POINTER(c_int)]),
    "reduce": (None, [c_int, PDPlrMtx, c_double]),
    "cpy": (None, [c_int, PDPlrMtx, PDPlrMtx]),
    "scal": (None, [c_int, POINTER(c_double), PDPlrMtx]),
    "axpy": (None, [c_int, POINTER(c_double), PDPlrMtx, PDPlrMtx]),
    "adpy": (None, [c_int, POINTER(c_double), c_double_p, PDPlrMtx]),
    "d2gep": (None, [c_int, c_double_p, c_int, PDPlrMtx, c_double, c_int, POINTER(c_int)]),
    "geppmm": (None, [c_char, c_char, c_int, POINTER(c_double), PDPlrMtx, PDPlrMtx,
                      POINTER(c_double), PDPlrMtx, c_double]),
}


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    if a.dtype != np.float64:
        raise TypeError("float64 array required")
    return a.ctypes.data_as(c_double_p)


class PlrApi:
    """Typed wrappers over one library's DPLR entry points."""

    def __init__(self, lib: ctypes.CDLL, prefix: str):
        self.lib = lib
        self.fn = {}
        for name, (res, args) in _SIGNATURES.items():
            try:
                f = getattr(lib, prefix + name)
            except AttributeError:
                continue
            f.restype, f.argtypes = res, args
            self.fn[name] = f

    def has(self, name: str) -> bool:
        return name in self.fn

    # structure ------------------------------------------------------------
    def nz(self, m: int, a) -> int:
        return int(self.fn["nz"](m, a))

    def rnk(self, m: int, a, nlvl: int) -> list[int]:
        buf = (c_int * max(nlvl, 1))(*([-1] * max(nlvl, 1)))
        self.fn["rnk"](m, a, buf)
        return list(buf)[:nlvl]

    def gep2d(self, m: int, a, ldb: int | None = None) -> np.ndarray:
        ldb = m if ldb is None else ldb
        out = np.zeros((ldb, m), order="F")
        self.fn["gep2d"](m, a, _ptr(out), ldb)
        return out[:m]

    # hot path -------------------------------------------------------------
    def gepmv(self, trans: str, m: int, alpha: float, a, x: np.ndarray, incx: int,
              beta: float, y: np.ndarray, incy: int) -> None:
        self.fn["gepmv"](trans.encode(), m, c_double(alpha), a, _ptr(x), incx,
                         c_double(beta), _ptr(y), incy)

    def gepdmm(self, transa: str, transb: str, m: int, n: int, alpha: float, a,
               b: np.ndarray, ldb: int, beta: float, c: np.ndarray, ldc: int) -> None:
        self.fn["gepdmm"](transa.encode(), transb.encode(), m, n, c_double(alpha), a, _ptr(b),
                          ldb, c_double(beta), _ptr(c), ldc)

    def geprk(self, m: int, k: int, alpha: float, u: np.ndarray, ldu: int, v: np.ndarray,
              ldv: int, s: np.ndarray, incs: int, a, eps: float) -> None:
        self.fn["geprk"](m, k, c_double(alpha), _ptr(u), ldu, _ptr(v), ldv, _ptr(s), incs, a,
                         eps)

    def geinv(self, m: int, a, b, eps: float) -> int:
        info = c_int(-12345)
        self.fn["geinv"](m, a, b, eps, ctypes.byref(info))
        return info.value

    def reduce(self, m: int, a, eps: float) -> None:
        self.fn["reduce"](m, a, eps)

    # structure-level arithmetic --------------------------------------------
    def cpy(self, m: int, a, b) -> None:
        self.fn["cpy"](m, a, b)

    def scal(self, m: int, alpha: float, a) -> None:
        self.fn["scal"](m, ctypes.byref(c_double(alpha)), a)

    def axpy(self, m: int, alpha: float, a, b) -> None:
        self.fn["axpy"](m, ctypes.byref(c_double(alpha)), a, b)

    def adpy(self, m: int, alpha: float, d: np.ndarray, b) -> None:
        self.fn["adpy"](m, ctypes.byref(c_double(alpha)), _ptr(d), b)

    def geppmm(self, transa: str, transb: str, m: int, alpha: float, a, b, beta: float, c,
               eps: float) -> None:
        self.fn["geppmm"](transa.encode(), transb.encode(), m, ctypes.byref(c_double(alpha)), a, b,
                          ctypes.byref(c_double(beta)), c, eps)

    # dense -> PLR compression ---------------------------------------------
    def d2gep(self, m: int, a: np.ndarray, lda: int, b, eps: float, nlvl: int) -> int:
        """a: the column-major dense matrix, flat or 2-D Fortran-ordered."""
        info = c_int(-12345)
        flat = a.reshape(-1, order="F") if a.ndim == 2 else a
        self.fn["d2gep"](m, _ptr(flat), lda, b, eps, nlvl, ctypes.byref(info))
        return info.value
