"""Loader for libdplr_gb300.so (the CUDA library behind the C ABI).

There is no fallback: if the library is missing or cannot be loaded, every
entry point raises, so a GPU run can never silently use another path.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char, c_double, c_int, c_longlong, c_void_p

from .capi import PlrApi
from .tree import PDPlrMtx, c_double_p

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libdplr_gb300.so")

_lib = None
_api = None


class NativeError(RuntimeError):
    pass


def _bind(lib: ctypes.CDLL) -> None:
    def sig(name, res, args):
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args

    sig("dplr_gpu_last_error", ctypes.c_char_p, [])
    sig("dplr_gpu_plan_create", c_int, [c_int, PDPlrMtx, c_void_p, POINTER(c_void_p)])
    sig("dplr_gpu_plan_destroy", None, [c_void_p])
    sig("dplr_gpu_plan_refresh", c_int, [c_void_p, PDPlrMtx, c_void_p])
    sig("dplr_gpu_plan_info", c_int, [c_void_p, POINTER(c_int), POINTER(c_longlong),
                                      POINTER(c_int), POINTER(c_int)])
    sig("dplr_gpu_plan_device_bytes", c_longlong, [c_void_p])
    sig("dplr_gpu_apply", c_int, [c_void_p, c_char, c_int, c_double, c_void_p, c_int, c_double,
                                  c_void_p, c_int, c_void_p])
    sig("dplr_gpu_register", c_int, [c_int, PDPlrMtx])
    sig("dplr_gpu_unregister", c_int, [PDPlrMtx])
    sig("dplr_gpu_factor", c_int, [c_void_p, c_int, c_void_p])
    sig("dplr_gpu_factor_device_bytes", c_longlong, [c_void_p])
    sig("dplr_gpu_solve", c_int, [c_void_p, c_char, c_int, c_void_p, c_int, c_void_p, c_int,
                                  c_void_p])
    sig("dplr_gpu_solve_refined", c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_int,
                                          c_double, c_int, c_int, POINTER(c_double),
                                          POINTER(c_int), c_void_p])
    sig("dplr_gpu_prepare_sliced", c_int, [c_void_p, c_void_p])
    sig("dplr_gpu_prepare_mixed", c_int, [c_void_p, c_int, c_void_p])
    sig("dplr_gpu_prepare_mixed_caps", c_int, [c_void_p, c_int, c_int, c_void_p])
    sig("dplr_gpu_prepare_pairs", c_int, [c_void_p, c_void_p])
    sig("dplr_gpu_geppmm", c_int, [c_char, c_char, c_int, c_double, PDPlrMtx, PDPlrMtx, c_double,
                                   PDPlrMtx, c_double, c_void_p])
    sig("dplr_gpu_reduce_svd", c_int, [c_int, PDPlrMtx, c_double, c_int])
    sig("dplr_gpu_d2gep", c_int, [c_int, c_void_p, c_int, PDPlrMtx, c_double, c_int, c_int,
                                  POINTER(c_int)])
    sig("dplr_gpu_scal", c_int, [c_void_p, c_double, c_void_p])
    sig("dplr_gpu_adpy", c_int, [c_void_p, c_double, c_void_p, c_void_p])
    sig("dplr_gpu_residual", c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_int, c_void_p,
                                     c_int, c_int, c_void_p])
    sig("dplr_gpu_solve_refined_host", c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_int,
                                               c_double, c_int, c_int, POINTER(c_double),
                                               POINTER(c_int), c_void_p])
    sig("dplr_gpu_pool_size", c_longlong, [c_void_p])
    sig("dplr_gpu_pool_blocks", c_int, [c_void_p, POINTER(c_int), POINTER(c_int)])
    sig("dplr_gpu_pool_block", c_int, [c_void_p, c_int, POINTER(c_longlong), POINTER(c_longlong),
                                       POINTER(c_longlong), POINTER(c_int), POINTER(c_int),
                                       POINTER(c_int), POINTER(c_int)])
    sig("dplr_gpu_pool_read", c_int, [c_void_p, c_void_p, c_void_p])
    sig("dplr_gpu_pool_write", c_int, [c_void_p, c_void_p, c_void_p])
    sig("dplr_gpu_grad_factors", c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_int, c_double,
                                         c_void_p, c_void_p])
    sig("dplr_gpu_batch_create", c_int, [c_int, POINTER(c_int), POINTER(PDPlrMtx), c_void_p,
                                         POINTER(c_void_p)])
    sig("dplr_gpu_batch_offsets", c_int, [c_void_p, POINTER(c_int), POINTER(c_int)])
    sig("dplr_gpu_graph_create", c_int, [c_void_p, c_char, c_char, c_int, c_void_p, c_int, c_void_p,
                                         c_int, c_void_p, POINTER(c_void_p)])
    sig("dplr_gpu_graph_launch", c_int, [c_void_p, c_void_p])
    sig("dplr_gpu_graph_kernels", c_longlong, [c_void_p])
    sig("dplr_gpu_graph_destroy", None, [c_void_p])
    sig("dplr_gpu_autotune", c_int, [c_void_p, c_int, c_void_p, POINTER(c_int), POINTER(c_int),
                                     POINTER(c_double)])
    sig("dplr_gpu_launch_count", c_longlong, [])
    sig("dplr_gpu_profile_start", c_int, [])
    sig("dplr_gpu_profile_stop", c_int, [])
    sig("dplr_gpu_profile_entry", c_int, [c_int, POINTER(ctypes.c_char_p), POINTER(c_double),
                                          POINTER(c_double), POINTER(c_double), POINTER(c_int)])
    for name, res, args in _OPTIONAL:
        if hasattr(lib, name):
            sig(name, res, args)


# Entry points added by later modules of the library (bound when present).
_OPTIONAL: list = [
    ("dplr_gpu_debug_fail_alloc", None, [c_int]),
    ("dplr_gpu_debug_wait_limit", c_int, [c_int]),
    ("dplr_gpu_plan_copy", c_int, [c_void_p, c_void_p, POINTER(c_void_p)]),
    ("dplr_gpu_axpy", c_int, [c_double, c_void_p, c_void_p, c_void_p, POINTER(c_void_p)]),
    ("dplr_gpu_gep2d", c_int, [c_void_p, c_void_p, c_longlong, c_void_p]),
    ("dplr_gpu_plan_reduce_svd", c_int, [c_void_p, c_double, c_int, c_void_p, POINTER(c_void_p)]),
    ("dplr_gpu_set_recompress", None, [c_double]),
    ("dplr_gpu_apply_form", c_int, [c_void_p]),
]


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NativeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        try:
            _lib = ctypes.CDLL(LIB_PATH)
        except OSError as e:
            raise NativeError(f"cannot load {LIB_PATH}: {e}") from e
        _bind(_lib)
    return _lib


def api() -> PlrApi:
    """The drop-in DPLR entry points (dplrgepmv, dplrgepdmm, ...)."""
    global _api
    if _api is None:
        _api = PlrApi(lib(), "dplr")
    return _api


def launch_count() -> int:
    return int(lib().dplr_gpu_launch_count())


def profile_start() -> None:
    check(lib().dplr_gpu_profile_start(), "dplr_gpu_profile_start")


def profile_stop() -> dict:
    """Per kernel kind: {name: (ms, flops, bytes, launches)} since profile_start()."""
    n = lib().dplr_gpu_profile_stop()
    if n < 0:
        check(n, "dplr_gpu_profile_stop")
    out = {}
    for i in range(n):
        name, ms, fl, by, la = ctypes.c_char_p(), c_double(), c_double(), c_double(), c_int()
        check(lib().dplr_gpu_profile_entry(i, ctypes.byref(name), ctypes.byref(ms), ctypes.byref(fl),
                                           ctypes.byref(by), ctypes.byref(la)), "profile entry")
        out[name.value.decode()] = (ms.value, fl.value, by.value, la.value)
    return out


def last_error() -> str:
    return lib().dplr_gpu_last_error().decode()


def check(rc: int, what: str) -> None:
    if rc != 0:
        raise NativeError(f"{what} failed ({rc}): {last_error()}")


__all__ = ["lib", "api", "last_error", "check", "NativeError", "LIB_PATH", "c_double_p"]
