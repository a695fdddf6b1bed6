"""dplr_gpu_apply_noalloc: the apply for callers that cannot allocate.

Latency-critical paths that must not call cudaMalloc/cudaFree, and hosts
with a fixed device-memory
budget use this entry point; its scratch is a static device array inside
the library.  It must give the same result as dplr_gpu_apply (1e-12
relative, the tolerance of the apply tests) on two calls in a row, and
reject a request larger than its fixed scratch.  The file is named so that
pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from dplr_gb300 import gen

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL = 1e-12


def _noalloc_fn():
    from dplr_gb300 import _native
    lib = _native.lib()
    f = lib.dplr_gpu_apply_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_char, ctypes.c_int, ctypes.c_double, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    return f


def rel(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


def test_noalloc_apply_matches_apply_on_two_calls():
    from dplr_gb300.plan import GpuPlan
    f = _noalloc_fn()
    t = gen.random_tree(2048, 64, [40, 24, 16, 8, 4], seed=31)
    p = GpuPlan(t)
    m = t.size
    stream = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    for trans in ("N", "T"):
        for call in range(2):
            x = torch.randn(5, m, dtype=torch.float64, device="cuda", generator=g)
            y0 = torch.randn(5, m, dtype=torch.float64, device="cuda", generator=g)
            want = p.apply(x, trans=trans, alpha=0.7, beta=-0.3, out=y0.clone())
            got = y0.clone()
            rc = f(p.handle, trans.encode(), 5, 0.7, x.data_ptr(), m, -0.3, got.data_ptr(), m, stream)
            torch.cuda.synchronize()
            assert rc == 0, f"call {call}: rc {rc}"
            assert rel(got, want) <= TOL, f"{trans} call {call}"
    p.close()


def test_noalloc_apply_rejects_oversized_request():
    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan
    f = _noalloc_fn()
    t = gen.random_tree(4096, 64, 64, seed=32)
    p = GpuPlan(t)
    m = t.size
    n = 4096                      # far more scratch than the static array holds
    x = torch.zeros(n, m, dtype=torch.float64, device="cuda")
    y = torch.zeros(n, m, dtype=torch.float64, device="cuda")
    rc = f(p.handle, b"N", n, 1.0, x.data_ptr(), m, 0.0, y.data_ptr(), m,
           torch.cuda.current_stream().cuda_stream)
    assert rc == -1
    assert "static scratch" in _native.last_error()
    p.close()


def test_noalloc_apply_allocates_nothing():
    """The property callers rely on: with every device allocation the library
    might make set up to fail (the fault-injection hook), the call on a
    fresh plan, which has no apply scratch of its own yet, still succeeds,
    gives the same result, and leaves the plan's device memory unchanged."""
    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan
    f = _noalloc_fn()
    lib = _native.lib()
    t = gen.random_tree(1024, 64, [20, 12, 6, 3], seed=33)
    m = t.size
    stream = torch.cuda.current_stream().cuda_stream
    x = torch.randn(3, m, dtype=torch.float64, device="cuda")
    ref = GpuPlan(t)
    want = ref.apply(x)
    fresh = GpuPlan(t)
    before = lib.dplr_gpu_plan_device_bytes(fresh.handle)
    got = torch.zeros_like(x)
    torch.cuda.synchronize()
    try:
        lib.dplr_gpu_debug_fail_alloc(0)          # the next library allocation would fail
        rc = f(fresh.handle, b"N", 3, 1.0, x.data_ptr(), m, 0.0, got.data_ptr(), m, stream)
        torch.cuda.synchronize()
    finally:
        lib.dplr_gpu_debug_fail_alloc(-1)
    assert rc == 0, _native.last_error()
    assert rel(got, want) <= TOL
    assert lib.dplr_gpu_plan_device_bytes(fresh.handle) == before
    fresh.close()
    ref.close()
