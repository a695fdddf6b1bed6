"""Failure paths made on the host (no GPU fault is ever provoked).

Device allocations of plans, factorisations and scratch go through one
allocator whose k-th call can be made to fail (dplr_gpu_debug_fail_alloc).
Every entry point must then return DPLR_GPU_ENOMEM (the DPLR drop-ins print
"<function>: <reason>" like the reference, src/dplrpdmm.c:180-199), leave
its outputs untouched, free what it had allocated, and the next call
without injection must succeed.
"""
import ctypes

import numpy as np
import pytest

from dplr_gb300 import gen, tree

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ENOMEM = -3


@pytest.fixture
def lib():
    from dplr_gb300 import _native
    lb = _native.lib()
    yield lb
    lb.dplr_gpu_debug_fail_alloc(-1)


def _plan_create(lib, t):
    a = tree.to_c(t)
    h = ctypes.c_void_p()
    rc = lib.dplr_gpu_plan_create(t.size, a, None, ctypes.byref(h))
    tree.free_c(a)
    return rc, h


def test_plan_creation_fails_cleanly_at_every_allocation(lib):
    from dplr_gb300 import _native
    t = gen.random_tree(1024, 64, [16, 8, 4, 2], seed=1)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failures = 0
    for k in range(0, 40):
        lib.dplr_gpu_debug_fail_alloc(k)
        rc, h = _plan_create(lib, t)
        lib.dplr_gpu_debug_fail_alloc(-1)
        if rc == 0:                         # all of its allocations came before the k-th
            lib.dplr_gpu_plan_destroy(h)
            break
        assert rc == ENOMEM, (k, rc, _native.last_error())
        assert "allocate" in _native.last_error()
        failures += 1
    assert failures >= 3
    torch.cuda.synchronize()
    assert abs(torch.cuda.mem_get_info()[0] - free0) <= 8 << 20      # nothing leaked
    rc, h = _plan_create(lib, t)
    assert rc == 0
    lib.dplr_gpu_plan_destroy(h)


def test_drop_in_product_reports_and_leaves_output_untouched(lib, capfd):
    from dplr_gb300 import _native
    t = gen.random_tree(512, 32, [12, 8, 5, 3], seed=2)
    m = t.size
    a = tree.to_c(t)
    b = np.random.default_rng(0).standard_normal(m * 3)
    c0 = np.random.default_rng(1).standard_normal(m * 3)
    c = c0.copy()
    lib.dplr_gpu_debug_fail_alloc(0)
    _native.api().gepdmm("N", "N", m, 3, 1.0, a, b, m, 0.5, c, m)
    lib.dplr_gpu_debug_fail_alloc(-1)
    err = capfd.readouterr().err
    assert "dplrgepdmm:" in err and "allocate" in err
    assert np.array_equal(c, c0)
    _native.api().gepdmm("N", "N", m, 3, 1.0, a, b, m, 0.5, c, m)   # recovers
    tree.free_c(a)
    assert not np.array_equal(c, c0)


def test_factorisation_and_solve_fail_then_recover(lib):
    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan
    t = gen.random_tree(1024, 64, [16, 8, 4, 2], seed=3)
    plan = GpuPlan(t)
    lib.dplr_gpu_debug_fail_alloc(0)
    with pytest.raises(_native.NativeError, match=r"\(-3\)"):
        plan.factor()
    lib.dplr_gpu_debug_fail_alloc(-1)
    plan.factor()
    b = torch.randn(4, t.size, dtype=torch.float64, device="cuda")
    x = torch.full_like(b, 7.0)
    lib.dplr_gpu_debug_fail_alloc(0)
    with pytest.raises(_native.NativeError, match=r"\(-3\)"):
        plan.solve_refined(b, tol=1e-12, maxiter=5, out=x, precise=False)
    lib.dplr_gpu_debug_fail_alloc(-1)
    x, res, _ = plan.solve_refined(b, tol=1e-12, maxiter=5, out=x, precise=False)
    assert res <= 1e-12
    plan.close()


def test_tensor_core_waits_expire_cleanly_and_the_plan_recovers(lib):
    """With the role-to-role waits of the tcgen05 kernels bounded to a few
    polls, they expire: the kernels drain, free tensor memory and record
    the expiry; the plan's next call reports it, the call after that runs
    normally and gives the same residual as before."""
    from dplr_gb300 import _native, gen_gpu
    from dplr_gb300.plan import GpuPlan
    t = gen_gpu.kernel_tree_2d(n=4096, leaf=128, rmax=64, seed=3)
    p = GpuPlan(t)
    p.prepare_sliced()
    g = torch.Generator(device="cpu").manual_seed(0)
    x = torch.randn(64, t.size, generator=g, dtype=torch.float64).cuda()
    b = torch.randn(64, t.size, generator=g, dtype=torch.float64).cuda()
    r0 = p.residual(x, b, precise=True)
    torch.cuda.synchronize()
    try:
        assert lib.dplr_gpu_debug_wait_limit(4) == 0
        p.residual(x, b, precise=True)
        torch.cuda.synchronize()
    finally:
        assert lib.dplr_gpu_debug_wait_limit(0) == 0
    with pytest.raises(_native.NativeError, match="bounded wait expired"):
        p.residual(x, b, precise=True)
    r1 = p.residual(x, b, precise=True)
    torch.cuda.synchronize()
    assert torch.equal(r0, r1)
    p.close()
