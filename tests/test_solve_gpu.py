"""Woodbury factorisation and solves on the GPU against the FP64 oracle.

x = A^-1 b from dplr_gpu_solve is checked (1) against a dense LU solve of
the expanded matrix (small cases) and (2) through its relative residual
||A x - b|| / ||b|| computed by the oracle's own FP64 apply; the refined
solve must reach 1e-12.
"""
import numpy as np
import pytest

from dplr_gb300 import gen, tree
from oracle import pyoracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def oracle_resid(t, x, b, trans="N"):
    """max_j ||op(A) x_j - b_j|| / ||b_j|| with the oracle's FP64 apply."""
    orc = pyoracle.oracle("best")
    m, n = t.size, x.shape[0]
    a = tree.to_c(t)
    y = np.zeros(m * n)
    orc.gepdmm(trans, "N", m, n, 1.0, a, np.ascontiguousarray(x).reshape(-1), m, 0.0, y, m)
    tree.free_c(a)
    r = y.reshape(n, m) - b
    return float(np.max(np.linalg.norm(r, axis=1) / np.linalg.norm(b, axis=1)))


CASES = {
    "rand1k": lambda: gen.random_tree(1024, 64, [20, 12, 8, 4], seed=1),
    "uneven": lambda: gen.random_tree(2048, 32, [40, 0, 7, 16, 1, 3], seed=2),
    "exp4k": lambda: gen.exp1d_tree(gen.sorted_uniform(4096, 3), 0.1, 1e-2, 64, 4, seed=3),
    "dense": lambda: tree.Dense(np.random.default_rng(4).standard_normal((64, 64)) + 16 * np.eye(64)),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("trans", ["N", "T"])
def test_solve_matches_dense(name, trans):
    from dplr_gb300.plan import GpuPlan
    t = CASES[name]()
    m = t.size
    p = GpuPlan(t)
    p.factor()          # the transposed solve reuses the forward factors
    rng = np.random.default_rng(5)
    b = rng.standard_normal((7, m))
    x = p.solve(torch.tensor(b, device="cuda"), trans=trans).cpu().numpy()
    dense = tree.to_dense(t)
    want = np.linalg.solve(dense if trans == "N" else dense.T, b.T).T
    err = np.linalg.norm(x - want) / np.linalg.norm(want)
    assert err <= 1e-9 * np.linalg.cond(dense), err
    assert oracle_resid(t, x, b, trans) <= 1e-10   # unrefined; refinement is tested below
    p.close()


@pytest.mark.parametrize("name", list(CASES))
def test_refined_solve_reaches_1e12(name):
    from dplr_gb300.plan import GpuPlan
    t = CASES[name]()
    m = t.size
    p = GpuPlan(t)
    p.factor()
    b = np.random.default_rng(6).standard_normal((33, m))
    x, res, its = p.solve_refined(torch.tensor(b, device="cuda"), tol=1e-12, maxiter=5)
    assert res <= 1e-12
    assert oracle_resid(t, x.cpu().numpy(), b) <= 1.5e-12
    p.close()


def test_solve_is_inverse_of_apply():
    from dplr_gb300.plan import GpuPlan
    t = gen.random_tree(4096, 64, [32, 24, 16, 8, 8, 4], seed=9)
    p = GpuPlan(t)
    p.factor(transposed=True)
    xs = torch.randn(16, t.size, dtype=torch.float64, device="cuda")
    for trans in "NT":
        b = p.apply(xs, trans=trans)
        x = p.solve(b, trans=trans)
        assert (torch.linalg.norm(x - xs) / torch.linalg.norm(xs)).item() <= 1e-11
    p.close()


def test_singular_leaf_reported():
    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan
    t = gen.random_tree(256, 32, 4, seed=10)
    node = t
    while isinstance(node, tree.HNode):
        node = node.nw
    node.d[:] = 0.0
    p = GpuPlan(t)
    with pytest.raises(_native.NativeError, match="singular"):
        p.factor()
    p.close()


@pytest.mark.parametrize("maxiter", [0, 3])
def test_refined_solve_with_host_buffers(maxiter):
    """dplr_gpu_solve_refined_host (B and X in host memory, X copied back
    while the refinement checks each iterate) returns the device path's X
    bit for bit, with its residual and correction count, whether it stops
    converged or at maxiter (DPLR_GPU_ENOTCONV, X the last iterate)."""
    import ctypes
    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan
    t = CASES["exp4k"]()
    m = t.size
    p = GpuPlan(t)
    p.factor()
    b = np.random.default_rng(8).standard_normal((5, m))
    tol = 1e-12 if maxiter else 1e-30
    xd, res_d, its_d = p.solve_refined(torch.tensor(b, device="cuda"), tol=tol, maxiter=maxiter, precise=False,
                                       strict=False)
    bh = torch.tensor(b).pin_memory()
    xh = torch.full((5, m), np.nan, dtype=torch.float64).pin_memory()
    res, its = ctypes.c_double(), ctypes.c_int()
    rc = _native.lib().dplr_gpu_solve_refined_host(p.handle, 5, bh.data_ptr(), m, xh.data_ptr(), m, tol, maxiter,
                                                   0, ctypes.byref(res), ctypes.byref(its), None)
    assert rc == (0 if maxiter else -5)
    assert torch.equal(xh, xd.cpu())
    assert res.value == res_d and its.value == its_d
    p.close()


def test_refactorisation_after_new_values_reuses_the_layout():
    """New factor values (dplr_gpu_pool_write) keep the factorisation's
    layout: the next factor() recomputes the numbers only.  The solve after
    a refactorisation of the same values is bit-identical; a singular leaf
    written in between is reported (and the plan refuses to solve), and
    restoring the values makes the plan factor and solve again."""
    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan
    t = gen.random_tree(1024, 64, [12, 8, 4, 2], seed=11)
    p = GpuPlan(t)
    p.factor()
    b = torch.randn(3, t.size, dtype=torch.float64, device="cuda")
    x0 = p.solve(b).clone()
    xt0 = p.solve(b, trans="T").clone()
    pool = p.read_pool()
    p.write_pool(pool)
    p.factor()
    assert torch.equal(p.solve(b), x0)
    assert torch.equal(p.solve(b, trans="T"), xt0)
    leaf = next(blk for blk in p.pool_blocks() if blk["kind"] == "leaf")
    bad = pool.clone()
    bad[leaf["d"]:leaf["d"] + leaf["b"] * leaf["b"]] = 0.0
    p.write_pool(bad)
    with pytest.raises(_native.NativeError, match="singular"):
        p.factor()
    with pytest.raises(_native.NativeError, match="not factored"):
        p.solve(b)
    p.write_pool(pool)
    p.factor()
    assert torch.equal(p.solve(b), x0)
    p.close()
