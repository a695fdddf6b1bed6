"""GPU apply (dplrgepmv / dplrgepdmm / dplr_gpu_apply) against the oracle.

Seeded trees of several shapes (uniform, uneven and zero ranks, ranks above
the 64-wide rank tile, a non-uniform tree whose leaves sit at different
depths), every op combination, strides, padded leading dimensions and the
alpha/beta special cases.  Tolerance: 1e-12 relative (Frobenius) against
the FP64 oracle.
"""
import ctypes

import numpy as np
import pytest

from dplr_gb300 import gen, tree
from oracle import pyoracle

pytestmark = pytest.mark.gpu
TOL = 1e-12


def nonuniform_tree(n, leaf, rank, seed):
    rng = np.random.default_rng(seed)

    def build(m, level):
        if m <= leaf or (m <= 4 * leaf and rng.random() < 0.5):
            return tree.Dense(rng.standard_normal((m, m)) + m * np.eye(m))
        h = m // 2

        def lr():
            r = int(rng.integers(0, rank + 1))
            return tree.LowRank(rng.standard_normal((h, r)), rng.random(r) + 0.1,
                                rng.standard_normal((h, r)))
        return tree.HNode(build(h, level + 1), lr(), build(h, level + 1), lr())
    return build(n, 0)


TREES = {
    "uniform1k": lambda: gen.random_tree(1024, 64, 16, seed=1),
    "uneven2k": lambda: gen.random_tree(2048, 32, [70, 0, 9, 33, 1, 5], seed=2, capacity_extra=3),
    "nonuniform": lambda: nonuniform_tree(1024, 16, 12, seed=3),
    "dense_only": lambda: tree.Dense(np.random.default_rng(4).standard_normal((96, 96))),
    "exp4k": lambda: gen.exp1d_tree(gen.sorted_uniform(4096, 5), 0.1, 1e-2, 64, 8, seed=5),
}


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def gpu():
    from dplr_gb300 import _native
    return _native.api()


@pytest.fixture(scope="module")
def orc():
    return pyoracle.oracle("best")


@pytest.mark.parametrize("name", list(TREES))
@pytest.mark.parametrize("trans", ["N", "T"])
def test_pmv(gpu, orc, name, trans):
    t = TREES[name]()
    m = t.size
    rng = np.random.default_rng(7)
    for alpha, beta, incx, incy in [(1.0, 0.0, 1, 1), (-0.5, 1.5, 2, 1), (2.0, 1.0, 1, 3)]:
        x = rng.standard_normal(m * incx)
        y0 = rng.standard_normal(m * incy)
        outs = []
        for api in (gpu, orc):
            a = tree.to_c(t)
            y = y0.copy()
            api.gepmv(trans, m, alpha, a, x, incx, beta, y, incy)
            tree.free_c(a)
            outs.append(y)
        assert rel(outs[0], outs[1]) <= TOL, (alpha, beta, incx, incy)


@pytest.mark.parametrize("name", list(TREES))
@pytest.mark.parametrize("ops", ["NN", "TN", "NT", "TT"])
@pytest.mark.parametrize("n", [1, 3, 8, 17, 40])
def test_pdmm(gpu, orc, name, ops, n):
    t = TREES[name]()
    m = t.size
    rng = np.random.default_rng(n)
    ta, tb = ops
    rows_b, cols_b = (m, n) if tb == "N" else (n, m)
    ldb, ldc = rows_b + 2, m + 1
    b = rng.standard_normal(ldb * cols_b)
    c0 = rng.standard_normal(ldc * n)
    beta = 0.0 if n % 2 else 0.75
    outs = []
    for api in (gpu, orc):
        a = tree.to_c(t)
        c = c0.copy()
        api.gepdmm(ta, tb, m, n, -1.25, a, b, ldb, beta, c, ldc)
        tree.free_c(a)
        outs.append(c.reshape(ldc, n, order="F"))
    assert np.array_equal(outs[0][m:], c0.reshape(ldc, n, order="F")[m:])
    assert rel(outs[0][:m], outs[1][:m]) <= TOL


def test_alpha_zero_quirk(gpu, orc):
    """alpha == 0: dplrgepmv scales y by beta twice (DPLR src/dplrpmv.c:140-160)."""
    t = TREES["uniform1k"]()
    m = t.size
    y0 = np.random.default_rng(0).standard_normal(m)
    x = np.full(m, np.nan)        # never read when alpha == 0
    outs = []
    for api in (gpu, orc):
        a = tree.to_c(t)
        y = y0.copy()
        api.gepmv("N", m, 0.0, a, x, 1, 0.5, y, 1)
        tree.free_c(a)
        outs.append(y)
    assert np.array_equal(outs[0], outs[1])
    assert np.allclose(outs[0], 0.25 * y0)


def test_beta_zero_ignores_nan_output(gpu):
    t = TREES["uneven2k"]()
    m = t.size
    x = np.random.default_rng(1).standard_normal(m)
    y = np.full(m, np.nan)
    a = tree.to_c(t)
    gpu.gepmv("N", m, 1.0, a, x, 1, 0.0, y, 1)
    tree.free_c(a)
    assert np.all(np.isfinite(y))
    assert rel(y, tree.to_dense(t) @ x) <= TOL


def test_registered_plan_reused_and_refreshable(gpu, orc):
    from dplr_gb300 import _native
    lib = _native.lib()
    t = TREES["exp4k"]()
    m = t.size
    a = tree.to_c(t)
    try:
        _native.check(lib.dplr_gpu_register(m, a), "register")
        x = np.random.default_rng(3).standard_normal(m)
        y = np.zeros(m)
        gpu.gepmv("N", m, 1.0, a, x, 1, 0.0, y, 1)
        assert rel(y, tree.to_dense(t) @ x) <= TOL
        # Modify the host tree: the registered plan is stale until re-registered.
        node = a
        while node.contents.type != tree.PLR_DMTX:
            node = node.contents.dh.nw
        node.contents.dd.d[0] += 1.0
        _native.check(lib.dplr_gpu_register(m, a), "re-register")
        y2 = np.zeros(m)
        gpu.gepmv("N", m, 1.0, a, x, 1, 0.0, y2, 1)
        assert abs((y2 - y)[0] - x[0]) < 1e-9
        _native.check(lib.dplr_gpu_unregister(a), "unregister")
    finally:
        tree.free_c(a)


def test_invalid_arguments_leave_output_untouched(gpu, capfd):
    t = TREES["uniform1k"]()
    m = t.size
    a = tree.to_c(t)
    x = np.ones(m)
    y = np.arange(m, dtype=float)
    gpu.gepmv("N", m + 2, 1.0, a, x, 1, 0.0, y, 1)          # wrong size
    gpu.gepmv("N", m, 1.0, a, x, 0, 0.0, y, 1)              # zero increment
    c = np.arange(m * 2, dtype=float)
    gpu.gepdmm("N", "N", m, 2, 1.0, a, np.ones(m * 2), m, 0.0, c, m - 1)   # ldc < m
    tree.free_c(a)
    assert np.array_equal(y, np.arange(m, dtype=float))
    assert np.array_equal(c, np.arange(m * 2, dtype=float))
    err = capfd.readouterr().err
    assert "dplrgepmv: invalid A size" in err and "dplrgepdmm: invalid leading dimensions" in err


@pytest.mark.parametrize("name", list(TREES))
def test_plan_nnz_matches_dplrnz(name):
    """plan_info's nnz is DPLR's dplrnz: size * (rank_ne + rank_sw) per H node
    plus the leaves (src/dplrnz.c:17-62)."""
    from dplr_gb300.plan import GpuPlan
    t = TREES[name]()
    p = GpuPlan(t)
    assert p.nnz == tree.nnz(t)
    p.close()
