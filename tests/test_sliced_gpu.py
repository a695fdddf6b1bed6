"""Exact-slice (bf16 tensor-core) residual R = B - A X.

The residual is checked against one computed in extended precision
(numpy longdouble on the dense expansion), and shown to be far more
accurate than the FP64 apply on a matrix with strong cancellation
(|A||x| >> |b|); refinement with it reaches relative residuals that FP64
residuals cannot certify.
"""
import numpy as np
import pytest

from dplr_gb300 import gen, tree

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def apply_ld(node, x):
    """A x from the PLR factors in extended precision (numpy longdouble)."""
    ld = np.longdouble
    if isinstance(node, tree.Dense):
        return node.d.astype(ld) @ x
    h = node.nw.size

    def lr(b, xs):
        return (b.u.astype(ld) * b.sig.astype(ld)) @ (b.v.astype(ld).T @ xs)
    top = apply_ld(node.nw, x[:h]) + lr(node.ne, x[h:])
    bot = apply_ld(node.se, x[h:]) + lr(node.sw, x[:h])
    return np.vstack([top, bot])


def exact_residual(t, x, b):
    """b - A x with the PLR operator applied in extended precision."""
    ax = apply_ld(t, x.astype(np.longdouble).T).T
    return b.astype(np.longdouble) - ax


def _residual_errors(t, x, b):
    from dplr_gb300.plan import GpuPlan
    p = GpuPlan(t)
    p.prepare_sliced()
    xt = torch.tensor(x, device="cuda")
    bt = torch.tensor(b, device="cuda")
    rs = p.residual(xt, bt, precise=True).cpu().numpy()
    r64 = p.residual(xt, bt, precise=False).cpu().numpy()
    p.close()
    want = exact_residual(t, x, b)
    nb = np.linalg.norm(b)
    return (float(np.linalg.norm((rs - want).astype(np.float64))) / nb,
            float(np.linalg.norm((r64 - want).astype(np.float64))) / nb)


def test_sliced_residual_on_random_tree():
    """Diagonally dominant random leaves: both residuals are accurate; the
    sliced one is never worse than the FP64 apply."""
    t = gen.random_tree(1024, 64, [24, 16, 8, 4], seed=2)
    rng = np.random.default_rng(4)
    x = rng.standard_normal((6, t.size))
    b = (tree.to_dense(t) @ x.T).T + 1e-6 * rng.standard_normal((6, t.size))
    err_s, err_64 = _residual_errors(t, x, b)
    assert err_s <= 2.0 * err_64 + 1e-18, (err_s, err_64)


def test_sliced_residual_under_cancellation():
    """Kernel matrix with x = A^-1 b: |A||x| >> |b| and the residual cancels
    across levels.  The exact-slice residual is limited only by the 57-bit
    slice truncation (about 2^-57 |A||x|), the FP64 apply by rounding in
    every dot product: the sliced residual must be clearly more accurate."""
    from dplr_gb300 import gen_gpu
    from dplr_gb300.plan import GpuPlan
    t = gen_gpu.kernel_tree_2d(n=4096, leaf=64, shift=1e-2, seed=3, rmax=64)
    p = GpuPlan(t)
    p.factor()
    rng = np.random.default_rng(4)
    b = rng.standard_normal((6, t.size))
    x = p.solve(torch.tensor(b, device="cuda")).cpu().numpy()
    p.close()
    err_s, err_64 = _residual_errors(t, x, b)
    assert err_s * 2 <= err_64, (err_s, err_64)
    assert err_s <= 1e-13, (err_s, err_64)


def test_refinement_with_sliced_residual_reaches_1e13():
    """FP64 inner solves: the FP64 residual stalls near 4e-13 on this
    matrix, the exact-slice residual certifies 1e-13."""
    from dplr_gb300 import gen_gpu
    from dplr_gb300.plan import GpuPlan
    t = gen_gpu.kernel_tree_2d(n=16384, leaf=128, shift=1e-2, seed=6, rmax=96)
    p = GpuPlan(t)
    p.factor()
    p.prepare_sliced()
    g = torch.Generator(device="cpu").manual_seed(1)
    b = torch.randn(16, t.size, generator=g, dtype=torch.float64).cuda()
    x, res, its = p.solve_refined(b, tol=1e-13, maxiter=10, precise=True)
    assert res <= 1e-13
    _, res64, _ = p.solve_refined(b, tol=1e-13, maxiter=4, precise=False, strict=False)
    assert res64 > res, (res64, res)
    p.close()


@pytest.mark.parametrize("shape", ["kernel2d", "random"])
def test_mixed_refined_solve_reaches_1e12(shape):
    """Low-precision (sliced bf16) inner solves + exact-slice residuals.  The
    kernel matrix needs 6 slices (43 bits): its Woodbury sweep amplifies
    inner-solve errors by about 1e7."""
    from dplr_gb300 import gen_gpu
    from dplr_gb300.plan import GpuPlan
    from oracle import pyoracle
    if shape == "kernel2d":
        t = gen_gpu.kernel_tree_2d(n=16384, leaf=128, seed=6, rmax=96)
    else:
        t = gen.random_tree(4096, 64, [32, 24, 16, 8, 4, 2], seed=7)
    p = GpuPlan(t)
    p.factor()
    p.prepare_sliced()
    p.prepare_mixed(6 if shape == "kernel2d" else 4)
    b = torch.randn(40, t.size, dtype=torch.float64, device="cuda")
    x, res, its = p.solve_refined(b, tol=1e-12, maxiter=20, precise=True, mixed=True)
    assert res <= 1e-12
    # independent check with the oracle's FP64 apply (its own rounding ~1e-12)
    orc = pyoracle.oracle("best")
    a = tree.to_c(t)
    xb = x.cpu().numpy()
    y = np.zeros(xb.size)
    orc.gepdmm("N", "N", t.size, xb.shape[0], 1.0, a, np.ascontiguousarray(xb).reshape(-1), t.size,
               0.0, y, t.size)
    tree.free_c(a)
    bb = b.cpu().numpy()
    rel = np.max(np.linalg.norm(y.reshape(bb.shape) - bb, axis=1) / np.linalg.norm(bb, axis=1))
    assert rel <= 1e-11
    p.close()


def _plan(t, mma: bool, mixed_slices: int = 0):
    """Plan whose sliced products run on the mma.sync kernels (mma=True) or
    on the tcgen05 kernels (128-row tiles; leaves that are multiples of 128
    rows, or whose size divides 128 for the residual)."""
    import os
    from dplr_gb300.plan import GpuPlan
    old = os.environ.get("DPLR_GB300_SLICED_MMA")
    os.environ["DPLR_GB300_SLICED_MMA"] = "1" if mma else "0"
    try:
        p = GpuPlan(t)
        p.factor()
        p.prepare_sliced()
        if mixed_slices:
            p.prepare_mixed(mixed_slices)
    finally:
        if old is None:
            del os.environ["DPLR_GB300_SLICED_MMA"]
        else:
            os.environ["DPLR_GB300_SLICED_MMA"] = old
    return p


@pytest.mark.parametrize("kind", ["random_rank160", "kernel2d", "leaf64_rank4"])
def test_tcgen05_residual_matches_mma_sync(kind):
    """Both kernel families compute exact integer products of 57-bit slices
    and round once; their operand slicing differs (the tcgen05 path cuts U
    and T per 128-row tile-block), so the two agree to the slice-truncation
    level, about 2^-57 |A||x|.  70 right-hand sides exercise a ragged
    64-column tile; ranks above 128 exercise the panel's later rank tiles;
    64-row leaves and blocks (stored as half-empty 128-row tiles) with ranks
    1-4 exercise the small-block layout."""
    from dplr_gb300 import gen_gpu
    if kind == "kernel2d":
        t = gen_gpu.kernel_tree_2d(n=8192, leaf=128, rmax=96, seed=8)
    elif kind == "leaf64_rank4":
        t = gen.random_tree(2048, 64, [4, 1, 3, 2, 4], seed=11)
    else:
        t = gen.random_tree(2048, 128, [160, 140, 100, 40], seed=9)
    rng = np.random.default_rng(10)
    x = rng.standard_normal((70, t.size))
    b = rng.standard_normal((70, t.size))
    pt, pm = _plan(t, mma=False), _plan(t, mma=True)
    xt = torch.tensor(x, device="cuda")
    bt = torch.tensor(b, device="cuda")
    rt = pt.residual(xt, bt, precise=True).cpu().numpy()
    rm = pm.residual(xt, bt, precise=True).cpu().numpy()
    pt.close()
    pm.close()
    assert np.all(np.isfinite(rt))
    want = exact_residual(t, x, b)
    nax = float(np.linalg.norm((b - want).astype(np.float64)))      # ||A x||
    err_t = float(np.linalg.norm((rt - want).astype(np.float64))) / nax
    err_m = float(np.linalg.norm((rm - want).astype(np.float64))) / nax
    assert err_t <= 1e-15, err_t
    assert err_m <= 1e-15, err_m
    assert float(np.linalg.norm(rt - rm)) / nax <= 2e-15


@pytest.mark.parametrize("ns", [6, 7])
def test_tcgen05_mixed_refined_solve(ns):
    """Mixed refinement with the tcgen05 kernels reaches the tolerance and
    agrees with the mma.sync path's solution (7 slices: 8 diagonals, whose
    64-bit read-out drops 7 bits of the lowest one)."""
    from dplr_gb300 import gen_gpu
    t = gen_gpu.kernel_tree_2d(n=16384, leaf=128, rmax=96, seed=6)
    g = torch.Generator(device="cpu").manual_seed(2)
    b = torch.randn(70, t.size, generator=g, dtype=torch.float64).cuda()
    pt, pm = _plan(t, mma=False, mixed_slices=ns), _plan(t, mma=True, mixed_slices=ns)
    xt, rt, _ = pt.solve_refined(b, tol=1e-12, maxiter=10, precise=True, mixed=True)
    xm, rm, _ = pm.solve_refined(b, tol=1e-12, maxiter=10, precise=True, mixed=True)
    pt.close()
    pm.close()
    assert rt <= 1e-12 and rm <= 1e-12, (rt, rm)
    rel = float(((xt - xm).norm(dim=1) / xm.norm(dim=1)).max())
    assert rel <= 1e-9, rel


def test_seventh_slice_shrinks_inner_solve_error():
    """One unrefined mixed solve: each slice adds 7 bits, so 7 slices leave
    a residual about two orders of magnitude below 6 (the diagnostics on
    this matrix give ratios of about 100 per slice)."""
    from dplr_gb300 import gen_gpu
    t = gen_gpu.kernel_tree_2d(n=16384, leaf=128, rmax=96, seed=6)
    g = torch.Generator(device="cpu").manual_seed(3)
    b = torch.randn(16, t.size, generator=g, dtype=torch.float64).cuda()
    res = {}
    for ns in (5, 6, 7):
        p = _plan(t, mma=False, mixed_slices=ns)
        _, res[ns], _ = p.solve_refined(b, tol=1e-30, maxiter=0, precise=True, mixed=True, strict=False)
        p.close()
    assert res[6] < res[5] / 20 and res[7] < res[6] / 20, res


def test_tensor_core_capacitance_matches_fp64():
    """Nodes with two rank-128 blocks apply K^-1 from 8 exact slices on the
    tensor cores; the refined solves with it and with FP64 capacitance both
    reach the tolerance and agree, and one unrefined inner solve is as
    accurate either way."""
    from dplr_gb300 import gen_gpu
    from dplr_gb300.plan import GpuPlan
    t = gen_gpu.kernel_tree_2d(n=16384, leaf=128, rmax=128, seed=6)
    assert max(tree.ranks_by_level(t)) == 128
    g = torch.Generator(device="cpu").manual_seed(4)
    b = torch.randn(70, t.size, generator=g, dtype=torch.float64).cuda()
    out = {}
    for fp64 in (False, True):
        p = GpuPlan(t)
        p.factor()
        p.prepare_sliced()
        p.prepare_mixed(7, fp64_capacitance=fp64)
        _, r0, _ = p.solve_refined(b, tol=1e-30, maxiter=0, precise=True, mixed=True, strict=False)
        x, r, _ = p.solve_refined(b, tol=1e-12, maxiter=10, precise=True, mixed=True)
        out[fp64] = (x, r, r0)
        p.close()
    (xt, rt, r0t), (xf, rf, r0f) = out[False], out[True]
    assert rt <= 1e-12 and rf <= 1e-12, (rt, rf)
    assert float(((xt - xf).norm(dim=1) / xf.norm(dim=1)).max()) <= 1e-9
    assert r0t <= 4 * r0f and r0f <= 4 * r0t, (r0t, r0f)


def test_tcgen05_residual_of_a_small_block_batch():
    """A batch of leaf-64, rank <= 4 trees (as the 512-matrix workload) on
    the tcgen05 residual: every matrix's rows against the exact residual of
    its own tree, and against the mma.sync kernels."""
    import os
    from dplr_gb300.plan import GpuPlan
    trees = [gen.random_tree(1024, 64, [2, 4, 1, 3], seed=21), gen.random_tree(2048, 64, [1, 1, 4, 2, 3], seed=22),
             gen.random_tree(1024, 64, [3, 0, 2, 1], seed=23)]
    rng = np.random.default_rng(24)
    m = sum(t.size for t in trees)
    x = rng.standard_normal((5, m))
    b = rng.standard_normal((5, m))
    out = {}
    for mma in (False, True):
        old = os.environ.get("DPLR_GB300_SLICED_MMA")
        os.environ["DPLR_GB300_SLICED_MMA"] = "1" if mma else "0"
        try:
            p = GpuPlan.batch(trees)
            p.prepare_sliced()
        finally:
            if old is None:
                del os.environ["DPLR_GB300_SLICED_MMA"]
            else:
                os.environ["DPLR_GB300_SLICED_MMA"] = old
        out[mma] = p.residual(torch.tensor(x, device="cuda"), torch.tensor(b, device="cuda"),
                              precise=True).cpu().numpy()
        p.close()
    o = 0
    for t in trees:
        n = t.size
        want = exact_residual(t, x[:, o:o + n], b[:, o:o + n])
        nax = float(np.linalg.norm((b[:, o:o + n] - want).astype(np.float64)))
        for mma in (False, True):
            err = float(np.linalg.norm((out[mma][:, o:o + n] - want).astype(np.float64))) / nax
            assert err <= 1e-15, (mma, err)
        o += n
