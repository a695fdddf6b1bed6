"""Batches of independent PLR matrices in one plan (block diagonal), CUDA
graph replay, and the autotuner.

Matrices of uneven size (512 to 4096 rows, leaf 64) and uneven rank (1 to 4,
1D exponential kernels with length scales in [0.05, 0.5]) are applied and
solved together; every matrix's block of the result must match the same
matrix planned alone and the dense product.
"""
import numpy as np
import pytest

from dplr_gb300 import gen, tree

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _trees(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = 64 << int(rng.integers(3, 7))
        x = np.sort(rng.uniform(0.0, 1.0, n))
        out.append(gen.exp1d_tree(x, ell=float(rng.uniform(0.05, 0.5)), shift=1e-2, leaf=64,
                                  rank=int(rng.integers(1, 5)), seed=seed * 1000 + i))
    return out


def _rhs(m, n, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(n, m, generator=g, dtype=torch.float64).cuda()


def test_batch_apply_and_solve_match_single_plans():
    from dplr_gb300.plan import GpuPlan
    trees = _trees(12, 1)
    batch = GpuPlan.batch(trees)
    offs = batch.offsets()
    assert offs[0] == 0 and len(offs) == len(trees)
    assert batch.m == sum(t.size for t in trees)
    X = _rhs(batch.m, 7, 2)
    Y = batch.apply(X)
    batch.factor(transposed=True)
    S = batch.solve(X)
    St = batch.solve(X, trans="T")
    for t, o in zip(trees, offs):
        xs = X[:, o:o + t.size].contiguous()
        single = GpuPlan(t)
        ys = single.apply(xs)
        single.factor(transposed=True)
        ss = single.solve(xs)
        sts = single.solve(xs, trans="T")
        dense = tree.to_dense(t)
        want = (dense @ xs.cpu().numpy().T).T
        got = Y[:, o:o + t.size].cpu().numpy()
        assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))
        assert torch.allclose(Y[:, o:o + t.size], ys, rtol=1e-14, atol=0)
        # The batch sweeps its levels with the batch-wide level width, so its
        # kernels sum in another order than the single plan's; the Woodbury
        # sweep amplifies that rounding difference.  Both are solves of the
        # same matrix: compare norm-wise and check each one's residual.
        for got_s, want_s, tr in ((S[:, o:o + t.size], ss, "N"), (St[:, o:o + t.size], sts, "T")):
            rel = float(((got_s - want_s).norm(dim=1) / want_s.norm(dim=1)).max())
            assert rel <= 1e-9, rel
            r = xs - single.apply(got_s.contiguous(), trans=tr)
            assert float((r.norm(dim=1) / xs.norm(dim=1)).max()) <= 1e-9
        single.close()
    x, res, its = batch.solve_refined(X, tol=1e-12, maxiter=6, precise=False)
    assert res <= 1e-12
    batch.close()


def test_graph_replay_matches_direct_calls():
    from dplr_gb300.plan import GpuGraph, GpuPlan
    trees = _trees(8, 3)
    batch = GpuPlan.batch(trees)
    batch.factor()
    X = _rhs(batch.m, 5, 4)
    Yd = batch.apply(X)
    Sd = batch.solve(X)
    Y = torch.zeros_like(X)
    S = torch.zeros_like(X)
    ga = GpuGraph(batch, "A", X, Y)
    gs = GpuGraph(batch, "S", X, S)
    assert ga.kernels >= 1 and gs.kernels >= 3        # the apply is one persistent launch
    for _ in range(3):
        Y.zero_()
        S.zero_()
        ga.launch()
        gs.launch()
        torch.cuda.synchronize()
        assert torch.equal(Y, Yd)
        assert torch.equal(S, Sd)
    # replay reads the current contents of x
    X.mul_(2.0)
    ga.launch()
    torch.cuda.synchronize()
    assert torch.allclose(Y, 2.0 * Yd, rtol=1e-15, atol=0)
    ga.close()
    gs.close()
    batch.close()


def test_autotune_keeps_results():
    from dplr_gb300.plan import GpuPlan
    trees = _trees(6, 5)
    batch = GpuPlan.batch(trees)
    X = _rhs(batch.m, 9, 6)
    before = batch.apply(X)
    cfg = batch.autotune(9)
    assert cfg["chunk_rows"] in (256, 512, 1024, 2048) and cfg["nb_cap"] in (1, 2, 4, 8, 16)
    assert cfg["apply_ms"] > 0
    after = batch.apply(X)
    # another chunk length sums the panels in another order: rounding-level changes only
    assert float((before - after).abs().max()) <= 1e-14 * float(before.abs().max())
    batch.factor()
    s = batch.solve(X)
    r = batch.residual(s, X, precise=False)
    assert float((r.norm(dim=1) / X.norm(dim=1)).max()) <= 1e-10
    batch.close()


def test_refined_solve_converges_per_matrix():
    """The refined solve of a batch measures every column over each
    matrix's own rows: the residual it reports is the largest per-matrix
    relative residual (as for each matrix solved alone), not that of the
    stacked column, which a matrix with a small right-hand side would not
    move."""
    from dplr_gb300.plan import GpuPlan
    trees = _trees(4, 3)
    batch = GpuPlan.batch(trees)
    batch.factor()
    offs = batch.offsets()
    b = _rhs(batch.m, 2, 7)
    b[:, offs[1]:offs[1] + trees[1].size] *= 1e-6
    # no correction: the reported residual is that of the first solve
    x, res, its = batch.solve_refined(b, tol=0.0, maxiter=0, precise=False, strict=False)
    assert its == 0
    r = batch.residual(x, b, precise=False)
    per = []
    for o, t in zip(offs, trees):
        rr, bb = r[:, o:o + t.size], b[:, o:o + t.size]
        per.append(float((rr.norm(dim=1) / bb.norm(dim=1)).max()))
    stacked = float((r.norm(dim=1) / b.norm(dim=1)).max())
    assert abs(res - max(per)) <= 1e-9 * max(per), (res, per, stacked)
    assert max(per) >= stacked * (1.0 - 1e-12)
    # refined to the tolerance, every matrix meets it
    x, res, _ = batch.solve_refined(b, tol=1e-11, maxiter=6, precise=False)
    r = batch.residual(x, b, precise=False)
    for o, t in zip(offs, trees):
        rr, bb = r[:, o:o + t.size], b[:, o:o + t.size]
        assert float((rr.norm(dim=1) / bb.norm(dim=1)).max()) <= 1e-11
    batch.close()


@pytest.mark.parametrize("op,corrections", [("C", 1), ("R", 2)])
def test_refined_graph_replays_the_refined_solve(op, corrections):
    """Graph ops 'C' and 'R' replay the solve with one or two correction
    steps (FP64 residuals, no host synchronisation inside): bit for bit the
    iterates of dplr_gpu_solve_refined stopped after as many corrections."""
    from dplr_gb300.plan import GpuGraph, GpuPlan
    trees = _trees(6, 5)
    batch = GpuPlan.batch(trees)
    batch.factor()
    X = _rhs(batch.m, 4, 9)
    want, _, its = batch.solve_refined(X, tol=0.0, maxiter=corrections, precise=False, strict=False)
    assert its == corrections
    Y = torch.zeros_like(X)
    g = GpuGraph(batch, op, X, Y)
    for _ in range(2):
        Y.zero_()
        g.launch()
        torch.cuda.synchronize()
        assert torch.equal(Y, want)
    g.close()
    batch.close()
