"""Structure arithmetic on device-resident plans (csrc/devops.cu) against the
host drop-ins (dplrcpy, dplraxpy, dplrgep2d), which are themselves checked
node by node against the reference's C (tests/test_host_ops.py).
"""
import numpy as np
import pytest

from dplr_gb300 import gen, tree

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _pool_tree(plan, like):
    """The plan's factors as a Python tree shaped like `like` (ranks from the
    plan), read back from the device pool."""
    pool = plan.read_pool().cpu().numpy()
    blocks = iter(plan.pool_blocks())
    lr = [b for b in plan.pool_blocks() if b["kind"] == "lowrank"]
    lf = [b for b in plan.pool_blocks() if b["kind"] == "leaf"]
    del blocks
    it_lr, it_lf = iter(lr), iter(lf)

    def walk(node):
        if isinstance(node, tree.Dense):
            b = next(it_lf)
            n = b["b"]
            return tree.Dense(pool[b["d"]:b["d"] + n * n].reshape(n, n, order="F"))
        out = []
        for blk in (next(it_lr), next(it_lr)):
            n, r = blk["n"], blk["rank"]
            out.append(tree.LowRank(pool[blk["u"]:blk["u"] + n * r].reshape(n, r, order="F"),
                                    pool[blk["sig"]:blk["sig"] + r].copy(),
                                    pool[blk["v"]:blk["v"] + n * r].reshape(n, r, order="F")))
        return tree.HNode(walk(node.nw), out[0], walk(node.se), out[1])

    return walk(like)


def _same(a, b, exact=True):
    if isinstance(a, tree.HNode):
        for k in ("nw", "ne", "se", "sw"):
            _same(getattr(a, k), getattr(b, k), exact)
        return
    pairs = [(a.d, b.d)] if isinstance(a, tree.Dense) else [(a.u, b.u), (a.v, b.v), (a.sig, b.sig)]
    if isinstance(a, tree.LowRank):
        assert a.rank == b.rank
    for x, y in pairs:
        if exact:
            assert np.array_equal(x, y)
        else:
            np.testing.assert_allclose(x, y, rtol=2.3e-16, atol=0)


def test_plan_copy_is_exact():
    from dplr_gb300.plan import GpuPlan
    t = gen.random_tree(1024, 64, [9, 0, 4, 2], seed=1)
    p = GpuPlan(t)
    c = p.copy()
    assert torch.equal(c.read_pool(), p.read_pool())
    x = torch.randn(3, t.size, dtype=torch.float64, device="cuda")
    assert torch.equal(c.apply(x), p.apply(x))
    _same(_pool_tree(c, t), t)
    c.close()
    p.close()


@pytest.mark.parametrize("alpha", [1.5, -0.75, 0.0])
def test_axpy_matches_the_host_drop_in(alpha):
    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan
    ta = gen.random_tree(1024, 64, [7, 3, 0, 2], seed=2)
    tb = gen.random_tree(1024, 64, [5, 6, 1, 0], seed=3)
    pa, pb = GpuPlan(ta), GpuPlan(tb)
    pc = pa.axpy(alpha, pb)
    a, b = tree.to_c(ta), tree.to_c(tb)
    _native.api().axpy(ta.size, alpha, a, b)          # host dplraxpy: b := alpha a + b
    want = tree.from_c(b)
    tree.free_c(a)
    tree.free_c(b)
    got = _pool_tree(pc, tb)
    _same(got, want, exact=False)
    # the device result applies as the host one
    x = torch.randn(2, ta.size, dtype=torch.float64, device="cuda")
    y = pc.apply(x).cpu().numpy()
    yw = (tree.to_dense(want) @ x.cpu().numpy().T).T
    assert np.linalg.norm(y - yw) <= 1e-13 * np.linalg.norm(yw)
    for p in (pa, pb, pc):
        p.close()


def test_gep2d_is_the_dense_matrix():
    from dplr_gb300.plan import GpuPlan
    t = gen.random_tree(768, 48, [11, 5, 2, 1], seed=4)
    p = GpuPlan(t)
    d = p.to_dense().cpu().numpy().T          # row j of the tensor is column j
    want = tree.to_dense(t)
    assert np.max(np.abs(d - want)) <= 1e-14 * np.max(np.abs(want))
    p.close()


def test_gep2d_of_a_batch_is_block_diagonal():
    from dplr_gb300.plan import GpuPlan
    trees = [gen.random_tree(256, 32, [3, 2], seed=5), gen.random_tree(512, 64, [4, 1, 2], seed=6)]
    p = GpuPlan.batch(trees)
    d = p.to_dense().cpu().numpy().T
    want = np.zeros((768, 768))
    want[:256, :256] = tree.to_dense(trees[0])
    want[256:, 256:] = tree.to_dense(trees[1])
    assert np.max(np.abs(d - want)) <= 1e-14 * np.max(np.abs(want))
    p.close()


def test_device_pipeline_scale_add_factor_solve():
    """A := 2 A; C := -0.5 A + B; factor and solve C; all on the device."""
    from dplr_gb300.plan import GpuPlan
    ta = gen.random_tree(1024, 64, [6, 4, 2, 1], seed=7)
    tb = gen.random_tree(1024, 64, [3, 3, 3, 3], seed=8, diag_shift=3000.0)
    pa, pb = GpuPlan(ta), GpuPlan(tb)
    pa.scal(2.0)
    pc = pa.axpy(-0.5, pb)
    pc.factor()
    b = torch.randn(4, ta.size, dtype=torch.float64, device="cuda")
    x, res, _ = pc.solve_refined(b, tol=1e-12, maxiter=5, precise=False)
    dense = (-1.0 * tree.to_dense(ta)) + tree.to_dense(tb)
    r = b.cpu().numpy() - (dense @ x.cpu().numpy().T).T
    assert np.max(np.linalg.norm(r, axis=1) / np.linalg.norm(b.cpu().numpy(), axis=1)) <= 1e-11
    for p in (pa, pb, pc):
        p.close()


def test_axpy_rejects_different_structures():
    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan
    pa = GpuPlan(gen.random_tree(1024, 64, [2, 2], seed=9))
    pb = GpuPlan(gen.random_tree(1024, 128, [2, 2], seed=9))
    with pytest.raises(_native.NativeError, match="structure"):
        pa.axpy(1.0, pb)
    pa.close()
    pb.close()
