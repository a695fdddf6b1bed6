"""SVD-based recompression (dplr_gpu_reduce_svd), the alternative to
dplrreduce's Gram-Schmidt with dplrreduce's thresholds (eps/4 per level,
src/dplrreduce.c:46).

The restatement (oracle/recompress.py) is pinned on the CPU to the
definition: every block becomes its exact SVD truncated below the block's
threshold.  The GPU is held to the restatement: equal ranks and
capacities, singular values and blocks to rounding.
"""
import numpy as np
import pytest

from dplr_gb300 import gen, tree
from oracle import recompress as orec


def _doubled(t):
    """t with every low-rank block written twice side by side: the same
    matrix times 2 at twice the rank (what an append without
    recompression produces)."""
    if isinstance(t, tree.HNode):
        def dup(L):
            return tree.LowRank(np.hstack([L.u, L.u]), np.concatenate([L.sig, L.sig]),
                                np.hstack([L.v, L.v]), capacity=2 * L.rank + 3)
        return tree.HNode(_doubled(t.nw), dup(t.ne), _doubled(t.se), dup(t.sw))
    return tree.Dense(2.0 * t.d)


def _blocks(t, out=None, eps=None, e=None):
    """[(block, threshold)] in pre-order, thresholds eps/4 per level."""
    out = [] if out is None else out
    if isinstance(t, tree.HNode):
        e2 = (eps if e is None else e) / 4.0
        out += [(t.ne, e2), (t.sw, e2)]
        _blocks(t.nw, out, eps, e2)
        _blocks(t.se, out, eps, e2)
    return out


def assert_same_blocks(got, want, tol):
    for (g, _), (w, _) in zip(_blocks(got, eps=1.0), _blocks(want, eps=1.0)):
        assert g.rank == w.rank and g.capacity == w.capacity
        if w.rank:
            scale = max(1.0, float(w.sig[0]))
            np.testing.assert_allclose(g.sig, w.sig, rtol=0, atol=tol * scale)
            np.testing.assert_allclose((g.u * g.sig) @ g.v.T, (w.u * w.sig) @ w.v.T, rtol=0, atol=tol * scale)


# ---------------------------------------------------------------- CPU -----

def test_restatement_is_the_truncated_svd_of_every_block():
    t = _doubled(gen.random_tree(256, 32, [7, 5, 3], seed=3, diag_shift=2.0))
    eps = 1e-6
    r = orec.reduce_svd(t, eps)
    for (L, thr), (R, _) in zip(_blocks(t, eps=eps), _blocks(r, eps=eps)):
        s = np.linalg.svd((L.u * L.sig) @ L.v.T, compute_uv=False)
        keep = s[s >= thr]
        assert R.rank == len(keep) == L.rank // 2          # the doubled columns collapse
        np.testing.assert_allclose(R.sig, keep, rtol=1e-12)
        assert R.capacity == L.capacity
    np.testing.assert_allclose(tree.to_dense(r), tree.to_dense(t), atol=1e-12)


def test_restatement_drops_columns_below_the_threshold():
    t = gen.random_tree(256, 32, 8, seed=4, decay=0.1)    # sig decays by 10x per column
    r = orec.reduce_svd(t, 1e-2)
    assert max(tree.ranks_by_level(r)) < max(tree.ranks_by_level(t))
    err = np.abs(tree.to_dense(r) - tree.to_dense(t)).max()
    assert err <= 1e-2


# ---------------------------------------------------------------- GPU -----

def _gpu(t, eps, workers=0):
    from dplr_gb300 import compress
    return compress.reduce_svd(t, eps, workers)


@pytest.mark.gpu
@pytest.mark.parametrize("eps", [1e-9, 1e-4, 1e-1])
def test_gpu_matches_restatement(eps):
    t = _doubled(gen.random_tree(1024, 64, [9, 7, 5, 3], seed=5, diag_shift=2.0, decay=0.3))
    got = _gpu(t, eps)
    assert_same_blocks(got, orec.reduce_svd(t, eps), tol=1e-12)
    for g, w in zip([g for g, _ in _blocks(got, eps=1.0)], [w for w, _ in _blocks(t, eps=1.0)]):
        assert g.rank <= w.rank


@pytest.mark.gpu
def test_gpu_handles_rank_above_block_size():
    """Blocks of 16 rows carrying 40 columns (as products and appends leave
    them): k = min(n, r) = 16 singular values at most."""
    rng = np.random.default_rng(8)

    def lr(n, r):
        return tree.LowRank(rng.standard_normal((n, r)), np.abs(rng.standard_normal(r)) + 0.1,
                            rng.standard_normal((n, r)), capacity=r + 2)

    t = tree.HNode(tree.Dense(rng.standard_normal((16, 16))), lr(16, 40),
                   tree.Dense(rng.standard_normal((16, 16))), lr(16, 40))
    got = _gpu(t, 1e-10)
    assert got.ne.rank == 16 and got.sw.rank == 16
    assert_same_blocks(got, orec.reduce_svd(t, 1e-10), tol=1e-11)
    np.testing.assert_allclose(tree.to_dense(got), tree.to_dense(t), atol=1e-10)


@pytest.mark.gpu
def test_gpu_bounds_the_rank_growth_of_a_product():
    """C = A A of a compressed kernel grows ranks by appending; the SVD
    recompression brings them back down within the threshold."""
    from dplr_gb300 import _native, workloads
    a = gen.compress_dense(workloads.gauss2d_dense(512, seed=2), 1e-10, 3)
    api = _native.api()
    ca, cc = tree.to_c(a), tree.to_c(a)
    try:
        api.geppmm("N", "N", 512, 1.0, ca, ca, 0.0, cc, 1e-12)
        c = tree.from_c(cc)
    finally:
        tree.free_c(ca)
        tree.free_c(cc)
    r = _gpu(c, 1e-8, workers=3)
    assert max(tree.ranks_by_level(r)) < max(tree.ranks_by_level(c))
    assert np.abs(tree.to_dense(r) - tree.to_dense(c)).max() <= 1e-8 * 3
    assert_same_blocks(r, orec.reduce_svd(c, 1e-8), tol=1e-11)


@pytest.mark.gpu
def test_batched_kernel_matches_the_library_path(monkeypatch):
    """Blocks of rank <= 64 take the batched kernel (Householder QR and
    one-sided Jacobi in one CTA per block), larger ones the library SVD.
    A tree with both: the result matches the restatement either way, and
    with DPLR_GB300_SVD_BATCH_RANK=0 (every block on the library) too; the
    kept columns are orthonormal."""
    t = _doubled(gen.random_tree(1024, 64, [40, 24, 12, 6], seed=6, diag_shift=2.0, decay=0.7))
    assert t.ne.rank == 80 and t.nw.ne.rank == 48        # library and batched blocks
    eps = 1e-6
    want = orec.reduce_svd(t, eps)
    got = _gpu(t, eps)
    assert_same_blocks(got, want, tol=1e-12)
    for g, _ in _blocks(got, eps=1.0):
        if g.rank:
            k = np.eye(g.rank)
            assert np.abs(g.u.T @ g.u - k).max() <= 1e-12
            assert np.abs(g.v.T @ g.v - k).max() <= 1e-12
    monkeypatch.setenv("DPLR_GB300_SVD_BATCH_RANK", "0")
    assert_same_blocks(_gpu(t, eps), want, tol=1e-12)


@pytest.mark.gpu
def test_batched_kernel_on_tall_repeated_and_zero_blocks():
    """The batched kernel at its edges: 2048 rows with every column
    repeated (the copies' reflectors fall below rounding and are skipped),
    a block whose sig are all zero, and eps = 0 (every singular value
    kept, the product unchanged)."""
    rng = np.random.default_rng(12)
    n = 2048
    u, v = rng.standard_normal((n, 8)), rng.standard_normal((n, 8))
    s = np.abs(rng.standard_normal(8)) + 0.5
    tall = tree.LowRank(np.hstack([u, u]), np.concatenate([s, s]), np.hstack([v, v]), capacity=18)
    zero = tree.LowRank(rng.standard_normal((n, 5)), np.zeros(5), rng.standard_normal((n, 5)), capacity=5)
    t = tree.HNode(tree.Dense(rng.standard_normal((n, n))), tall, tree.Dense(rng.standard_normal((n, n))), zero)
    got = _gpu(t, 1e-8)
    assert got.ne.rank == 8 and got.sw.rank == 0
    assert_same_blocks(got, orec.reduce_svd(t, 1e-8), tol=1e-12)
    small = _doubled(gen.random_tree(256, 32, [6, 4, 3], seed=9, diag_shift=2.0))
    got0 = _gpu(small, 0.0)
    for (g, _), (w, _) in zip(_blocks(got0, eps=1.0), _blocks(small, eps=1.0)):
        assert g.rank == w.rank
    dense = tree.to_dense(small)
    assert np.abs(tree.to_dense(got0) - dense).max() <= 1e-12 * np.abs(dense).max()


@pytest.mark.gpu
def test_gpu_rejects_invalid_arguments():
    from dplr_gb300 import _native
    lib = _native.lib()
    c = tree.to_c(gen.random_tree(64, 16, 2, seed=1))
    try:
        assert lib.dplr_gpu_reduce_svd(-1, c, 1e-8, 0) == -1
        assert lib.dplr_gpu_reduce_svd(64, c, -1.0, 0) == -1
        assert lib.dplr_gpu_reduce_svd(32, c, 1e-8, 0) == -1
    finally:
        tree.free_c(c)


# ----------------------------------------------------- device plans -------

def _plan_tree(plan, like):
    """Blocks of a plan read back from its pool, shaped like `like`."""
    pool = plan.read_pool().cpu().numpy()
    blocks = plan.pool_blocks()
    lr = iter([b for b in blocks if b["kind"] == "lowrank"])
    lf = iter([b for b in blocks if b["kind"] == "leaf"])

    def walk(node):
        if isinstance(node, tree.Dense):
            b = next(lf)
            n = b["b"]
            return tree.Dense(pool[b["d"]:b["d"] + n * n].reshape(n, n, order="F"))
        out = []
        for blk in (next(lr), next(lr)):
            n, r = blk["n"], blk["rank"]
            out.append(tree.LowRank(pool[blk["u"]:blk["u"] + n * r].reshape(n, r, order="F"),
                                    pool[blk["sig"]:blk["sig"] + r].copy(),
                                    pool[blk["v"]:blk["v"] + n * r].reshape(n, r, order="F")))
        return tree.HNode(walk(node.nw), out[0], walk(node.se), out[1])

    return walk(like)


@pytest.mark.gpu
@pytest.mark.parametrize("eps", [1e-9, 1e-4])
def test_plan_recompression_matches_the_host_tree_one(eps):
    """dplr_gpu_plan_reduce_svd on a device plan gives the blocks
    dplr_gpu_reduce_svd gives on the host tree (same ranks, same truncated
    products), with no host round trip."""
    from dplr_gb300.plan import GpuPlan
    t = _doubled(gen.random_tree(1024, 64, [9, 7, 5, 3], seed=5, diag_shift=2.0, decay=0.3))
    p = GpuPlan(t)
    r = p.reduce_svd(eps)
    got = _plan_tree(r, t)
    want = _gpu(t, eps)
    for (g, _), (w, _) in zip(_blocks(got, eps=1.0), _blocks(want, eps=1.0)):
        assert g.rank == w.rank
        if w.rank:
            scale = max(1.0, float(w.sig[0]))
            np.testing.assert_allclose(g.sig, w.sig, rtol=0, atol=1e-12 * scale)
            np.testing.assert_allclose((g.u * g.sig) @ g.v.T, (w.u * w.sig) @ w.v.T, rtol=0, atol=1e-12 * scale)
    x = np.random.default_rng(0).standard_normal((3, t.size))
    import torch
    y = r.apply(torch.tensor(x, device="cuda")).cpu().numpy()
    yw = (tree.to_dense(want) @ x.T).T
    assert np.linalg.norm(y - yw) <= 1e-12 * np.linalg.norm(yw)
    p.close()
    r.close()


@pytest.mark.gpu
def test_recompression_after_rank_growing_operations():
    """Off by default (DPLR never recompresses): dplraxpy of A into a copy of
    A doubles every rank.  With dplr_gpu_set_recompress(eps) the host drop-in
    and the device dplr_gpu_axpy both return the recompressed sum 2 A, at A's
    ranks."""
    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan
    lib, api = _native.lib(), _native.api()
    a = gen.random_tree(512, 32, [6, 4, 3], seed=9, diag_shift=2.0, decay=0.3)
    ranks_a = tree.ranks_by_level(a)

    def host_axpy():
        ca, cb = tree.to_c(a), tree.to_c(a)
        api.axpy(a.size, 1.0, ca, cb)
        out = tree.from_c(cb)
        tree.free_c(ca)
        tree.free_c(cb)
        return out

    try:
        grown = host_axpy()
        assert tree.ranks_by_level(grown) == [2 * r for r in ranks_a]
        lib.dplr_gpu_set_recompress(1e-9)
        reduced = host_axpy()
        assert tree.ranks_by_level(reduced) == ranks_a
        np.testing.assert_allclose(tree.to_dense(reduced), 2.0 * tree.to_dense(a), atol=1e-11)
        pa = GpuPlan(a)
        pc = pa.axpy(1.0, pa)
        got = _plan_tree(pc, a)
        assert tree.ranks_by_level(got) == ranks_a
        np.testing.assert_allclose(tree.to_dense(got), 2.0 * tree.to_dense(a), atol=1e-11)
        pa.close()
        pc.close()
    finally:
        lib.dplr_gpu_set_recompress(-1.0)
