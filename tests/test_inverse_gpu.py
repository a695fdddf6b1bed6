"""GPU dplrgeinv / dplrgeprk / dplrreduce against the CPU oracle.

The GPU inverse must reproduce DPLR's representation of inv(A): the same
tree, the same ranks and capacities (grown by the same dplrresizelr
steps), and every block product U diag(sig) V^T within 1e-12 of the
oracle's relative to the norm of the inverse (factor columns with
negligible singular values point in rounding-defined directions, so they
are compared through the products).
"""
import numpy as np
import pytest

import golden_io
from dplr_gb300 import gen, tree
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def caps(node, out=None):
    out = [] if out is None else out
    if isinstance(node, tree.HNode):
        out.append((node.ne.rank, node.ne.capacity, node.sw.rank, node.sw.capacity))
        caps(node.nw, out)
        caps(node.se, out)
    return out


TREES = {
    "rand": lambda: gen.random_tree(512, 32, [12, 8, 5, 3], seed=1),
    "uneven": lambda: gen.random_tree(1024, 64, [9, 0, 4, 2], seed=2, capacity_extra=3),
    "exp": lambda: gen.exp1d_tree(gen.sorted_uniform(1024, 3), 0.1, 1e-2, 64, 3, seed=3),
    "leaf_only": lambda: tree.Dense(np.random.default_rng(4).standard_normal((48, 48)) + 10 * np.eye(48)),
}


def run_inv(api, t, eps, reuse=None):
    a = tree.to_c(t)
    b = tree.new_empty() if reuse is None else reuse
    info = api.geinv(t.size, a, b, eps)
    out = tree.from_c(b) if info == 0 else None
    tree.free_c(a)
    return info, out, b


@pytest.mark.parametrize("name", list(TREES))
@pytest.mark.parametrize("eps", [0.0, 1e-8])
def test_geinv_matches_oracle(name, eps):
    from dplr_gb300 import _native
    gpu, orc = _native.api(), pyoracle.oracle("best")
    t = TREES[name]()
    ig, bg, cg = run_inv(gpu, t, eps)
    io, bo, co = run_inv(orc, t, eps)
    tree.free_c(cg)
    tree.free_c(co)
    assert ig == io == 0
    assert caps(bg) == caps(bo)
    # operator parity at 1e-12 of the inverse's norm; individual singular
    # values are an intermediate of two different rounding paths (DPLR
    # inverts X = S^-1 K, the GPU K), so they are held to 1e-10
    golden_io.compare_trees(bg, bo, 1e-12, sig_tol=1e-10, allow=2.0 * eps)
    if eps == 0.0:
        d = tree.to_dense(t)
        inv = tree.to_dense(bg)
        assert np.linalg.norm(inv @ d - np.eye(t.size)) / np.sqrt(t.size) < 1e-9


def test_geinv_reuses_output_tree():
    """A second call into the same B keeps DPLR's reuse semantics."""
    from dplr_gb300 import _native
    gpu, orc = _native.api(), pyoracle.oracle("best")
    t = TREES["rand"]()
    outs = []
    for api in (gpu, orc):
        _, _, b = run_inv(api, t, 0.0)
        _, second, b = run_inv(api, t, 0.0, reuse=b)
        outs.append(second)
        tree.free_c(b)
    assert caps(outs[0]) == caps(outs[1])
    golden_io.compare_trees(outs[0], outs[1], 1e-12, sig_tol=1e-10)


def test_geinv_singular_leaf_sets_info():
    from dplr_gb300 import _native
    gpu, orc = _native.api(), pyoracle.oracle("best")
    t = TREES["rand"]()
    leaf = t.se
    while isinstance(leaf, tree.HNode):
        leaf = leaf.nw
    leaf.d[:, 3] = 0.0
    infos = []
    for api in (gpu, orc):
        info, _, b = run_inv(api, t, 0.0)
        infos.append(info)
        tree.free_c(b)
    assert infos[0] > 0 and infos[0] == infos[1]


@pytest.mark.parametrize("alpha,eps", [(0.7, 1e-12), (-1.4, 1e-2), (2.0, 0.0)])
def test_geprk_matches_oracle(alpha, eps):
    from dplr_gb300 import _native
    gpu, orc = _native.api(), pyoracle.oracle("best")
    t = gen.random_tree(512, 32, [6, 3, 2, 1], seed=7, capacity_extra=1)
    m, k = t.size, 4
    rng = np.random.default_rng(8)
    u = rng.standard_normal((m + 3) * k)
    v = rng.standard_normal((m + 1) * k)
    s = np.abs(rng.standard_normal(2 * k))
    res = []
    for api in (gpu, orc):
        a = tree.to_c(t)
        api.geprk(m, k, alpha, u, m + 3, v, m + 1, s, 2, a, eps)
        res.append(tree.from_c(a))
        tree.free_c(a)
    assert caps(res[0]) == caps(res[1])
    golden_io.compare_trees(res[0], res[1], 1e-12)


def redundant_tree(n, leaf, rank, seed):
    """Blocks of nominal rank `rank` whose columns span only rank/2 directions
    plus 1e-13 noise, so that dortlr truncates them."""
    rng = np.random.default_rng(seed)

    def lr(h):
        base_u = np.linalg.qr(rng.standard_normal((h, rank // 2)))[0]
        base_v = np.linalg.qr(rng.standard_normal((h, rank // 2)))[0]
        mix = rng.standard_normal((rank // 2, rank))
        u = base_u @ mix + 1e-13 * rng.standard_normal((h, rank))
        v = base_v @ rng.standard_normal((rank // 2, rank))
        return tree.LowRank(u, np.abs(rng.standard_normal(rank)) + 0.5, v)

    def build(mm):
        if mm <= leaf:
            return tree.Dense(rng.standard_normal((mm, mm)))
        h = mm // 2
        return tree.HNode(build(h), lr(h), build(h), lr(h))
    return build(n)


@pytest.mark.parametrize("eps", [1e-6, 1e-2])
def test_reduce_matches_oracle(eps):
    from dplr_gb300 import _native
    gpu, orc = _native.api(), pyoracle.oracle("best")
    t = redundant_tree(512, 64, 8, seed=11)
    res = []
    for api in (gpu, orc):
        a = tree.to_c(t)
        api.reduce(t.size, a, eps)
        res.append(tree.from_c(a))
        tree.free_c(a)
    assert [r[0] for r in caps(res[0])] == [r[0] for r in caps(res[1])]
    golden_io.compare_trees(res[0], res[1], 1e-10)
    if eps <= 1e-6:
        # a tight threshold only drops the 1e-13 noise directions
        d0 = tree.to_dense(t)
        err = np.linalg.norm(tree.to_dense(res[0]) - d0) / np.linalg.norm(d0)
        assert err < 1e-6
