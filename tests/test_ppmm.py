"""PLR x PLR product dplrgeppmm (src/dplrppmm.c:998).

The fixtures under tests/golden/ppmm hold C after the reference's own
dplrgeppmm for all four (transa, transb) and several (alpha, beta, eps).
On the CPU the oracle restatement (oracle/ppmm.py) is pinned against them;
on a GPU the library's dplrgeppmm is held to the fixtures and to the
oracle on larger trees.  Structure, ranks and capacities must be equal;
values agree to rounding.
"""
import glob
import os

import numpy as np
import pytest

import golden_io
from dplr_gb300 import gen, tree
from oracle import ppmm as oppmm

PPMM = sorted(glob.glob(os.path.join(golden_io.GOLDEN, "ppmm", "*.npz")))


def _cases():
    out = []
    for path in PPMM:
        rec = golden_io.load(path)
        for k in sorted(rec):
            if k.endswith("_cfg"):
                out.append((os.path.basename(path)[:-4], k[:-4]))
    return out


CASES = _cases()
_recs: dict = {}


def _rec(name):
    if name not in _recs:
        _recs[name] = golden_io.load(os.path.join(golden_io.GOLDEN, "ppmm", name + ".npz"))
    return _recs[name]


def _inputs(rec):
    return [tree.unflatten(rec[f"{k}_meta"], rec[f"{k}_data"]) for k in ("A", "B", "C")]


def _cfg(rec, case):
    ta, tb, al, be, ep = rec[case + "_cfg"]
    return chr(int(ta)), chr(int(tb)), float(al), float(be), float(ep)


def assert_trees_match(got, want, rtol=1e-12, path=""):
    """Same node types, sizes, ranks and capacities; values to rounding
    (relative to the largest magnitude of the node's arrays)."""
    assert type(got) is type(want), path
    assert got.size == want.size, path
    if isinstance(want, tree.HNode):
        for k in ("nw", "ne", "se", "sw"):
            assert_trees_match(getattr(got, k), getattr(want, k), rtol, path + k + "/")
        return
    if isinstance(want, tree.LowRank):
        assert got.rank == want.rank, (path, got.rank, want.rank)
        assert got.capacity == want.capacity, (path, got.capacity, want.capacity)
        pairs = [(got.u, want.u), (got.v, want.v), (got.sig, want.sig)]
    else:
        pairs = [(got.d, want.d)]
    for g, w in pairs:
        scale = max(1.0, float(np.abs(w).max())) if w.size else 1.0
        np.testing.assert_allclose(g, w, rtol=0, atol=rtol * scale, err_msg=path)


@pytest.mark.parametrize("name,case", CASES, ids=[f"{n}-{c}" for n, c in CASES])
def test_oracle_matches_reference_ppmm(name, case):
    rec = _rec(name)
    a, b, c = _inputs(rec)
    ta, tb, al, be, ep = _cfg(rec, case)
    oppmm.geppmm(ta, tb, al, a, b, be, c, ep)
    want = tree.unflatten(rec[case + "_meta"], rec[case + "_data"])
    assert_trees_match(c, want)


def test_oracle_product_is_the_dense_product():
    """With eps = 0 nothing is dropped: to_dense(C) = alpha op(A) op(B) + beta C."""
    a = gen.random_tree(128, 16, [5, 3, 2], seed=31, diag_shift=2.0)
    b = gen.random_tree(128, 16, [2, 4, 3], seed=32, diag_shift=2.0)
    c0 = gen.random_tree(128, 16, [3, 1, 2], seed=33, diag_shift=2.0)
    da, db, dc = tree.to_dense(a), tree.to_dense(b), tree.to_dense(c0)
    for ta in "NT":
        for tb in "NT":
            c = gen.random_tree(128, 16, [3, 1, 2], seed=33, diag_shift=2.0)
            oppmm.geppmm(ta, tb, 0.7, a, b, -0.3, c, 0.0)
            opa = da.T if ta == "T" else da
            opb = db.T if tb == "T" else db
            np.testing.assert_allclose(tree.to_dense(c), 0.7 * opa @ opb - 0.3 * dc, atol=1e-11 * 128)


def test_oracle_rejects_mismatched_structures():
    a = gen.random_tree(128, 16, 2, seed=1)
    b = gen.random_tree(128, 32, 2, seed=2)
    with pytest.raises(ValueError):
        oppmm.geppmm("N", "N", 1.0, a, b, 0.0, gen.random_tree(128, 16, 2, seed=3), 1e-8)


# ---------------------------------------------------------------- GPU -----

def _gpu_ppmm(ta, tb, al, a, b, be, c, ep):
    from dplr_gb300 import _native
    api = _native.api()
    ca, cb, cc = tree.to_c(a), tree.to_c(b), tree.to_c(c)
    try:
        api.geppmm(ta, tb, a.size, al, ca, cb, be, cc, ep)
        return tree.from_c(cc)
    finally:
        for p in (ca, cb, cc):
            tree.free_c(p)


@pytest.mark.gpu
@pytest.mark.parametrize("name,case", CASES, ids=[f"{n}-{c}" for n, c in CASES])
def test_gpu_matches_reference_ppmm(name, case):
    rec = _rec(name)
    a, b, c = _inputs(rec)
    ta, tb, al, be, ep = _cfg(rec, case)
    got = _gpu_ppmm(ta, tb, al, a, b, be, c, ep)
    want = tree.unflatten(rec[case + "_meta"], rec[case + "_data"])
    assert_trees_match(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_gpu_matches_oracle_on_larger_trees(ta, tb):
    """1024 x 1024, leaves of 64 (four levels), uneven ranks with rank-0
    blocks, spare capacity: ranks, capacities and columns as the oracle's."""
    a = gen.random_tree(1024, 64, [9, 0, 5, 7], seed=41, capacity_extra=2, diag_shift=3.0)
    b = gen.random_tree(1024, 64, [3, 6, 6, 1], seed=42, diag_shift=3.0)
    c = gen.random_tree(1024, 64, [4, 2, 0, 3], seed=43, capacity_extra=5, diag_shift=3.0)
    got = _gpu_ppmm(ta, tb, -0.6, a, b, 1.7, c, 1e-9)
    oppmm.geppmm(ta, tb, -0.6, a, b, 1.7, c, 1e-9)
    assert_trees_match(got, c, rtol=1e-11)


@pytest.mark.gpu
def test_gpu_product_is_the_dense_product():
    a = gen.random_tree(512, 64, [6, 4, 3], seed=51, diag_shift=2.0)
    b = gen.random_tree(512, 64, [2, 5, 3], seed=52, diag_shift=2.0)
    c = gen.random_tree(512, 64, [3, 3, 1], seed=53, diag_shift=2.0)
    da, db, dc = tree.to_dense(a), tree.to_dense(b), tree.to_dense(c)
    for ta in "NT":
        for tb in "NT":
            got = _gpu_ppmm(ta, tb, 1.3, a, b, 0.4, c, 0.0)
            opa = da.T if ta == "T" else da
            opb = db.T if tb == "T" else db
            want = 1.3 * opa @ opb + 0.4 * dc
            assert np.abs(tree.to_dense(got) - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.gpu
def test_gpu_rejects_mismatched_structures_and_leaves_c_untouched():
    from dplr_gb300 import _native
    lib = _native.lib()
    a = gen.random_tree(256, 32, 2, seed=1)
    b = gen.random_tree(256, 64, 2, seed=2)       # one level fewer
    c = gen.random_tree(256, 32, 2, seed=3)
    ca, cb, cc = tree.to_c(a), tree.to_c(b), tree.to_c(c)
    try:
        rc = lib.dplr_gpu_geppmm(b"N", b"N", 256, 1.0, ca, cb, 0.0, cc, 1e-8, None)
        assert rc == -1 and "do not match" in _native.last_error()
        assert tree.trees_close(tree.from_c(cc), c, rtol=0.0)
        rc = lib.dplr_gpu_geppmm(b"N", b"N", -4, 1.0, ca, ca, 0.0, cc, 1e-8, None)
        assert rc == -1 and "invalid matrix size" in _native.last_error()
    finally:
        for p in (ca, cb, cc):
            tree.free_c(p)


def _with_nan_leaf(t):
    """Copy of t with NaN in its first leaf."""
    m, d = tree.flatten(t)
    out = tree.unflatten(m, d.copy())
    node = out
    while isinstance(node, tree.HNode):
        node = node.nw
    node.d[0, 0] = np.nan
    return out


def test_oracle_alpha_zero_does_not_read_a_or_b():
    a = _with_nan_leaf(gen.random_tree(128, 16, 3, seed=61))
    b = gen.random_tree(128, 16, 2, seed=62)
    c = gen.random_tree(128, 16, 2, seed=63)
    dc = tree.to_dense(c)
    oppmm.geppmm("N", "N", 0.0, a, b, 0.5, c, 1e-8)
    np.testing.assert_allclose(tree.to_dense(c), 0.5 * dc, rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_gpu_alpha_zero_does_not_read_a_or_b():
    a = _with_nan_leaf(gen.random_tree(256, 32, 3, seed=61))
    b = gen.random_tree(256, 32, 2, seed=62)
    c = gen.random_tree(256, 32, [2, 0, 1], seed=63, capacity_extra=1)
    got = _gpu_ppmm("T", "N", 0.0, a, b, -0.5, c, 1e-8)
    oppmm.geppmm("T", "N", 0.0, a, b, -0.5, c, 1e-8)
    assert np.isfinite(tree.to_dense(got)).all()
    assert_trees_match(got, c, rtol=1e-14)


def test_bench_cpu_leg_times_the_restatement_and_compares():
    """bench.py's CPU leg of the product workload: one product by the
    restatement on the given input, and its difference from a product."""
    import copy

    import bench
    from dplr_gb300 import workloads
    a = gen.random_tree(256, 32, [5, 3, 2], seed=71, diag_shift=2.0)
    want = copy.deepcopy(a)
    oppmm.geppmm("N", "N", 1.0, a, a, 0.5, want, workloads.PPMM["eps"])
    cb, diff = bench.ppmm_cpu_leg(a, want)
    assert cb["kind"] == "port" and cb["value"] > 0 and diff == 0.0
