"""Host drop-ins dplrcpy / dplrscal / dplraxpy / dplradpy against the
reference's own C (src/dplrcpy.c, src/dplrscal.c, src/dplraxpy.c), built
from the reference sources into oracle/_ref where they are present.

Both libraries get separate C copies of the same seeded trees; the results
are read back and compared node by node: values (bit-exact except the dense
axpy, where the reference's BLAS daxpy may fuse the multiply-add), ranks,
capacities, and the messages of invalid calls.
"""
import numpy as np
import pytest

from dplr_gb300 import gen, tree
from oracle import pyoracle

ref = pyoracle.reference()
pytestmark = pytest.mark.skipif(ref is None or not ref.has("axpy"),
                                reason="reference sources not built here")


TREES = {
    "uniform": lambda s: gen.random_tree(256, 32, 6, seed=s),
    "uneven": lambda s: gen.random_tree(512, 32, [9, 0, 4, 7], seed=s, capacity_extra=2),
    "dense": lambda s: tree.Dense(np.random.default_rng(s).standard_normal((48, 48))),
}


def same(a, b, rtol=0.0):
    """Node-by-node equality of two Python trees (values, ranks, capacities)."""
    if type(a) is not type(b):
        return False
    if isinstance(a, tree.Dense):
        if not rtol:
            return np.array_equal(a.d, b.d)
        return np.allclose(a.d, b.d, rtol=rtol, atol=rtol * float(np.abs(b.d).max()))
    if isinstance(a, tree.LowRank):
        return (a.rank == b.rank and a.capacity == b.capacity and np.array_equal(a.u, b.u)
                and np.array_equal(a.v, b.v) and np.array_equal(a.sig, b.sig))
    return all(same(getattr(a, k), getattr(b, k), rtol) for k in ("nw", "ne", "se", "sw"))


def ours_api():
    from dplr_gb300 import _native
    return _native.api()


@pytest.mark.parametrize("name", list(TREES))
@pytest.mark.parametrize("alpha", [2.5, -0.75, 0.0])
def test_scal(name, alpha):
    t = TREES[name](1)
    res = []
    for api in (ours_api(), ref):
        a = tree.to_c(t)
        api.scal(t.size, alpha, a)
        res.append(tree.from_c(a))
        tree.free_c(a)
    assert same(res[0], res[1])


@pytest.mark.parametrize("name", ["uniform", "uneven", "dense"])
@pytest.mark.parametrize("target", ["empty", "other_shape", "same_shape"])
def test_cpy(name, target):
    t = TREES[name](2)
    res = []
    for api in (ours_api(), ref):
        a = tree.to_c(t)
        if target == "empty":
            b = tree.new_empty()
        elif target == "other_shape":
            b = tree.to_c(gen.random_tree(128, 32, 3, seed=9))
        else:
            b = tree.to_c(TREES[name](3))
        api.cpy(t.size, a, b)
        res.append(tree.from_c(b))
        tree.free_c(a)
        tree.free_c(b)
    assert same(res[0], res[1])
    assert np.array_equal(tree.to_dense(res[0]), tree.to_dense(t))


@pytest.mark.parametrize("name", ["uniform", "uneven", "dense"])
@pytest.mark.parametrize("alpha", [1.5, -2.0, 0.0])
def test_axpy(name, alpha):
    x, y = TREES[name](4), TREES[name](5)
    res = []
    for api in (ours_api(), ref):
        a, b = tree.to_c(x), tree.to_c(y)
        api.axpy(x.size, alpha, a, b)
        res.append(tree.from_c(b))
        tree.free_c(a)
        tree.free_c(b)
    assert same(res[0], res[1], rtol=1e-15)
    want = tree.to_dense(y) + alpha * tree.to_dense(x)
    got = tree.to_dense(res[0])
    assert np.linalg.norm(got - want) <= 1e-13 * max(np.linalg.norm(want), 1.0)


@pytest.mark.parametrize("name", list(TREES))
def test_adpy(name):
    t = TREES[name](6)
    d = np.random.default_rng(7).standard_normal(t.size)
    res = []
    for api in (ours_api(), ref):
        b = tree.to_c(t)
        api.adpy(t.size, -1.25, d.copy(), b)
        res.append(tree.from_c(b))
        tree.free_c(b)
    assert same(res[0], res[1])


def test_invalid_calls_match(capfd):
    """Size and type mismatches print DPLR's messages and change nothing."""
    x, y = TREES["uniform"](1), TREES["uniform"](2)
    msgs, res = [], []
    for api in (ours_api(), ref):
        a, b = tree.to_c(x), tree.to_c(y)
        api.axpy(x.size * 2, 1.0, a, b)               # wrong size
        api.scal(-1, 2.0, a)                          # negative size
        api.adpy(x.size + 1, 1.0, np.zeros(x.size + 1), b)
        res.append((tree.from_c(a), tree.from_c(b)))
        tree.free_c(a)
        tree.free_c(b)
        msgs.append(capfd.readouterr().err.splitlines())
    assert msgs[0] == msgs[1] and len(msgs[0]) == 3
    assert same(res[0][0], res[1][0]) and same(res[0][1], res[1][1])
    assert same(res[0][0], x) and same(res[0][1], y)
