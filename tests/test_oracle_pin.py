"""Pin the oracle to the reference's own C sources (where they were built).

With the same BLAS library, the restatement must reproduce the reference
bit for bit on fresh seeded inputs: every BLAS call is the same call.
Skipped where oracle/_ref was not built (the reference tree is absent);
the golden vectors in tests/golden carry the pin there.
"""
import numpy as np
import pytest

from dplr_gb300 import gen, tree
from oracle import pyoracle

REF = pyoracle.reference()
pytestmark = pytest.mark.skipif(REF is None, reason="reference library not built here")


def _trees():
    yield gen.random_tree(128, 16, [4, 2, 0], seed=21, capacity_extra=1)
    yield gen.random_tree(256, 32, lambda lvl, rng: int(rng.integers(0, 9)), seed=22)
    x = gen.sorted_uniform(128, seed=23)
    yield gen.compress_dense(gen.exp_kernel_1d(x, 0.2, 1e-2), 1e-12, 2)


@pytest.mark.parametrize("idx", range(3))
def test_bitwise_apply(idx):
    t = list(_trees())[idx]
    orc = pyoracle.oracle("blas")
    m = t.size
    rng = np.random.default_rng(idx)
    for tr in "NT":
        x = rng.standard_normal(m * 2)
        y0 = rng.standard_normal(m)
        outs = []
        for api in (orc, REF):
            a = tree.to_c(t)
            y = y0.copy()
            api.gepmv(tr, m, 0.7, a, x, 2, -0.3, y, 1)
            outs.append(y)
            tree.free_c(a)
        assert np.array_equal(outs[0], outs[1])
    for ta in "NT":
        for tb in "NT":
            n = 3
            b = rng.standard_normal(m * n)
            c0 = rng.standard_normal(m * n)
            outs = []
            for api in (orc, REF):
                a = tree.to_c(t)
                c = c0.copy()
                api.gepdmm(ta, tb, m, n, 1.1, a, b, m if tb == "N" else n, 0.5, c, m)
                outs.append(c)
                tree.free_c(a)
            assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("idx", range(3))
def test_bitwise_inverse_and_prk(idx):
    t = list(_trees())[idx]
    orc = pyoracle.oracle("blas")
    m = t.size
    got = []
    for api in (orc, REF):
        a = tree.to_c(t)
        b = tree.new_empty()
        info = api.geinv(m, a, b, 1e-9)
        assert info == 0
        got.append(tree.flatten(tree.from_c(b)))
        tree.free_c(a)
        tree.free_c(b)
    assert np.array_equal(got[0][0], got[1][0])
    assert np.array_equal(got[0][1], got[1][1])
