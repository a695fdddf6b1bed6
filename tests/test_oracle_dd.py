"""The double-double residual checker of the oracle (oracle/dd_resid.c).

It is the independent accuracy check of the GPU's refined solves at full
size, so it is pinned here on the CPU: against numpy's extended precision
(longdouble) on the same PLR operator, and against the oracle's FP64
dplrgepdmm, whose rounding it must bound.
"""
import numpy as np
import pytest

from dplr_gb300 import gen, tree
from oracle import pyoracle


def apply_ld(node, x):
    """A x from the PLR factors in numpy longdouble (x: m x k)."""
    ld = np.longdouble
    if isinstance(node, tree.Dense):
        return node.d.astype(ld) @ x
    h = node.nw.size

    def lr(b, xs):
        return (b.u.astype(ld) * b.sig.astype(ld)) @ (b.v.astype(ld).T @ xs)
    return np.vstack([apply_ld(node.nw, x[:h]) + lr(node.ne, x[h:]),
                      apply_ld(node.se, x[h:]) + lr(node.sw, x[:h])])


def apply_abs(node, x):
    """|A| x with every factor taken entrywise in absolute value."""
    if isinstance(node, tree.Dense):
        return np.abs(node.d) @ x
    h = node.nw.size

    def lr(b, xs):
        return (np.abs(b.u) * np.abs(b.sig)) @ (np.abs(b.v).T @ xs)
    return np.vstack([apply_abs(node.nw, x[:h]) + lr(node.ne, x[h:]),
                      apply_abs(node.se, x[h:]) + lr(node.sw, x[:h])])


@pytest.mark.parametrize("seed", [0, 1])
def test_dd_residual_matches_extended_precision(seed):
    t = gen.random_tree(512, 32, [12, 8, 5, 3], seed=seed)
    m = t.size
    rng = np.random.default_rng(seed + 10)
    x = rng.standard_normal((5, m))
    ax = apply_ld(t, x.T.astype(np.longdouble)).T
    # b = A x + a small, known perturbation: the residual cancels almost all of b
    b = np.asarray(ax + rng.standard_normal((5, m)) * 1e-9, dtype=np.float64)
    want = np.linalg.norm(np.asarray(b.astype(np.longdouble) - ax, dtype=np.float64), axis=1)
    orc = pyoracle.oracle("best")
    a = tree.to_c(t)
    rn, an = pyoracle.resid_dd(orc, a, x, b, threads=3)
    tree.free_c(a)
    absn = np.linalg.norm(apply_abs(t, np.abs(x).T).T, axis=1)
    np.testing.assert_allclose(an, absn, rtol=1e-13)
    # longdouble carries 64 bits (x86) or 113 (aarch64): both far beyond the
    # 1e-9 residual, so the two must agree to well within its rounding
    assert np.all(np.abs(rn - want) <= 1e-16 * an), (rn, want, an)
    assert np.all(rn > 1e-9)


def test_dd_residual_bounds_the_fp64_apply():
    """The FP64 dplrgepdmm residual differs from the exact one by its own
    rounding, which stays within n u |A||x| (n: the longest dot product)."""
    t = gen.random_tree(1024, 64, [24, 16, 8, 4], seed=2)
    m = t.size
    rng = np.random.default_rng(3)
    x = rng.standard_normal((4, m))
    b = rng.standard_normal((4, m))
    orc = pyoracle.oracle("best")
    a = tree.to_c(t)
    y = b.copy().reshape(-1)
    orc.gepdmm("N", "N", m, 4, -1.0, a, np.ascontiguousarray(x).reshape(-1), m, 1.0, y, m)
    rn, an = pyoracle.resid_dd(orc, a, x, b, threads=2)
    tree.free_c(a)
    r64 = np.linalg.norm(y.reshape(4, m), axis=1)
    assert np.all(np.abs(r64 - rn) <= m * 1.1e-16 * an + 1e-300)


def test_dd_residual_rejects_bad_arguments():
    orc = pyoracle.oracle("best")
    t = gen.random_tree(256, 32, [4, 2], seed=0)
    a = tree.to_c(t)
    x = np.zeros((1, 256))
    rc = orc.lib.orc_resid_dd(128, a, 1, x.ctypes.data_as(tree.c_double_p), 256,
                              x.ctypes.data_as(tree.c_double_p), 256, x.ctypes.data_as(tree.c_double_p),
                              x.ctypes.data_as(tree.c_double_p), 1)
    tree.free_c(a)
    assert rc == -1


@pytest.mark.parametrize("seed", [0, 5])
def test_inverse_shape_stand_in_has_the_inverse_ranks(seed):
    """The timing stand-in for inv(A) (oracle/shape.c) has exactly the ranks
    and stored entries of the inverse the oracle's dplrgeinv builds."""
    orc = pyoracle.oracle("best")
    t = gen.random_tree(1024, 32, [9, 0, 4, 7, 2], seed=seed)
    a, binv, shape = tree.to_c(t), tree.new_empty(), tree.new_empty()
    assert orc.geinv(t.size, a, binv, 0.0) == 0
    assert orc.lib.orc_inverse_shape(t.size, a, shape, 0.5) == 0

    def ranks(node, out):
        if isinstance(node, tree.HNode):
            out.append((node.ne.rank, node.sw.rank))
            ranks(node.nw, out)
            ranks(node.se, out)
        return out

    got, want = tree.from_c(shape), tree.from_c(binv)
    assert ranks(got, []) == ranks(want, [])
    assert orc.nz(t.size, shape) == orc.nz(t.size, binv)
    for c in (a, binv, shape):
        tree.free_c(c)
