"""dortlr (src/dortlr.f90:12-207) pinned to its mathematical contract.

The Fortran cannot be compiled here (no Fortran compiler) and its only C
caller is broken as shipped, so no reference output exists.  The C
restatement (oracle/dplr_oracle.c, orc_dortlr) and the GPU kernel
(dplrreduce on the device) are therefore held to what the routine does
mathematically, with sval in RMS units (a column's norm is |x| / sqrt(n)):

* a hand-worked 2 x 2 case of rank 3, followed step by step through the
  u-pass (:43-106) and the v-pass (:110-170): one column collapses onto
  another, the product is kept exactly;
* input that is already an SVD (RMS-orthonormal u and v): the rank is the
  number of sval > eps, the kept values and the truncated product are
  exact;
* general input, one iteration (as dplrreduce runs it): the surviving v
  columns are RMS-orthonormal, the surviving u columns have RMS norm 1, and
  the product changes by at most eps sqrt(nnu nnv) per dropped column;
* redundant columns (nominal rank 2k spanning k directions) collapse to
  rank k without changing the product.
"""
import numpy as np
import pytest

from dplr_gb300 import tree
from oracle import pyoracle

S13, S178 = np.sqrt(13.0), np.sqrt(178.0)
# The hand-worked case: u = [(1,1), (1,1), (1,-1)], v = [(1,1), (1,-1), (1,1)],
# sval = (3, 2, 1), eps = 0.5.  u-pass: u_1 - u_0 = 0 folds 2/3 v_1 into v_0
# (then v_0 = (5,1)/sqrt(13), s_0 = sqrt(13)) and leaves s_1 = 0; u_2 is
# already orthogonal.  v-pass: v_2 loses 3/sqrt(13) v_0 (v_2 = (-1,5)/sqrt(13),
# s_2 = 2/sqrt(13)), 3/13 u_2 folds into u_0 (u_0 = (16,10)/sqrt(178),
# s_0 = sqrt(178/13)).  Column 2 moves into the hole at slot 1.
HAND_IN = (np.array([[1.0, 1.0, 1.0], [1.0, 1.0, -1.0]]),
           np.array([[1.0, 1.0, 1.0], [1.0, -1.0, 1.0]]),
           np.array([3.0, 2.0, 1.0]), 0.5)
HAND_OUT = (2,
            np.array([[16.0 / S178, 1.0], [10.0 / S178, -1.0]]),
            np.array([[5.0 / S13, -1.0 / S13], [1.0 / S13, 5.0 / S13]]),
            np.array([np.sqrt(178.0 / 13.0), 2.0 / S13]))


def _run_oracle(u, v, s, eps, niter=1):
    u, v, s = np.asfortranarray(u.copy()), np.asfortranarray(v.copy()), s.copy()
    r = pyoracle.dortlr(pyoracle.oracle("best"), u, v, s, eps, niter)
    return r, u[:, :r], v[:, :r], s[:r]


def _product(u, v, s):
    return (u * s) @ v.T


def test_hand_worked_case():
    r, u, v, s = _run_oracle(*HAND_IN)
    want_r, want_u, want_v, want_s = HAND_OUT
    assert r == want_r
    np.testing.assert_allclose(u, want_u, atol=1e-15)
    np.testing.assert_allclose(v, want_v, atol=1e-15)
    np.testing.assert_allclose(s, want_s, rtol=1e-15)
    np.testing.assert_allclose(_product(u, v, s), [[6.0, 2.0], [4.0, 0.0]], atol=1e-14)


def _rms_orthonormal(rng, n, k):
    return np.linalg.qr(rng.standard_normal((n, k)))[0] * np.sqrt(n)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_svd_input_keeps_exactly_the_values_above_eps(seed):
    rng = np.random.default_rng(seed)
    n, k, eps = 64, 12, 1e-3
    u, v = _rms_orthonormal(rng, n, k), _rms_orthonormal(rng, n, k)
    s = np.abs(rng.standard_normal(k)) * 10.0 ** rng.uniform(-6, 0, k)
    r, u2, v2, s2 = _run_oracle(u, v, s, eps)
    keep = s > eps
    assert r == int(keep.sum())
    np.testing.assert_allclose(np.sort(s2)[::-1], np.sort(s[keep])[::-1], rtol=1e-14)
    want = _product(u[:, keep], v[:, keep], s[keep])
    assert np.linalg.norm(_product(u2, v2, s2) - want) <= 1e-13 * np.linalg.norm(want)


@pytest.mark.parametrize("seed", [3, 4, 5])
def test_general_input_contract(seed):
    rng = np.random.default_rng(seed)
    nu, nv, k = 96, 80, 16
    u = rng.standard_normal((nu, k))
    v = rng.standard_normal((nv, k))
    s = 10.0 ** rng.uniform(-7, 0, k)
    eps = 1e-4
    a = _product(u, v, s)
    r, u2, v2, s2 = _run_oracle(u, v, s, eps)
    assert 0 < r <= k
    assert np.all(s2 > eps)
    # surviving v columns RMS-orthonormal, u columns RMS-normalised
    np.testing.assert_allclose(v2.T @ v2 / nv, np.eye(r), atol=1e-14)
    np.testing.assert_allclose(np.linalg.norm(u2, axis=0) / np.sqrt(nu), 1.0, atol=1e-14)
    # the product moves by at most eps (RMS units) per dropped column
    err = np.linalg.norm(_product(u2, v2, s2) - a)
    assert err <= (k - r) * eps * np.sqrt(nu * nv) + 1e-13 * np.linalg.norm(a)


def test_redundant_columns_collapse_without_loss():
    rng = np.random.default_rng(6)
    n, k = 64, 5
    bu, bv = rng.standard_normal((n, k)), rng.standard_normal((n, k))
    mix = rng.standard_normal((k, 2 * k))
    u, v = bu @ mix, np.hstack([bv, bv])
    s = np.ones(2 * k)
    a = _product(u, v, s)
    r, u2, v2, s2 = _run_oracle(u, v, s, 1e-8)
    assert r == k
    assert np.linalg.norm(_product(u2, v2, s2) - a) <= 1e-12 * np.linalg.norm(a)


# ------------------------------------------------------------------ GPU -----

def _one_level_tree(u, v, s):
    """H node of size 2n whose ne and sw blocks are u diag(s) v^T."""
    n = u.shape[0]
    leaf = tree.Dense(np.eye(n))
    return tree.HNode(leaf, tree.LowRank(u.copy(), s.copy(), v.copy()),
                      tree.Dense(np.eye(n)), tree.LowRank(u.copy(), s.copy(), v.copy()))


def _gpu_reduce(u, v, s, eps):
    """dortlr through the GPU dplrreduce of a one-level tree (dplrreduce
    runs dortlr on the top blocks with eps/4, src/dplrreduce.c:46)."""
    from dplr_gb300 import _native
    t = _one_level_tree(u, v, s)
    a = tree.to_c(t)
    _native.api().reduce(t.size, a, 4.0 * eps)
    out = tree.from_c(a)
    tree.free_c(a)
    return [(b.rank, b.u[:, :b.rank], b.v[:, :b.rank], b.sig[:b.rank]) for b in (out.ne, out.sw)]


@pytest.mark.gpu
def test_gpu_hand_worked_case():
    u, v, s, eps = HAND_IN
    want_r, want_u, want_v, want_s = HAND_OUT
    for r, u2, v2, s2 in _gpu_reduce(u, v, s, eps):
        assert r == want_r
        np.testing.assert_allclose(u2, want_u, atol=1e-15)
        np.testing.assert_allclose(v2, want_v, atol=1e-15)
        np.testing.assert_allclose(s2, want_s, rtol=1e-15)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [3, 4])
def test_gpu_general_input_contract(seed):
    rng = np.random.default_rng(seed)
    n, k, eps = 128, 16, 1e-4
    u, v = rng.standard_normal((n, k)), rng.standard_normal((n, k))
    s = 10.0 ** rng.uniform(-7, 0, k)
    a = _product(u, v, s)
    want = _run_oracle(u, v, s, eps)
    for r, u2, v2, s2 in _gpu_reduce(u, v, s, eps):
        assert r == want[0]
        np.testing.assert_allclose(v2.T @ v2 / n, np.eye(r), atol=1e-14)
        np.testing.assert_allclose(np.linalg.norm(u2, axis=0) / np.sqrt(n), 1.0, atol=1e-14)
        assert np.linalg.norm(_product(u2, v2, s2) - a) <= (k - r) * eps * n + 1e-13 * np.linalg.norm(a)
        np.testing.assert_allclose(s2, want[3], rtol=1e-12)


@pytest.mark.gpu
def test_gpu_svd_input_keeps_exactly_the_values_above_eps():
    rng = np.random.default_rng(7)
    n, k, eps = 64, 12, 1e-3
    u, v = _rms_orthonormal(rng, n, k), _rms_orthonormal(rng, n, k)
    s = np.abs(rng.standard_normal(k)) * 10.0 ** rng.uniform(-6, 0, k)
    keep = s > eps
    for r, u2, v2, s2 in _gpu_reduce(u, v, s, eps):
        assert r == int(keep.sum())
        np.testing.assert_allclose(np.sort(s2)[::-1], np.sort(s[keep])[::-1], rtol=1e-14)
