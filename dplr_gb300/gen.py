"""Synthetic PLR inputs: seeded points, kernel matrices and trees.

* ``compress_dense`` restates DPLR's dense-to-PLR compression
  (src/dplrd2p.c:22-331): per off-diagonal block a full SVD, rank = index
  of the first singular value below the block's absolute threshold, U
  kept, V stored as V; the threshold is eps/2 when the diagonal children
  are leaves and eps/4 otherwise, passed down recursively.
* ``exp1d_tree`` builds the 1D exponential-kernel trees without forming
  the dense matrix: for sorted points each off-diagonal block of
  exp(-|x_i-x_j|/l) is exactly rank one; a requested fixed rank r > 1 is
  met with r-1 orthonormal tail columns at round-off level singular
  values (the shape a truncated SVD of a rank-one block has).
* ``random_tree`` builds seeded trees of any shape and rank profile
  (uneven ranks, rank-0 blocks) for parity tests.
"""
from __future__ import annotations

import numpy as np

from .tree import Dense, HNode, LowRank, Node


# --------------------------------------------------------------------------
# dense compression (restates src/dplrd2p.c)
# --------------------------------------------------------------------------

def _lowrank_svd(block: np.ndarray, eps: float) -> LowRank:
    u, s, vt = np.linalg.svd(block, full_matrices=False)
    rank = int(np.argmax(s < eps)) if np.any(s < eps) else len(s)
    return LowRank(u[:, :rank].copy(), s[:rank].copy(), vt[:rank].T.copy())


def compress_dense(a: np.ndarray, eps: float, nlvl: int) -> Node:
    """Dense m x m -> PLR with nlvl levels and absolute accuracy eps."""
    m = a.shape[0]
    if m % (1 << nlvl):
        raise ValueError("m not divisible by 2**nlvl")
    if nlvl == 0:
        return Dense(np.array(a, dtype=np.float64, order="F"))
    eps2 = eps / 2.0 if nlvl == 1 else eps / 4.0
    h = m // 2
    ne = _lowrank_svd(a[:h, h:], eps2)
    sw = _lowrank_svd(a[h:, :h], eps2)
    return HNode(compress_dense(a[:h, :h], eps2, nlvl - 1), ne,
                 compress_dense(a[h:, h:], eps2, nlvl - 1), sw)


def exp_kernel_1d(x: np.ndarray, ell: float, shift: float) -> np.ndarray:
    d = np.abs(x[:, None] - x[None, :])
    return np.exp(-d / ell) + shift * np.eye(len(x))


def sorted_uniform(n: int, seed: int) -> np.ndarray:
    return np.sort(np.random.default_rng(seed).random(n))


# --------------------------------------------------------------------------
# matrix-free 1D exponential trees
# --------------------------------------------------------------------------

def _tail(rng, n: int, k: int, against: np.ndarray) -> np.ndarray:
    """k orthonormal columns orthogonal to `against` (n x 1)."""
    if k <= 0:
        return np.zeros((n, 0))
    g = rng.standard_normal((n, k))
    g -= against @ (against.T @ g)
    q, _ = np.linalg.qr(g)
    return q


def exp1d_tree(x: np.ndarray, ell: float, shift: float, leaf: int, rank: int,
               seed: int = 0, tail_scale: float = 1e-15) -> Node:
    """PLR of exp(-|x_i-x_j|/ell) + shift*I over sorted points x."""
    rng = np.random.default_rng(seed)

    def block(xr: np.ndarray, xc: np.ndarray, top: bool) -> LowRank:
        # rows xr, columns xc; for the ne block rows precede columns.
        c = xr[-1] if top else xc[-1]
        if top:      # x_i <= c <= x_j : exp(-(x_j-x_i)/l) = exp(-(c-x_i)/l) exp(-(x_j-c)/l)
            fu, fv = np.exp(-(c - xr) / ell), np.exp(-(xc - c) / ell)
        else:        # x_j <= c <= x_i
            fu, fv = np.exp(-(xr - c) / ell), np.exp(-(c - xc) / ell)
        nu, nv = np.linalg.norm(fu), np.linalg.norm(fv)
        s1 = nu * nv
        u1, v1 = (fu / nu)[:, None], (fv / nv)[:, None]
        k = max(rank, 1) - 1
        u = np.hstack([u1, _tail(rng, len(xr), k, u1)])
        v = np.hstack([v1, _tail(rng, len(xc), k, v1)])
        sig = np.concatenate([[s1], s1 * tail_scale * np.geomspace(1.0, 1e-2, k)]) if k else np.array([s1])
        return LowRank(u, sig, v)

    def build(xs: np.ndarray) -> Node:
        m = len(xs)
        if m <= leaf:
            return Dense(exp_kernel_1d(xs, ell, shift))
        h = m // 2
        return HNode(build(xs[:h]), block(xs[:h], xs[h:], True),
                     build(xs[h:]), block(xs[h:], xs[:h], False))

    return build(x)


# --------------------------------------------------------------------------
# random trees for parity tests
# --------------------------------------------------------------------------

def random_tree(n: int, leaf: int, ranks, seed: int = 0, diag_shift: float | None = None,
                capacity_extra: int = 0, decay: float = 0.5) -> Node:
    """Seeded PLR tree with leaves of size `leaf` and per-level ranks.

    `ranks` is an int (same everywhere), a per-level list, or a callable
    (level, rng) -> rank.  Leaves get `diag_shift` (default: n) on the
    diagonal so that the matrix is comfortably invertible.  Singular values
    decay geometrically so the blocks look like compressed kernels.
    """
    rng = np.random.default_rng(seed)
    shift = float(n) if diag_shift is None else diag_shift

    def rank_at(level):
        if callable(ranks):
            return int(ranks(level, rng))
        if isinstance(ranks, (list, tuple)):
            return int(ranks[min(level, len(ranks) - 1)])
        return int(ranks)

    def lowrank(m: int, r: int) -> LowRank:
        r = min(r, m)
        u, _ = np.linalg.qr(rng.standard_normal((m, max(r, 1))))
        v, _ = np.linalg.qr(rng.standard_normal((m, max(r, 1))))
        sig = np.sqrt(m) * decay ** np.arange(r) * (0.5 + rng.random(r))
        cap = r + int(capacity_extra)
        return LowRank(u[:, :r].copy(), sig, v[:, :r].copy(), capacity=cap)

    def build(m: int, level: int) -> Node:
        if m <= leaf:
            d = rng.standard_normal((m, m)) + shift * np.eye(m)
            return Dense(d)
        h = m // 2
        return HNode(build(h, level + 1), lowrank(h, rank_at(level)),
                     build(m - h, level + 1), lowrank(h, rank_at(level)))

    return build(n, 0)
