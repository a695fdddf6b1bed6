"""GPU generation of large synthetic PLR matrices (matrix-free compression).

DPLR compresses a dense matrix with one full SVD per off-diagonal block
(src/dplrd2p.c:22-178); at N = 2^18 that needs the 550 GB dense matrix and
hours of SVDs.  This module builds the same kind of tree without forming
the matrix: kernel entries are evaluated on the fly in row chunks and each
off-diagonal block is compressed by a randomized range finder with one
power iteration (Halko, Martinsson & Tropp 2011, Alg. 4.4 + 5.1), batched
over all nodes of a level.

Kernel matrices are symmetric, so each H node compresses its ne block once
and stores sw = ne^T (U_sw = V_ne, V_sw = U_ne).

Precision: blocks of size <= ``fp64_below`` rows are sampled in FP64 and
their ranks chosen adaptively (sigma_i >= tol * sigma_1, clamped to
[rmin, rmax]); larger blocks are sampled in FP32 (their numerical rank at
the tolerance exceeds rmax, so they are truncated to rmax, and FP32
sampling gives factors accurate to ~1e-7 relative).  The tree produced is
the matrix every solver is measured against; its distance to the exact
kernel matrix is reported by ``kernel_error_estimate``.

This is input preparation, not part of the measured path; it uses torch
(cuBLAS GEMMs, cuSOLVER QR/SVD) for convenience.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch

from .tree import Dense, HNode, LowRank


@dataclass
class GenStats:
    ranks: list = field(default_factory=list)       # per level (min, max)
    tail_ratio: list = field(default_factory=list)  # per level max sigma_{r+1}/sigma_1 estimate
    seconds: float = 0.0


def kd_order(pts: np.ndarray, leaf: int) -> np.ndarray:
    """Permutation ordering points by kd-tree bisection: split the longer
    bounding-box extent at the median, recursively, down to `leaf` points."""
    idx = np.arange(len(pts))
    out = []

    def rec(ix: np.ndarray):
        if len(ix) <= leaf:
            out.append(ix)
            return
        p = pts[ix]
        ext = p.max(axis=0) - p.min(axis=0)
        d = int(np.argmax(ext))
        h = len(ix) // 2
        part = np.argpartition(p[:, d], h - 1)
        rec(ix[part[:h]])
        rec(ix[part[h:]])

    rec(idx)
    return np.concatenate(out)


def _kernel(xa: torch.Tensor, xb: torch.Tensor, inv2l2: float, kind: str) -> torch.Tensor:
    """K(xa, xb) for batched point sets (B, na, d) x (B, nb, d)."""
    diff = xa[:, :, None, :] - xb[:, None, :, :]
    if kind == "gauss":
        return torch.exp(-(diff * diff).sum(-1) * inv2l2)
    r = torch.sqrt((diff * diff).sum(-1))
    return torch.exp(-r * inv2l2)


def _kmul(xr, xc, M, inv2l2, kind, budget):
    """K(xr, xc) @ M for a batch of nodes, in row chunks of bounded size."""
    B, nr, _ = xr.shape
    nc = xc.shape[1]
    rows = max(1, min(nr, budget // max(1, B * nc * 3)))
    out = torch.empty(B, nr, M.shape[2], dtype=M.dtype, device=M.device)
    for r0 in range(0, nr, rows):
        r1 = min(nr, r0 + rows)
        out[:, r0:r1] = torch.bmm(_kernel(xr[:, r0:r1], xc, inv2l2, kind), M)
    return out


def _compress_level(x1, x2, p, inv2l2, kind, dtype, gen, budget):
    """Randomized SVD of K(x1, x2) for a batch of nodes -> (U, S, V)."""
    B, n, _ = x1.shape
    om = torch.randn(B, n, p, device=x1.device, dtype=dtype, generator=gen)
    y = _kmul(x1, x2, om, inv2l2, kind, budget)
    q, _ = torch.linalg.qr(y)
    z = _kmul(x2, x1, q, inv2l2, kind, budget)          # K^T Q (K(x2,x1) = K(x1,x2)^T)
    qz, _ = torch.linalg.qr(z)
    y = _kmul(x1, x2, qz, inv2l2, kind, budget)          # one power iteration
    q, _ = torch.linalg.qr(y)
    bt = _kmul(x2, x1, q, inv2l2, kind, budget)          # (Q^T K)^T, n x p
    qb, rb = torch.linalg.qr(bt)
    ur, s, vrh = torch.linalg.svd(rb)                    # rb = ur diag(s) vrh
    # K ~ Q B = Q (qb rb)^T = Q rb^T qb^T = (Q vrh^T) diag(s) (qb ur)^T
    u = torch.bmm(q, vrh.transpose(1, 2))
    v = torch.bmm(qb, ur)
    return u, s, v


def kernel_tree_2d(n: int = 1 << 18, leaf: int = 256, ell: float = 0.05, shift: float = 1e-2,
                   tol: float = 1e-10, rmin: int = 8, rmax: int = 128, seed: int = 0,
                   fp64_below: int = 512, device: str = "cuda", kind: str = "gauss",
                   stats: GenStats | None = None):
    """HODLR tree of exp(-r^2/(2 l^2)) + shift*I on n uniform points in the
    unit square in kd-tree order (the mixed-precision benchmark matrix)."""
    import time
    t0 = time.time()
    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    pts = pts[kd_order(pts, leaf)]
    return _kernel_tree(pts, leaf, ell, shift, tol, rmin, rmax, seed, fp64_below, device, kind,
                        stats, t0)


def _kernel_tree(pts, leaf, ell, shift, tol, rmin, rmax, seed, fp64_below, device, kind, stats,
                 t0):
    import time
    n = len(pts)
    inv2l2 = 1.0 / (2 * ell * ell) if kind == "gauss" else 1.0 / ell
    X = torch.tensor(pts, dtype=torch.float64, device=device)
    levels = int(round(math.log2(n // leaf)))
    gen = torch.Generator(device=device)
    gen.manual_seed(seed + 1)
    budget = 1 << 28                               # kernel entries per chunk
    blocks = {}                                    # (level, node) -> LowRank ne
    st = stats if stats is not None else GenStats()
    for lvl in range(levels):
        nodes = 1 << lvl
        size = n // nodes
        h = size // 2
        dtype = torch.float64 if h <= fp64_below else torch.float32
        p = rmax + 16
        xs = X.view(nodes, size, -1).to(dtype)
        x1, x2 = xs[:, :h], xs[:, h:]
        if p >= h:
            # small blocks: exact SVD of the dense block
            k = _kernel(x1, x2, inv2l2, kind)
            u, s, vh = torch.linalg.svd(k)
            v = vh.transpose(1, 2)
        else:
            u, s, v = _compress_level(x1, x2, p, inv2l2, kind, dtype, gen, budget)
        s64 = s.double()
        rel = s64 / s64[:, :1]
        rk = (rel >= tol).sum(1).clamp(min=min(rmin, h), max=min(rmax, h))
        tail = rel[torch.arange(nodes, device=rel.device), rk.clamp(max=rel.shape[1] - 1)]
        st.ranks.append((int(rk.min()), int(rk.max())))
        st.tail_ratio.append(float(tail.max()))
        u64, v64 = u.double().cpu().numpy(), v.double().cpu().numpy()
        s_np, rk_np = s64.cpu().numpy(), rk.cpu().numpy()
        for q in range(nodes):
            r = int(rk_np[q])
            blocks[(lvl, q)] = LowRank(np.ascontiguousarray(u64[q, :, :r]), s_np[q, :r].copy(),
                                       np.ascontiguousarray(v64[q, :, :r]))
    nleaf = n // leaf
    xl = X.view(nleaf, leaf, -1)
    kl = _kernel(xl, xl, inv2l2, kind) + shift * torch.eye(leaf, dtype=torch.float64, device=device)
    kl = kl.cpu().numpy()

    def build(lvl, q):
        if lvl == levels:
            return Dense(np.asfortranarray(kl[q]))
        ne = blocks[(lvl, q)]
        sw = LowRank(ne.v, ne.sig, ne.u)
        return HNode(build(lvl + 1, 2 * q), ne, build(lvl + 1, 2 * q + 1), sw)

    tree_ = build(0, 0)
    st.seconds = time.time() - t0
    return tree_


def kernel_tree_1d(n: int, leaf: int, ell: float, shift: float, rank: int, seed: int = 0,
                   device: str = "cuda", tol: float = 0.0, stats: GenStats | None = None):
    """1D exponential kernel exp(-|x_i-x_j|/l) on sorted uniform points with a
    fixed off-diagonal rank (truncated SVD of every block)."""
    import time
    t0 = time.time()
    rng = np.random.default_rng(seed)
    pts = np.sort(rng.random(n))[:, None]
    return _kernel_tree(pts, leaf, ell, shift, tol, rank, rank, seed, 1 << 30, device, "exp",
                        stats, t0)
