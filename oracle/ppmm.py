"""CPU restatement of DPLR's PLR x PLR product (test infrastructure only).

C := alpha * op(A) * op(B) + beta * C for PLR matrices A, B, C of one
structure, following src/dplrppmm.c:
  * dplrgeppmm (:998) picks one of four recursions by (transa, transb);
  * each recursion (dplrppmm :492, dplrptpmm :617, dplrpptmm :742,
    dplrptptmm :868) multiplies dense leaves (dgemm), and at an H node
    - appends to C.ne: op(A).nw x op(B).ne (dplrplmm :185, beta first)
      then op(A).ne x op(B).se (dplrlpmm :334),
    - appends to C.sw: op(A).sw x op(B).nw (dplrlpmm, beta first) then
      op(A).se x op(B).sw (dplrplmm),
    - recurses into C.nw and C.se (threshold eps/4), then adds the product
      of the two off-diagonal low-rank blocks (dplrgellmm :26) to each
      diagonal child with dplrgeprk (src/dplrprk.c:21);
  where op(M).ne = M.ne or M.sw^T and op(M).sw = M.sw or M.ne^T.
New columns are normalised with the block's threshold: a column whose
scaled norm falls below it keeps its raw values and gets sig = 0.
Capacities grow by dplrresizelr's rule (at least doubling).  Nodes are
the dataclasses of dplr_gb300.tree (LowRank.capacity tracked); arrays
hold the live columns only.  Products with subtrees go through the tree
(DPLR's dplrgepdmm recursion) with numpy BLAS calls, so the cost follows
the reference's and the restatement also serves as the timed CPU port.
"""
from __future__ import annotations

import numpy as np

from dplr_gb300.tree import Dense, HNode, LowRank


# ------------------------------------------------------------ helpers --

def _cap(L: LowRank) -> int:
    return L.rank if L.capacity is None else L.capacity


def _grow(L: LowRank, need: int) -> None:
    """Capacity after dplrresizelr(L, need) when capacity < need
    (src/dplrresizelr.c:15: at least doubling)."""
    c = _cap(L)
    if c < need:
        L.capacity = max(need, 2 * c)


def _append(L: LowRank, u: np.ndarray, s: np.ndarray, v: np.ndarray) -> None:
    L.u = np.concatenate([L.u, u], axis=1)
    L.v = np.concatenate([L.v, v], axis=1)
    L.sig = np.concatenate([L.sig, s])


def _scale_beta(L: LowRank, beta: float) -> None:
    """The beta step of dplrplmm / dplrlpmm: drop the columns when beta == 0
    (or none are live), else sig *= |beta| and u negated for beta < 0."""
    if beta == 0.0 or L.rank == 0:
        L.u, L.v, L.sig = L.u[:, :0], L.v[:, :0], L.sig[:0]
        return
    L.sig = L.sig * abs(beta)
    if beta < 0.0:
        L.u = -L.u


def _normalise(cols: np.ndarray, s: np.ndarray, eps: float):
    """Column norms f; sig = f*s, column scaled by 1/f, unless f*s < eps
    (then sig = 0 and the raw column is kept)."""
    out = cols.copy()
    sig = np.zeros(cols.shape[1])
    for j in range(cols.shape[1]):
        f = float(np.linalg.norm(cols[:, j]))
        if f * s[j] < eps:
            sig[j] = 0.0
        else:
            sig[j] = f * s[j]
            out[:, j] = cols[:, j] * (1.0 / f)
    return out, sig


def _dense(node) -> np.ndarray:
    from dplr_gb300.tree import to_dense
    return to_dense(node)


class _LR:
    """A low-rank block read as op(block): factors (u, s, v) of L or L^T."""

    def __init__(self, L: LowRank, trans: bool):
        self.u, self.v = (L.v, L.u) if trans else (L.u, L.v)
        self.s = L.sig
        self.rank = L.rank


class _Op:
    """op(M) for an H node or leaf M: its blocks as op(M) sees them."""

    def __init__(self, M, trans: bool):
        self.M, self.t = M, trans

    def nw(self):
        return _Op(self.M.nw, self.t)

    def se(self):
        return _Op(self.M.se, self.t)

    def ne(self) -> _LR:
        return _LR(self.M.sw, True) if self.t else _LR(self.M.ne, False)

    def sw(self) -> _LR:
        return _LR(self.M.ne, True) if self.t else _LR(self.M.sw, False)

    def dense(self) -> np.ndarray:
        d = _dense(self.M)
        return d.T if self.t else d

    def apply(self, x: np.ndarray) -> np.ndarray:
        """op(M) x by the tree (DPLR's dplrgepdmm recursion, no dense
        expansion)."""
        if isinstance(self.M, Dense):
            return (self.M.d.T if self.t else self.M.d) @ x
        h = self.M.nw.size
        top, bot = x[:h], x[h:]
        ne, sw = self.ne(), self.sw()
        y = np.empty((self.M.size,) + x.shape[1:])
        y[:h] = self.nw().apply(top)
        y[h:] = self.se().apply(bot)
        if ne.rank:
            y[:h] += (ne.u * ne.s) @ (ne.v.T @ bot)
        if sw.rank:
            y[h:] += (sw.u * sw.s) @ (sw.v.T @ top)
        return y

    def transposed(self) -> "_Op":
        return _Op(self.M, not self.t)


# ------------------------------------------------- block-level products --

def plmm(alpha: float, P: _Op, Lb: _LR, beta: float, C: LowRank, eps: float) -> None:
    """C := alpha op(P) Lb + beta C, Lb low rank (src/dplrppmm.c:185)."""
    _scale_beta(C, beta)
    if alpha == 0.0 or Lb.rank == 0:
        return
    _grow(C, C.rank + Lb.rank)
    y = alpha * P.apply(Lb.u)
    u, s = _normalise(y, Lb.s, eps)
    _append(C, u, s, Lb.v.copy())


def lpmm(alpha: float, La: _LR, P: _Op, beta: float, C: LowRank, eps: float) -> None:
    """C := alpha La op(P) + beta C, La low rank (src/dplrppmm.c:334)."""
    _scale_beta(C, beta)
    if alpha == 0.0 or La.rank == 0:
        return
    _grow(C, C.rank + La.rank)
    z = alpha * P.transposed().apply(La.v)
    v, s = _normalise(z, La.s, eps)
    _append(C, La.u.copy(), s, v)


def gellmm(alpha: float, L1: _LR, L2: _LR, eps: float):
    """(u3, s3, v3) with u3 diag(s3) v3^T = alpha L1 L2 (src/dplrppmm.c:26,
    beta = 0): rank min(r1, r2), the shorter side copied."""
    r1, r2 = L1.rank, L2.rank
    n = L1.u.shape[0]
    if r1 == 0 or r2 == 0 or alpha == 0.0:
        return np.zeros((n, 0)), np.zeros(0), np.zeros((n, 0))
    if r1 < r2:
        temp = (L2.u.T @ L1.v) * L2.s[:, None]        # r2 x r1
        v3, s3 = _normalise(alpha * (L2.v @ temp), L1.s, eps)
        return L1.u.copy(), s3, v3
    temp = (L1.v.T @ L2.u) * L1.s[:, None]            # r1 x r2
    u3, s3 = _normalise(alpha * (L1.u @ temp), L2.s, eps)
    return u3, s3, L2.v.copy()


def geprk(alpha: float, u: np.ndarray, s: np.ndarray, v: np.ndarray, A, eps: float) -> None:
    """A += alpha u diag(s) v^T on a PLR node (src/dplrprk.c:21)."""
    k = u.shape[1]
    if alpha == 0.0 or k == 0:
        return
    if isinstance(A, Dense):
        A.d = A.d + alpha * ((u * s) @ v.T)
        return
    eps2 = eps / 2.0 if isinstance(A.nw, Dense) else eps / 4.0
    h = A.nw.size
    for L, uu, vv in ((A.ne, u[:h], v[h:]), (A.sw, u[h:], v[:h])):
        _grow(L, L.rank + k)
        nu, nv, ns = uu.copy(), vv.copy(), np.zeros(k)
        for i in range(k):
            f1 = float(np.linalg.norm(uu[:, i]))
            f2 = float(np.linalg.norm(vv[:, i]))
            if abs(alpha) * s[i] * f1 * f2 < eps2:
                ns[i] = 0.0
            else:
                ns[i] = abs(alpha) * s[i] * f1 * f2
                g1 = 1.0 / f1 if alpha > 0.0 else -1.0 / f1
                nu[:, i] = uu[:, i] * g1
                nv[:, i] = vv[:, i] * (1.0 / f2)
        _append(L, nu, ns, nv)
    geprk(alpha, u[:h], s, v[:h], A.nw, eps2)
    geprk(alpha, u[h:], s, v[h:], A.se, eps2)


# ------------------------------------------------------------ recursion --

def _ppmm(alpha: float, A: _Op, B: _Op, beta: float, C, eps: float) -> None:
    if isinstance(C, Dense):
        # dgemm: alpha == 0 reads neither A nor B, beta == 0 does not read C
        prod = alpha * (A.dense() @ B.dense()) if alpha != 0.0 else np.zeros_like(C.d)
        C.d = prod + (beta * C.d if beta != 0.0 else 0.0)
        return
    eps2 = eps / 4.0
    plmm(alpha, A.nw(), B.ne(), beta, C.ne, eps2)
    lpmm(alpha, A.ne(), B.se(), 1.0, C.ne, eps2)
    lpmm(alpha, A.sw(), B.nw(), beta, C.sw, eps2)
    plmm(alpha, A.se(), B.sw(), 1.0, C.sw, eps2)
    _ppmm(alpha, A.nw(), B.nw(), beta, C.nw, eps2)
    u, s, v = gellmm(alpha, A.ne(), B.sw(), eps2)
    geprk(1.0, u, s, v, C.nw, eps2)
    _ppmm(alpha, A.se(), B.se(), beta, C.se, eps2)
    u, s, v = gellmm(alpha, A.sw(), B.ne(), eps2)
    geprk(1.0, u, s, v, C.se, eps2)


def _same_structure(a, b) -> bool:
    if type(a) is not type(b) or a.size != b.size:
        return False
    if isinstance(a, HNode):
        return _same_structure(a.nw, b.nw) and _same_structure(a.se, b.se)
    return True


def geppmm(transa: str, transb: str, alpha: float, A, B, beta: float, C, eps: float) -> None:
    """In place on C (Python tree): C := alpha op(A) op(B) + beta C."""
    if not (_same_structure(A, B) and _same_structure(B, C)):
        raise ValueError("A, B and C structures differ")
    ta = transa in ("T", "t")
    tb = transb in ("T", "t")
    _ppmm(alpha, _Op(A, ta), _Op(B, tb), beta, C, eps)
