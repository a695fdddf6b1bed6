"""CPU restatement of the SVD-based recompression (test infrastructure only).

Every low-rank block U diag(s) V^T of a PLR tree is replaced by its SVD
truncated where sigma < the block's threshold, the threshold being eps/4
per level from the root as dplrreduce splits it (src/dplrreduce.c:46).
The SVD is taken the way the GPU takes it: QR of U diag(s) and of V, then
the SVD of Ru Rv^T.  Nodes are the dataclasses of dplr_gb300.tree; ranks
shrink, capacities stay.
"""
from __future__ import annotations

import numpy as np

from dplr_gb300.tree import HNode, LowRank


def truncated(L: LowRank, eps: float) -> LowRank:
    r = L.rank
    if r == 0 or L.size == 0:
        return L
    qu, ru = np.linalg.qr(L.u * L.sig)
    qv, rv = np.linalg.qr(L.v)
    um, s, vmt = np.linalg.svd(ru @ rv.T)
    k = int(np.argmax(s < eps)) if np.any(s < eps) else len(s)
    return LowRank((qu @ um[:, :k]).copy(), s[:k].copy(), (qv @ vmt[:k].T).copy(), capacity=L.capacity)


def reduce_svd(node, eps: float):
    """A new tree with every low-rank block truncated."""
    if not isinstance(node, HNode):
        return node
    e2 = eps / 4.0
    return HNode(reduce_svd(node.nw, e2), truncated(node.ne, e2), reduce_svd(node.se, e2),
                 truncated(node.sw, e2))
