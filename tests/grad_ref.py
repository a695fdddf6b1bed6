"""FP64 CPU reference gradients for the PLR adjoint (numpy, dense).

For a loss with dense derivative dL/dA = dA, the derivative with respect
to the factors of a low-rank block A[R, C] = U diag(s) V^T is
    dU = dA[R, C] V diag(s),  dV = dA[R, C]^T U diag(s),
    ds_k = U[:, k]^T dA[R, C] V[:, k],
and for a dense leaf A[R, R] = D it is dA[R, R].  For the solve loss
L = sum_j ||A^-1 b_j - t_j||^2: x = A^-1 b, lam = A^-T 2 (x - t),
dL/db = lam and dA = -sum_j lam_j x_j^T.
"""
import numpy as np

from dplr_gb300 import tree


def solve_loss(A, b, t):
    x = np.linalg.solve(A, b.T).T
    return float(np.sum((x - t) ** 2))


def solve_loss_grads(A, b, t):
    """(loss, dL/db, dense dL/dA) for rows of b, t as right-hand sides."""
    x = np.linalg.solve(A, b.T).T
    lam = np.linalg.solve(A.T, (2.0 * (x - t)).T).T
    return float(np.sum((x - t) ** 2)), lam, -(lam.T @ x)


def project_lowrank(u, s, v, dA_blk):
    return dA_blk @ v * s, dA_blk.T @ u * s, np.einsum("ik,il,lk->k", u, dA_blk, v)


def tree_grads(node, dA, row0=0, out=None, path=""):
    """Per-node factor gradients {path: (dU, ds, dV) or dD} for a dense dA."""
    out = {} if out is None else out
    if isinstance(node, tree.Dense):
        b = node.size
        out[path.rstrip(".") or "root"] = dA[row0:row0 + b, row0:row0 + b].copy()
        return out
    h = node.nw.size
    m = node.size
    du, dv, ds = project_lowrank(node.ne.u, node.ne.sig, node.ne.v, dA[row0:row0 + h, row0 + h:row0 + m])
    out[path + "ne"] = (du, ds, dv)
    du, dv, ds = project_lowrank(node.sw.u, node.sw.sig, node.sw.v,
                                 dA[row0 + h:row0 + m, row0:row0 + h])
    out[path + "sw"] = (du, ds, dv)
    tree_grads(node.nw, dA, row0, out, path + "nw.")
    tree_grads(node.se, dA, row0 + h, out, path + "se.")
    return out


def pool_grads(blocks, pool, dA):
    """Reference gradient in the GPU pool layout: `blocks` from
    GpuPlan.pool_blocks(), `pool` the factor values (numpy)."""
    g = np.zeros_like(pool)
    for blk in blocks:
        if blk["kind"] == "lowrank":
            n, r = blk["n"], blk["rank"]
            if r == 0:
                continue
            u = pool[blk["u"]:blk["u"] + n * r].reshape(r, n).T
            v = pool[blk["v"]:blk["v"] + n * r].reshape(r, n).T
            s = pool[blk["sig"]:blk["sig"] + r]
            R, C = blk["row0"], blk["col0"]
            du, dv, ds = project_lowrank(u, s, v, dA[R:R + n, C:C + n])
            g[blk["u"]:blk["u"] + n * r] = du.T.reshape(-1)
            g[blk["v"]:blk["v"] + n * r] = dv.T.reshape(-1)
            g[blk["sig"]:blk["sig"] + r] = ds
        else:
            b, R = blk["b"], blk["row0"]
            g[blk["d"]:blk["d"] + b * b] = dA[R:R + b, R:R + b].T.reshape(-1)
    return g
