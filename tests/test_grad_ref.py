"""The CPU reference gradient of the solve loss against central finite
differences (h = 1e-6) on a small PLR tree: checks the adjoint formulas
that the GPU gradient is compared with."""
import numpy as np

from dplr_gb300 import gen, tree

from grad_ref import solve_loss, solve_loss_grads, tree_grads


def _loss(t, b, tt):
    return solve_loss(tree.to_dense(t), b, tt)


def test_reference_gradient_matches_central_differences():
    rng = np.random.default_rng(3)
    x = np.sort(rng.uniform(0.0, 1.0, 128))
    t = gen.exp1d_tree(x, ell=0.1, shift=1e-2, leaf=16, rank=4, seed=1)
    b = rng.standard_normal((2, 128))
    tt = rng.standard_normal((2, 128))
    _, db, dA = solve_loss_grads(tree.to_dense(t), b, tt)
    g = tree_grads(t, dA)
    h = 1e-6
    checks = []
    # b entries
    for (j, i) in [(0, 3), (1, 77)]:
        bp, bm = b.copy(), b.copy()
        bp[j, i] += h
        bm[j, i] -= h
        checks.append(((solve_loss(tree.to_dense(t), bp, tt) - solve_loss(tree.to_dense(t), bm, tt)) / (2 * h),
                       db[j, i]))
    # factor entries: (path, attribute, index)
    cases = [("ne", "u", (5, 0)), ("sw", "v", (9, 1)), ("ne", "sig", (0,)), ("nw.sw", "u", (3, 2)),
             ("se.se.ne", "v", (2, 0))]
    for path, attr, idx in cases:
        node = t
        for part in path.split("."):
            node = getattr(node, part)
        arr = getattr(node, attr)
        old = arr[idx]
        arr[idx] = old + h
        lp = _loss(t, b, tt)
        arr[idx] = old - h
        lm = _loss(t, b, tt)
        arr[idx] = old
        du, ds, dv = g[path]
        want = {"u": du, "v": dv, "sig": ds}[attr][idx]
        checks.append(((lp - lm) / (2 * h), want))
    # a leaf entry
    leaf = t.nw.nw.nw
    old = leaf.d[2, 5]
    leaf.d[2, 5] = old + h
    lp = _loss(t, b, tt)
    leaf.d[2, 5] = old - h
    lm = _loss(t, b, tt)
    leaf.d[2, 5] = old
    checks.append(((lp - lm) / (2 * h), g["nw.nw.nw"][2, 5]))
    for fd, an in checks:
        assert abs(fd - an) <= 1e-5 * max(1.0, abs(an)), (fd, an)
