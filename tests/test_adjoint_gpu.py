"""Adjoint of the PLR apply and solve (torch.autograd over the C ABI).

Loss of the adjoint workload: L = sum_j ||A^-1 b_j - t_j||^2 on a 1D
exponential-kernel PLR (leaf 128, rank 16).  Gradients with respect to b
and to every stored factor (U, V, sig, leaves) are compared with the FP64
CPU reference gradient (dense LU, projected onto the factors) and with
central finite differences (h = 1e-6).
"""
import numpy as np
import pytest

from dplr_gb300 import gen, tree

from grad_ref import pool_grads, solve_loss_grads

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _case(n=2048, nrhs=2, seed=0):
    rng = np.random.default_rng(seed)
    x = np.sort(rng.uniform(0.0, 1.0, n))
    t = gen.exp1d_tree(x, ell=0.1, shift=1e-2, leaf=128, rank=16, seed=seed + 1)
    b = rng.standard_normal((nrhs, n))
    tt = rng.standard_normal((nrhs, n))
    return t, b, tt


def _loss_and_grads(plan, pool0, b, tt, refine=False):
    from dplr_gb300.autograd import plr_solve
    pool = pool0.clone().requires_grad_()
    bt = torch.tensor(b, device="cuda", requires_grad=True)
    x = plr_solve(plan, pool, bt, refine=refine)
    loss = ((x - torch.tensor(tt, device="cuda")) ** 2).sum()
    loss.backward()
    return float(loss.detach()), pool.grad.detach().cpu().numpy(), bt.grad.detach().cpu().numpy()


def test_solve_gradients_match_cpu_reference():
    from dplr_gb300.plan import GpuPlan
    t, b, tt = _case()
    plan = GpuPlan(t)
    pool0 = plan.read_pool()
    loss, gpool, gb = _loss_and_grads(plan, pool0, b, tt)
    lref, db_ref, dA = solve_loss_grads(tree.to_dense(t), b, tt)
    gref = pool_grads(plan.pool_blocks(), pool0.cpu().numpy(), dA)
    plan.close()
    assert abs(loss - lref) <= 1e-9 * abs(lref)
    assert np.max(np.abs(gb - db_ref)) <= 1e-8 * np.max(np.abs(db_ref))
    assert np.max(np.abs(gpool - gref)) <= 1e-8 * np.max(np.abs(gref))


def test_solve_gradients_central_differences():
    from dplr_gb300.autograd import plr_solve
    from dplr_gb300.plan import GpuPlan
    t, b, tt = _case(n=1024, nrhs=1, seed=4)
    plan = GpuPlan(t)
    pool0 = plan.read_pool()
    _, gpool, gb = _loss_and_grads(plan, pool0, b, tt)
    ttc = torch.tensor(tt, device="cuda")

    def loss_at(pool, bb):
        with torch.no_grad():
            x = plr_solve(plan, pool, torch.tensor(bb, device="cuda"))
            return float(((x - ttc) ** 2).sum())

    blocks = plan.pool_blocks()
    lr = [blk for blk in blocks if blk["kind"] == "lowrank"]
    lf = [blk for blk in blocks if blk["kind"] == "leaf"]
    idx = [lr[0]["u"] + 5, lr[1]["v"] + 17, lr[2]["sig"], lr[-1]["u"] + 40, lr[3]["sig"] + 3,
           lf[0]["d"] + 3 + 7 * lf[0]["b"], lf[-1]["d"] + 0]
    h = 1e-6
    for i in idx:
        p_plus, p_minus = pool0.clone(), pool0.clone()
        p_plus[i] += h
        p_minus[i] -= h
        fd = (loss_at(p_plus, b) - loss_at(p_minus, b)) / (2 * h)
        assert abs(fd - gpool[i]) <= 1e-5 * max(1.0, abs(gpool[i])), (i, fd, gpool[i])
    for (j, i) in [(0, 11), (0, 600)]:
        bp, bm = b.copy(), b.copy()
        bp[j, i] += h
        bm[j, i] -= h
        fd = (loss_at(pool0, bp) - loss_at(pool0, bm)) / (2 * h)
        assert abs(fd - gb[j, i]) <= 1e-5 * max(1.0, abs(gb[j, i])), (j, i, fd, gb[j, i])
    plan.close()


def test_apply_gradients_match_cpu_reference():
    from dplr_gb300.autograd import plr_apply
    from dplr_gb300.plan import GpuPlan
    t, _, _ = _case(n=2048, nrhs=3, seed=7)
    rng = np.random.default_rng(8)
    x = rng.standard_normal((3, t.size))
    w = rng.standard_normal((3, t.size))
    plan = GpuPlan(t)
    pool0 = plan.read_pool()
    pool = pool0.clone().requires_grad_()
    xt = torch.tensor(x, device="cuda", requires_grad=True)
    y = plr_apply(plan, pool, xt)
    (y * torch.tensor(w, device="cuda")).sum().backward()
    A = tree.to_dense(t)
    gref = pool_grads(plan.pool_blocks(), pool0.cpu().numpy(), w.T @ x)
    dx_ref = (A.T @ w.T).T
    gp = pool.grad.cpu().numpy()
    plan.close()
    assert np.max(np.abs(gp - gref)) <= 1e-12 * np.max(np.abs(gref))
    assert np.max(np.abs(xt.grad.cpu().numpy() - dx_ref)) <= 1e-12 * np.max(np.abs(dx_ref))


def test_pool_roundtrip_and_write_invalidates_factorisation():
    from dplr_gb300.plan import GpuPlan
    t, b, _ = _case(n=1024, nrhs=1, seed=9)
    plan = GpuPlan(t)
    plan.factor()
    pool = plan.read_pool()
    plan.write_pool(pool * 2.0)
    assert not plan.factored
    with pytest.raises(Exception):
        plan.solve(torch.tensor(b, device="cuda"))
    back = plan.read_pool()
    assert torch.equal(back, pool * 2.0)
    plan.close()
