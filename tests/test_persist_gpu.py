"""The one-launch persistent FP64 apply (csrc/persist.cu) against the oracle
and against the three-launch apply (DPLR_GB300_APPLY=launches).

Trees cover every rank tile the kernel picks (ranks 1-4 -> 8 columns, up to
100 -> two tiles of 64), rank-0 levels, ragged leaf sizes, one and many
right-hand sides (1, 3, 16, 40: right-hand-side tiles of 1, 2, 16 and a
ragged last tile), both ops, alpha/beta combinations and a batch of trees.
"""
import os

import numpy as np
import pytest

from dplr_gb300 import gen, tree
from oracle import pyoracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TREES = {
    "small_ranks": lambda: gen.random_tree(2048, 64, lambda lv, rng: int(rng.integers(1, 5)), seed=1),
    "mixed": lambda: gen.random_tree(2048, 64, [100, 40, 17, 9, 0, 3], seed=2),
    "exp1d": lambda: gen.exp1d_tree(gen.sorted_uniform(4096, 3), 0.1, 1e-2, 128, 4, seed=3),
    "leaf48": lambda: gen.random_tree(1536, 48, [20, 12, 6, 2, 1], seed=4),
}


def _apply(plan, x, trans, alpha, beta, y0, mode):
    old = os.environ.get("DPLR_GB300_APPLY")
    if mode:
        os.environ["DPLR_GB300_APPLY"] = mode
    else:
        os.environ.pop("DPLR_GB300_APPLY", None)
    try:
        y = y0.clone()
        plan.apply(x, trans=trans, alpha=alpha, beta=beta, out=y)
        torch.cuda.synchronize()
        return y
    finally:
        if old is None:
            os.environ.pop("DPLR_GB300_APPLY", None)
        else:
            os.environ["DPLR_GB300_APPLY"] = old


@pytest.mark.parametrize("name", list(TREES))
@pytest.mark.parametrize("nrhs", [1, 3, 16, 40])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_persistent_apply_matches_oracle_and_launches(name, nrhs, trans):
    from dplr_gb300.plan import GpuPlan
    t = TREES[name]()
    m = t.size
    plan = GpuPlan(t)
    g = torch.Generator(device="cpu").manual_seed(nrhs)
    x = torch.randn(nrhs, m, generator=g, dtype=torch.float64).cuda()
    y0 = torch.randn(nrhs, m, generator=g, dtype=torch.float64).cuda()
    for alpha, beta in ((1.0, 0.0), (-0.75, 1.25)):
        yp = _apply(plan, x, trans, alpha, beta, y0, None)
        yl = _apply(plan, x, trans, alpha, beta, y0, "launches")
        a = tree.to_c(t)
        want = y0.cpu().numpy().reshape(-1).copy()
        pyoracle.oracle("best").gepdmm(trans, "N", m, nrhs, alpha, a, x.cpu().numpy().reshape(-1), m, beta,
                                       want, m)
        tree.free_c(a)
        wn = np.linalg.norm(want)
        assert np.linalg.norm(yp.cpu().numpy().reshape(-1) - want) <= 1e-12 * wn
        assert float((yp - yl).norm()) <= 1e-13 * wn
    plan.close()


def test_persistent_apply_is_deterministic():
    from dplr_gb300.plan import GpuPlan
    t = TREES["mixed"]()
    plan = GpuPlan(t)
    x = torch.randn(16, t.size, dtype=torch.float64, device="cuda")
    y1 = plan.apply(x)
    y2 = plan.apply(x)
    assert torch.equal(y1, y2)
    plan.close()


def test_persistent_apply_on_a_batch():
    from dplr_gb300.plan import GpuPlan
    trees = [TREES["small_ranks"](), TREES["exp1d"](), gen.random_tree(512, 32, [5, 3, 1], seed=9)]
    plan = GpuPlan.batch(trees)
    offs = plan.offsets()
    x = torch.randn(5, plan.m, dtype=torch.float64, device="cuda")
    y = plan.apply(x).cpu().numpy()
    xh = x.cpu().numpy()
    orc = pyoracle.oracle("best")
    for o, t in zip(offs, trees):
        a = tree.to_c(t)
        want = np.zeros(5 * t.size)
        orc.gepdmm("N", "N", t.size, 5, 1.0, a, np.ascontiguousarray(xh[:, o:o + t.size]).reshape(-1), t.size,
                   0.0, want, t.size)
        tree.free_c(a)
        got = y[:, o:o + t.size].reshape(-1)
        assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
    plan.close()


def test_persistent_apply_in_a_captured_graph():
    """The persistent apply (a memset node and one kernel) replays from the
    library's CUDA graph with the same result as a direct call."""
    from dplr_gb300.plan import GpuGraph, GpuPlan
    t = TREES["mixed"]()
    plan = GpuPlan(t)
    x = torch.randn(8, t.size, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    g = GpuGraph(plan, "A", x, y)
    g.launch()
    torch.cuda.synchronize()
    assert torch.equal(y, plan.apply(x))
    g.close()
    plan.close()
