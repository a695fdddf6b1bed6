"""FP64-accurate 1-RHS apply on the FP32 pipes (dplr_gpu_prepare_pairs).

After prepare_pairs, op-N applies with one right-hand side run the float-pair
kernels.  They are checked:
- against the FP64 oracle (1e-12 relative, the parity bar of the apply);
- against the FP64 GPU kernels (1e-13: the pairs keep 48 bits and compensate
  their sums);
- on alpha/beta, zero and extreme-scale vectors;
- after pool writes, and on batched plans, op-T and multi-RHS applies (which
  keep the FP64 kernels);
- on the range check of the factors.
"""
import numpy as np
import pytest
import torch

from dplr_gb300 import gen, tree
from oracle import pyoracle

pytestmark = pytest.mark.gpu
TOL = 1e-12

TREES = {
    "uniform1k": lambda: gen.random_tree(1024, 64, 16, seed=1),
    "uneven2k": lambda: gen.random_tree(2048, 32, [70, 0, 9, 33, 1, 5], seed=2, capacity_extra=3),
    "exp4k": lambda: gen.exp1d_tree(gen.sorted_uniform(4096, 5), 0.1, 1e-2, 64, 8, seed=5),
    "rank160": lambda: gen.random_tree(2048, 128, [160, 140, 100, 40], seed=9),
}


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def orc():
    return pyoracle.oracle("best")


def oracle_apply(orc, t, x, alpha=1.0, beta=0.0, y=None):
    a = tree.to_c(t)
    out = np.zeros(t.size) if y is None else y.copy()
    orc.gepmv("N", t.size, alpha, a, x.copy(), 1, beta, out, 1)
    tree.free_c(a)
    return out


def plans(t):
    from dplr_gb300.plan import GpuPlan
    p64, pp = GpuPlan(t), GpuPlan(t)
    pp.prepare_pairs()
    return p64, pp


@pytest.mark.parametrize("name", list(TREES))
def test_pair_apply_matches_oracle_and_fp64(orc, name):
    t = TREES[name]()
    x = np.random.default_rng(7).standard_normal(t.size)
    want = oracle_apply(orc, t, x)
    p64, pp = plans(t)
    xt = torch.tensor(x, device="cuda").reshape(1, -1)
    y64 = p64.apply(xt).cpu().numpy().ravel()
    yp = pp.apply(xt).cpu().numpy().ravel()
    p64.close()
    pp.close()
    assert rel(yp, want) <= TOL
    assert rel(yp, y64) <= 1e-13


def test_pair_apply_kernel_matrix_2d():
    """The bench's matrix family at N = 16384 (leaf 128, ranks to 96)."""
    from dplr_gb300 import gen_gpu
    t = gen_gpu.kernel_tree_2d(n=16384, leaf=128, rmax=96, seed=6)
    x = torch.randn(1, t.size, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    p64, pp = plans(t)
    y64, yp = p64.apply(x), pp.apply(x)
    p64.close()
    pp.close()
    assert float((yp - y64).norm() / y64.norm()) <= 1e-13


def test_pair_apply_alpha_beta(orc):
    t = TREES["exp4k"]()
    rng = np.random.default_rng(11)
    x, y0 = rng.standard_normal(t.size), rng.standard_normal(t.size)
    want = oracle_apply(orc, t, x, alpha=-2.5, beta=0.75, y=y0)
    _, pp = plans(t)
    out = torch.tensor(y0, device="cuda").reshape(1, -1)
    pp.apply(torch.tensor(x, device="cuda").reshape(1, -1), alpha=-2.5, beta=0.75, out=out)
    pp.close()
    assert rel(out.cpu().numpy().ravel(), want) <= TOL


def test_pair_apply_zero_and_extreme_vectors():
    t = TREES["uniform1k"]()
    p64, pp = plans(t)
    zero = torch.zeros(1, t.size, dtype=torch.float64, device="cuda")
    assert float(pp.apply(zero).abs().max()) == 0.0
    x = torch.randn(1, t.size, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(5))
    for s in (1e-250, 1e-30, 1.0, 1e30, 1e250):
        y64, yp = p64.apply(x * s), pp.apply(x * s)
        assert torch.isfinite(yp).all()
        # norms of the unscaled results (squares of 1e-250 underflow)
        assert float(((yp - y64) / s).norm() / (y64 / s).norm()) <= 1e-13, s
    p64.close()
    pp.close()


def test_pair_copy_follows_pool_write(orc):
    t = TREES["exp4k"]()
    _, pp = plans(t)
    pool = pp.read_pool()
    pp.write_pool(pool * 3.0)                 # every pool entry tripled: a different matrix
    x = torch.randn(1, t.size, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(2))
    from dplr_gb300.plan import GpuPlan
    ref = GpuPlan(t)
    ref.write_pool(pool * 3.0)
    y_ref, yp = ref.apply(x), pp.apply(x)
    ref.close()
    pp.close()
    assert float((yp - y_ref).norm() / y_ref.norm()) <= 1e-13


def test_pair_plan_other_applies_use_fp64(orc):
    """op T and several right-hand sides keep the FP64 kernels (exact agreement)."""
    t = TREES["uneven2k"]()
    p64, pp = plans(t)
    x = torch.randn(3, t.size, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(4))
    assert torch.equal(pp.apply(x), p64.apply(x))
    assert torch.equal(pp.apply(x[:1], trans="T"), p64.apply(x[:1], trans="T"))
    p64.close()
    pp.close()


def test_pair_apply_batched_plan():
    from dplr_gb300.plan import GpuPlan
    trees = [gen.random_tree(512, 32, 8, seed=s) for s in range(5)] + [gen.random_tree(1024, 64, 12, seed=9)]
    b64, bp = GpuPlan.batch(trees), GpuPlan.batch(trees)
    bp.prepare_pairs()
    x = torch.randn(1, b64.m, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(8))
    y64, yp = b64.apply(x), bp.apply(x)
    b64.close()
    bp.close()
    assert float((yp - y64).norm() / y64.norm()) <= 1e-13


def test_pair_range_check():
    """Factors beyond 2^50 would overflow FP32 products: prepare refuses, and
    a pool write that leaves the range drops the copy (FP64 kernels again)."""
    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan
    t = TREES["uniform1k"]()
    p = GpuPlan(t)
    pool = p.read_pool()
    p.write_pool(pool * 2.0 ** 60)
    with pytest.raises(_native.NativeError):
        p.prepare_pairs()
    p.write_pool(pool)
    p.prepare_pairs()
    p.write_pool(pool * 2.0 ** 60)            # accepted; the pair copy is dropped
    x = torch.randn(1, t.size, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(1))
    ref = GpuPlan(t)
    ref.write_pool(pool * 2.0 ** 60)
    assert torch.equal(p.apply(x), ref.apply(x))
    p.close()
    ref.close()
