"""Parity at the benchmark's own configuration (N = 2^18, 256 RHS).

The benchmark reports the mixed-precision refined solve of the 2D
Gaussian-kernel PLR (262144 kd-ordered points in the unit square, leaf 256,
10 levels, adaptive ranks 8-128, 7-slice bf16 inner solves, exact-slice
residuals) as converged to a relative residual <= 1e-12.  Here the same
matrix, right-hand sides and solve are checked on the host by the oracle,
independently of every GPU residual:

* (b) the double-double residual (oracle/dd_resid.c: A x evaluated with
  error-free transformations, error ~n 2^-104 |A||x|) of every one of the
  256 columns must be <= 1e-12 relative to ||b||;
* (a) the oracle's FP64 dplrgepdmm residual of every column must be within
  1e-12 plus the FP64 product's own rounding.  That rounding is bounded
  (probabilistic bound of Higham and Mary, 2019) by
  lambda sqrt(K) u || |A||x| ||, with u = 2^-53, K = N/2 + leaf + max
  rank + levels + 1 the longest accumulation of one output entry, and
  lambda = 6; || |A||x| || comes from the double-double pass.  The two
  residuals must also agree with each other within that bound.
"""
import numpy as np
import pytest

from dplr_gb300 import tree
from oracle import pyoracle

pytestmark = [pytest.mark.gpu, pytest.mark.slow]
torch = pytest.importorskip("torch")

N, LEAF, RHS, RMAX = 1 << 18, 256, 256, 128


def test_headline_mixed_refined_solve_checked_by_the_oracle():
    from dplr_gb300 import gen_gpu
    from dplr_gb300.plan import GpuPlan
    t = gen_gpu.kernel_tree_2d(n=N, leaf=LEAF, rmax=RMAX, seed=0, device="cuda")
    plan = GpuPlan(t)
    plan.factor()
    plan.prepare_sliced()
    plan.prepare_mixed(7)
    g = torch.Generator(device="cuda")
    g.manual_seed(3)                         # the benchmark's right-hand sides (rank 0)
    B = torch.randn(RHS, N, dtype=torch.float64, device="cuda", generator=g)
    X, res, its = plan.solve_refined(B, tol=1e-12, maxiter=8, precise=True, mixed=True)
    assert res <= 1e-12, res
    Xh, Bh = X.cpu().numpy(), B.cpu().numpy()
    plan.close()
    del X, B
    torch.cuda.empty_cache()

    orc = pyoracle.oracle("best")
    a = tree.to_c(t)
    try:
        y = np.zeros(N * RHS)
        orc.gepdmm("N", "N", N, RHS, 1.0, a, np.ascontiguousarray(Xh).reshape(-1), N, 0.0, y, N)
        bn = np.linalg.norm(Bh, axis=1)
        r64 = np.linalg.norm(Bh - y.reshape(RHS, N), axis=1) / bn
        rdd, absn = pyoracle.resid_dd(orc, a, Xh, Bh)
    finally:
        tree.free_c(a)
    rdd = rdd / bn
    # (b) the exact residual of the stored operator
    assert rdd.max() <= 1e-12, (rdd.max(), int(rdd.argmax()))
    # (a) the FP64 residual, within its own rounding bound
    K = N // 2 + LEAF + RMAX + tree.depth(t) + 1
    bound = 6.0 * np.sqrt(K) * 2.0 ** -53 * absn / bn
    assert np.all(r64 <= 1e-12 + bound), (r64.max(), bound.max())
    assert np.all(np.abs(r64 - rdd) <= bound)
