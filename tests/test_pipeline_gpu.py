"""The reference driver's flow end to end on the GPU, at the reference's
CPU-runnable size: N = 4096 sorted uniform points, exp(-|x_i - x_j|/0.1)
+ 1e-2 I, compressed with eps = 1e-10 into 6 levels (leaves of 64), then
y = A x, B = inv(A) and x' = B y (dplrd2gep, dplrgepmv, dplrgeinv,
dplrgepmv; the sequence of test/testdplr.c).  Every step is checked
against the oracle (the reference's algorithm on the CPU) on the same
inputs."""
import numpy as np
import pytest

from dplr_gb300 import gen, tree
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _dense():
    x = gen.sorted_uniform(4096, seed=0)
    return gen.exp_kernel_1d(x, 0.1, 1e-2)


def _rank_ranges(a: np.ndarray, eps: float, nlvl: int):
    """Per block in DPLR's order (NE, SW, NW, SE): the ranks dplrd2gep's
    rule can give, (lo, hi).  Singular values further than the SVD's
    rounding (4 eps_64 sigma_1 sqrt(n), from numpy's SVD) from the block's
    threshold are decided by the matrix; those within it may fall on either
    side in any SVD code, the reference's dgesvd included.  At eps = 1e-10
    the deepest thresholds sit at that rounding level."""
    out = []

    def rec(blk, e, lv):
        if lv == 0:
            return
        e2 = e / 2.0 if lv == 1 else e / 4.0
        h = blk.shape[0] // 2
        for off in (blk[:h, h:], blk[h:, :h]):
            s = np.linalg.svd(off, compute_uv=False)
            noise = 4 * 2.2e-16 * s[0] * np.sqrt(h)
            out.append((int(np.sum(s >= e2 + noise)), int(np.sum(s >= e2 - noise))))
        rec(blk[:h, :h], e2, lv - 1)
        rec(blk[h:, h:], e2, lv - 1)

    rec(a, eps, nlvl)
    return out


def _ranks_in_order(t, out=None):
    out = [] if out is None else out
    if isinstance(t, tree.HNode):
        out += [t.ne.rank, t.sw.rank]
        _ranks_in_order(t.nw, out)
        _ranks_in_order(t.se, out)
    return out


def test_compress_apply_invert_apply_matches_the_oracle():
    from dplr_gb300 import _native, compress
    gpu = _native.api()
    orc = pyoracle.oracle("best")
    a = _dense()
    t = compress.d2gep(a, 1e-10, 6)
    # compression: DPLR's ranks, up to singular values within rounding of
    # a threshold
    got = _ranks_in_order(t)
    ranges = _rank_ranges(a, 1e-10, 6)
    assert len(got) == len(ranges)
    assert all(lo <= g <= hi for g, (lo, hi) in zip(got, ranges)), list(zip(got, ranges))
    assert np.abs(tree.to_dense(t) - a).max() <= 1e-10 * 6

    m = 4096
    rng = np.random.default_rng(1)
    x = rng.standard_normal(m)
    ct = tree.to_c(t)
    b_gpu, b_orc = tree.new_empty(), tree.new_empty()
    try:
        # y = A x
        y_gpu, y_orc = np.zeros(m), np.zeros(m)
        gpu.gepmv("N", m, 1.0, ct, x, 1, 0.0, y_gpu, 1)
        orc.gepmv("N", m, 1.0, ct, x, 1, 0.0, y_orc, 1)
        assert np.linalg.norm(y_gpu - y_orc) <= 1e-12 * np.linalg.norm(y_orc)
        # B = inv(A), both ways
        assert gpu.geinv(m, ct, b_gpu, 1e-10) == 0
        assert orc.geinv(m, ct, b_orc, 1e-10) == 0
        # x' = B y
        xg, xo = np.zeros(m), np.zeros(m)
        gpu.gepmv("N", m, 1.0, b_gpu, y_gpu, 1, 0.0, xg, 1)
        orc.gepmv("N", m, 1.0, b_orc, y_orc, 1, 0.0, xo, 1)
        assert np.linalg.norm(xg - xo) <= 1e-8 * np.linalg.norm(xo)
        assert np.linalg.norm(xg - x) <= 1e-6 * np.linalg.norm(x)
        # the inverse trees agree in structure and ranks
        tg, to = tree.from_c(b_gpu), tree.from_c(b_orc)
        assert _ranks_in_order(tg) == _ranks_in_order(to)
    finally:
        tree.free_c(ct)
        tree.free_c(b_gpu)
        tree.free_c(b_orc)
