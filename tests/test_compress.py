"""Dense -> PLR compression (dplrd2gep, src/dplrd2p.c:186).

The golden fixtures exp256 and invdist256 hold trees that the reference's
own dplrd2gep made from dense inputs rebuilt here: the numpy restatement
(gen.compress_dense) is pinned against them on the CPU, and the GPU
library's dplrd2gep (SVDs by its own batched kernel up to 64 rows, by
cuSOLVER above) is held to the same trees and to the
restatement on larger inputs.  Singular vectors are compared through the
blocks they build (their signs are the SVD's choice); ranks must be equal.
"""
import os

import numpy as np
import pytest

import golden_io
from dplr_gb300 import gen, tree

GOLDEN = golden_io.GOLDEN


def _fixture_inputs():
    """The dense matrices the fixtures were compressed from, with eps."""
    x = gen.sorted_uniform(256, seed=11)
    yield "exp256", gen.exp_kernel_1d(x, 0.1, 1e-2), 1e-10
    i = np.arange(256)
    d = np.abs(i[:, None] - i[None, :]).astype(float)
    yield "invdist256", np.where(d == 0, 0.0, 1.0 / np.where(d == 0, 1.0, d)), 1e-6


FIXTURES = list(_fixture_inputs())


def _gauss2d(m: int, seed: int) -> np.ndarray:
    pts = np.random.default_rng(seed).random((m, 2))
    # sort along a Morton-like key so that index blocks are spatial clusters
    key = np.argsort(np.floor(pts[:, 0] * 16) * 16 + pts[:, 1])
    pts = pts[key]
    d2 = ((pts[:, None, :] - pts[None, :, :]) ** 2).sum(-1)
    return np.exp(-d2 / 0.05) + 1e-3 * np.eye(m)


def assert_same_tree(got, want, sig_atol: float, blk_atol: float, leaf_atol: float = 0.0,
                     path: str = "") -> None:
    """Same structure and ranks, leaves within leaf_atol (bitwise by
    default), sig and blocks within tol (relative to the block's largest
    singular value when that exceeds 1)."""
    assert type(got) is type(want), path
    assert got.size == want.size, path
    if isinstance(want, tree.HNode):
        for k in ("nw", "ne", "se", "sw"):
            assert_same_tree(getattr(got, k), getattr(want, k), sig_atol, blk_atol, leaf_atol, path + k + "/")
    elif isinstance(want, tree.LowRank):
        assert got.rank == want.rank, (path, got.rank, want.rank)
        if want.rank:
            scale = max(1.0, float(want.sig[0]))
            np.testing.assert_allclose(got.sig, want.sig, rtol=0, atol=sig_atol * scale, err_msg=path)
            blk_g = (got.u * got.sig) @ got.v.T
            blk_w = (want.u * want.sig) @ want.v.T
            np.testing.assert_allclose(blk_g, blk_w, rtol=0, atol=blk_atol * scale, err_msg=path)
            # orthonormal columns, as an SVD gives them
            np.testing.assert_allclose(got.u.T @ got.u, np.eye(got.rank), atol=1e-12, err_msg=path)
            np.testing.assert_allclose(got.v.T @ got.v, np.eye(got.rank), atol=1e-12, err_msg=path)
    else:
        np.testing.assert_allclose(got.d, want.d, rtol=0, atol=leaf_atol, err_msg=path)


def _reconstruction_ok(t, a: np.ndarray, eps: float) -> None:
    # each level spends at most eps in total over its blocks
    err = np.abs(tree.to_dense(t) - a).max()
    assert err <= eps * max(1.0, np.log2(a.shape[0])), err


# ---------------------------------------------------------------- CPU -----

@pytest.mark.parametrize("name,a,eps", FIXTURES, ids=[f[0] for f in FIXTURES])
def test_restatement_matches_reference_compression(name, a, eps):
    want = golden_io.matrix(golden_io.load(os.path.join(GOLDEN, name + ".npz")))
    got = gen.compress_dense(a, eps, tree.depth(want))
    # the dense input is rebuilt with this host's exp(), which may differ
    # from the one the fixture was made with in the last bit
    assert_same_tree(got, want, sig_atol=1e-14, blk_atol=1e-14, leaf_atol=1e-15)


def test_restatement_rejects_uneven_levels():
    with pytest.raises(ValueError):
        gen.compress_dense(np.eye(12), 1e-8, 3)


# ---------------------------------------------------------------- GPU -----

def _api():
    from dplr_gb300 import _native
    api = _native.api()
    if not api.has("d2gep"):
        pytest.fail("dplrd2gep missing from libdplr_gb300.so")
    return api


def _gpu_compress(api, a: np.ndarray, eps: float, nlvl: int, lda: int | None = None, b=None):
    m = a.shape[0]
    lda = m if lda is None else lda
    buf = np.zeros((lda, m), order="F")
    buf[:m] = a
    own = b is None
    b = tree.new_empty() if own else b
    info = api.d2gep(m, buf, lda, b, eps, nlvl)
    out = tree.from_c(b) if info == 0 else None
    if own:
        tree.free_c(b)
    return info, out


@pytest.mark.gpu
@pytest.mark.parametrize("name,a,eps", FIXTURES, ids=[f[0] for f in FIXTURES])
def test_gpu_compression_matches_reference_fixtures(name, a, eps):
    api = _api()
    want = golden_io.matrix(golden_io.load(os.path.join(GOLDEN, name + ".npz")))
    info, got = _gpu_compress(api, a, eps, tree.depth(want))
    assert info == 0
    # the dense input is rebuilt with this host's exp(), which may differ
    # from the one the fixture was made with in the last bit
    assert_same_tree(got, want, sig_atol=1e-14, blk_atol=1e-14, leaf_atol=1e-15)
    # leaves are copies of the input
    assert_same_tree(got, gen.compress_dense(a, eps, tree.depth(want)), sig_atol=1e-13, blk_atol=1e-13)
    _reconstruction_ok(got, a, eps)


@pytest.mark.gpu
@pytest.mark.parametrize("m,nlvl,eps", [(1024, 4, 1e-8), (512, 2, 1e-10), (768, 3, 1e-6), (2048, 3, 1e-9)])
def test_gpu_compression_matches_restatement(m, nlvl, eps):
    api = _api()
    a = _gauss2d(m, seed=m + nlvl)
    want = gen.compress_dense(a, eps, nlvl)
    info, got = _gpu_compress(api, a, eps, nlvl, lda=m + 5)
    assert info == 0
    assert_same_tree(got, want, sig_atol=1e-13, blk_atol=1e-13)
    _reconstruction_ok(got, a, eps)


@pytest.mark.gpu
def test_gpu_compression_edge_cases():
    api = _api()
    rng = np.random.default_rng(5)
    a = rng.standard_normal((64, 64))
    # nlvl = 0: a dense copy
    info, got = _gpu_compress(api, a, 1e-8, 0, lda=70)
    assert info == 0 and isinstance(got, tree.Dense)
    np.testing.assert_array_equal(got.d, a)
    # eps = 0 keeps every nonzero singular value: full rank for a random matrix
    info, got = _gpu_compress(api, a, 0.0, 2)
    assert info == 0 and got.ne.rank == 32 and got.nw.sw.rank == 16
    np.testing.assert_allclose(tree.to_dense(got), a, atol=1e-12)
    # a zero matrix compresses to rank 0 everywhere
    info, got = _gpu_compress(api, np.zeros((64, 64)), 1e-8, 3)
    assert info == 0 and max(tree.ranks_by_level(got)) == 0
    assert not tree.to_dense(got).any()


@pytest.mark.gpu
def test_gpu_compression_reuses_and_rebuilds_b():
    api = _api()
    a = _gauss2d(256, seed=9)
    b = tree.new_empty()
    try:
        for eps, nlvl in [(1e-4, 2), (1e-10, 2), (1e-8, 3), (1e-6, 0), (1e-9, 1)]:
            info = api.d2gep(256, np.asfortranarray(a), 256, b, eps, nlvl)
            assert info == 0
            assert_same_tree(tree.from_c(b), gen.compress_dense(a, eps, nlvl), sig_atol=1e-13,
                             blk_atol=1e-13)
    finally:
        tree.free_c(b)


@pytest.mark.gpu
@pytest.mark.parametrize("m,lda,eps,nlvl", [(-1, 1, 1e-8, 0), (64, 63, 1e-8, 1), (64, 64, -1.0, 1),
                                            (48, 48, 1e-8, 5)])
def test_gpu_compression_invalid_arguments(m, lda, eps, nlvl):
    api = _api()
    b = tree.new_empty()
    try:
        info = api.d2gep(m, np.zeros(max(lda, 1) * max(m, 1)), lda, b, eps, nlvl)
        assert info == -1
    finally:
        tree.free_c(b)


def test_lapack_leg_matches_reference_ranks():
    """The bench's CPU leg (dgesvd and gesdd restatements) keeps the
    reference's ranks on the fixture inputs."""
    from dplr_gb300 import workloads
    for name, a, eps in FIXTURES:
        want = golden_io.matrix(golden_io.load(os.path.join(GOLDEN, name + ".npz")))
        nlvl = tree.depth(want)
        for driver in ("gesvd", "gesdd"):
            assert workloads._lapack_compress(a, eps, nlvl, driver) == workloads._ranks_all(want), (name, driver)


def test_gauss2d_dense_is_symmetric_and_clustered():
    from dplr_gb300 import workloads
    a = workloads.gauss2d_dense(1024, seed=1)
    np.testing.assert_array_equal(a, a.T)
    t = gen.compress_dense(a, 1e-8, 2)
    r = tree.ranks_by_level(t)
    assert r[0] < 512 // 4 and r[1] < 256 // 2    # off-diagonal blocks are low rank


@pytest.mark.gpu
def test_gpu_compression_worker_count_does_not_change_results():
    from dplr_gb300 import compress, workloads
    a = workloads.gauss2d_dense(1024, seed=4)
    one = compress.d2gep(a, 1e-9, 4, workers=1)
    many = compress.d2gep(a, 1e-9, 4, workers=8)
    ma, da = tree.flatten(one)
    mb, db = tree.flatten(many)
    np.testing.assert_array_equal(ma, mb)
    np.testing.assert_array_equal(da, db)


@pytest.mark.gpu
def test_gpu_compression_rejects_malformed_b():
    """A reused H node whose off-diagonal child is not low rank: info -1
    (dplrlrappx's type check, src/dplrd2p.c:48)."""
    api = _api()
    leaf = lambda n: tree.Dense(np.zeros((n, n), order="F"))
    bad = tree.HNode(leaf(32), leaf(32), leaf(32), leaf(32))
    b = tree.to_c(bad)
    try:
        assert api.d2gep(64, np.asfortranarray(np.eye(64)), 64, b, 1e-8, 1) == -1
    finally:
        tree.free_c(b)


@pytest.mark.gpu
def test_python_wrapper_raises_on_invalid_arguments():
    from dplr_gb300 import _native, compress
    with pytest.raises(_native.NativeError, match="divisible"):
        compress.d2gep(np.eye(48), 1e-8, 5)


@pytest.mark.gpu
def test_gpu_compression_full_rank_blocks_fall_back_to_the_full_svd():
    """Blocks of 512 with no decay (random entries): the sketch cannot pass
    its residual check, the full SVD decides; ranks are full."""
    api = _api()
    a = np.random.default_rng(17).standard_normal((1024, 1024))
    info, got = _gpu_compress(api, a, 1e-8, 1)
    assert info == 0 and got.ne.rank == 512 and got.sw.rank == 512
    want = gen.compress_dense(a, 1e-8, 1)
    assert_same_tree(got, want, sig_atol=1e-12, blk_atol=1e-12)


def test_python_wrapper_checks_shape_before_any_device_call():
    from dplr_gb300 import compress
    with pytest.raises(ValueError):
        compress.d2gep(np.zeros((4, 6)), 1e-8, 1)
