"""Argument checks of the compression, product and recompression entry
points of libdplr_gb300.so.  They run on the host before any device work
(DPLR's behaviour: an invalid call writes no output), so they are tested
here without a GPU."""
import ctypes

import numpy as np
import pytest

from dplr_gb300 import gen, tree


@pytest.fixture(scope="module")
def lib():
    import os
    from dplr_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        from dplr_gb300 import build
        build.build()
    return _native.lib()


def _err(lib_):
    return lib_.dplr_gpu_last_error().decode()


@pytest.mark.parametrize("m,lda,eps,nlvl,msg", [
    (-2, 1, 1e-8, 0, "invalid matrix size -2"),
    (64, 63, 1e-8, 1, "invalid leading dimension"),
    (64, 64, -1e-8, 1, "eps must be nonnegative"),
    (48, 48, 1e-8, 5, "m not divisible by 2**nlvl"),
])
def test_d2gep_rejects_invalid_arguments(lib, m, lda, eps, nlvl, msg):
    b = tree.new_empty()
    info = ctypes.c_int(123)
    a = np.zeros(max(lda, 1) * max(m, 1))
    try:
        rc = lib.dplr_gpu_d2gep(m, a.ctypes.data, lda, b, eps, nlvl, 0, ctypes.byref(info))
        assert rc == -1 and info.value == -1 and msg in _err(lib)
    finally:
        tree.free_c(b)


def test_d2gep_of_an_empty_matrix_needs_no_device(lib):
    b = tree.new_empty()
    info = ctypes.c_int(123)
    try:
        assert lib.dplr_gpu_d2gep(0, None, 0, b, 1e-8, 1, 0, ctypes.byref(info)) == 0
        assert info.value == 0
    finally:
        tree.free_c(b)


def test_geppmm_rejects_mismatched_or_malformed_trees_before_touching_c(lib):
    a = gen.random_tree(128, 16, 2, seed=1)
    c_tree = gen.random_tree(128, 16, 3, seed=3)
    ca, cc = tree.to_c(a), tree.to_c(c_tree)
    cb = tree.to_c(gen.random_tree(128, 32, 2, seed=2))      # one level fewer
    cd = tree.to_c(tree.Dense(np.eye(128)))
    try:
        cases = [
            ((b"N", b"N", -3, 1.0, ca, ca, 0.0, cc), "dplrppmm: invalid matrix size -3"),
            ((b"T", b"N", 128, 1.0, ca, cb, 0.0, cc), "dplrptpmm: A, B and C type do not match"),
            ((b"N", b"T", 128, 1.0, ca, cd, 0.0, cc), "dplrpptmm: A, B and C type do not match"),
            ((b"T", b"T", 64, 1.0, ca, ca, 0.0, cc), "dplrptptmm: invalid A, B or C size"),
        ]
        for args, msg in cases:
            assert lib.dplr_gpu_geppmm(*args, 1e-8, None) == -1
            assert msg in _err(lib), (msg, _err(lib))
        assert tree.trees_close(tree.from_c(cc), c_tree, rtol=0.0)
        assert lib.dplr_gpu_geppmm(b"N", b"N", 0, 1.0, ca, ca, 0.0, cc, 1e-8, None) == -1  # size 128 != 0
    finally:
        for p in (ca, cb, cc, cd):
            tree.free_c(p)


def test_reduce_svd_checks_and_rank_zero_trees(lib):
    t = gen.random_tree(64, 16, 0, seed=1)            # every block rank 0: nothing to do
    c = tree.to_c(t)
    try:
        assert lib.dplr_gpu_reduce_svd(64, c, 1e-8, 0) == 0
        assert lib.dplr_gpu_reduce_svd(-1, c, 1e-8, 0) == -1
        assert lib.dplr_gpu_reduce_svd(64, c, -1.0, 0) == -1 and "eps" in _err(lib)
        assert lib.dplr_gpu_reduce_svd(32, c, 1e-8, 0) == -1
        assert lib.dplr_gpu_reduce_svd(64, None, 1e-8, 0) == -1
    finally:
        tree.free_c(c)
