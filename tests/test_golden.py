"""Golden vectors (made by the reference's own code) replayed through the
CPU oracle and, on a GPU, through libdplr_gb300.so's C ABI."""
import os

import pytest

import golden_io
from oracle import pyoracle

CASES = golden_io.cases()
IDS = [os.path.basename(c)[:-4] for c in CASES]


@pytest.fixture(scope="module", params=["best", "loops"])
def orc(request):
    return pyoracle.oracle(request.param)


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_oracle_apply_matches_golden(orc, path):
    rec = golden_io.load(path)
    golden_io.replay_pmv(orc, rec, tol=1e-13)
    golden_io.replay_pdmm(orc, rec, tol=1e-13)


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_oracle_prk_matches_golden(orc, path):
    golden_io.replay_prk(orc, golden_io.load(path), tol=1e-12)


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_oracle_inverse_matches_golden(orc, path):
    golden_io.replay_inv(orc, golden_io.load(path), tol=1e-9, dense_tol=1e-11)


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_oracle_counts_match_golden(orc, path):
    from dplr_gb300 import tree
    rec = golden_io.load(path)
    t = golden_io.matrix(rec)
    a = tree.to_c(t)
    try:
        assert orc.nz(t.size, a) == int(rec["nz"][0])
        assert orc.rnk(t.size, a, len(rec["rnk"])) == [int(r) for r in rec["rnk"]]
    finally:
        tree.free_c(a)


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_gpu_apply_matches_golden(path):
    from dplr_gb300 import _native
    api = _native.api()
    rec = golden_io.load(path)
    golden_io.replay_pmv(api, rec, tol=1e-12)
    golden_io.replay_pdmm(api, rec, tol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_gpu_prk_matches_golden(path):
    from dplr_gb300 import _native
    api = _native.api()
    if not api.has("geprk"):
        pytest.skip("dplrgeprk not in this build")
    golden_io.replay_prk(api, golden_io.load(path), tol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_gpu_inverse_matches_golden(path):
    from dplr_gb300 import _native
    api = _native.api()
    if not api.has("geinv"):
        pytest.skip("dplrgeinv not in this build")
    golden_io.replay_inv(api, golden_io.load(path), tol=1e-12, dense_tol=1e-11, sig_tol=1e-10)
