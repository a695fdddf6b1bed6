"""Replay of the golden fixtures (tests/golden/*.npz) through a PlrApi.

The same replay runs against the CPU oracle and against the GPU library,
so both are held to the outputs the reference produced.
"""
from __future__ import annotations

import glob
import os

import numpy as np

from dplr_gb300 import tree

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases() -> list[str]:
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(path: str) -> dict:
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


def matrix(rec: dict):
    return tree.unflatten(rec["A_meta"], rec["A_data"])


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    d = np.linalg.norm(np.asarray(a) - np.asarray(b))
    n = np.linalg.norm(np.asarray(b))
    return float(d / n) if n > 0 else float(d)


def replay_pmv(api, rec: dict, tol: float) -> None:
    t = matrix(rec)
    m = t.size
    a = tree.to_c(t)
    try:
        i = 0
        while f"pmv{i}_cfg" in rec:
            tr, al, be, incx, incy = rec[f"pmv{i}_cfg"]
            x = rec[f"pmv{i}_x"].copy()
            y = rec[f"pmv{i}_y0"].copy()
            api.gepmv(chr(int(tr)), m, float(al), a, x, int(incx), float(be), y, int(incy))
            want = rec[f"pmv{i}_y"]
            # entries off the stride must be untouched
            mask = np.zeros(len(y), bool)
            mask[:: int(incy)] = True
            assert np.array_equal(y[~mask], rec[f"pmv{i}_y0"][~mask]), f"pmv{i} wrote off-stride"
            err = rel_err(y[mask], want[mask])
            assert err <= tol, f"pmv{i} ({chr(int(tr))}, alpha={al}, beta={be}) rel err {err}"
            i += 1
    finally:
        tree.free_c(a)


def replay_pdmm(api, rec: dict, tol: float) -> None:
    t = matrix(rec)
    m = t.size
    a = tree.to_c(t)
    try:
        i = 0
        while f"pdmm{i}_cfg" in rec:
            ta, tb, n, al, be, ldb, ldc = rec[f"pdmm{i}_cfg"]
            b = rec[f"pdmm{i}_B"].copy(order="F")
            c = rec[f"pdmm{i}_C0"].copy(order="F")
            api.gepdmm(chr(int(ta)), chr(int(tb)), m, int(n), float(al), a,
                       b.reshape(-1, order="F"), int(ldb), float(be), c.reshape(-1, order="F"),
                       int(ldc))
            want = rec[f"pdmm{i}_C"]
            assert np.array_equal(c[m:], rec[f"pdmm{i}_C0"][m:]), f"pdmm{i} wrote padding"
            err = rel_err(c[:m], want[:m])
            assert err <= tol, f"pdmm{i} ({chr(int(ta))}{chr(int(tb))}) rel err {err}"
            i += 1
    finally:
        tree.free_c(a)


def compare_trees(got, want, tol: float, where: str = "", scale: float | None = None,
                  sig_tol: float | None = None, allow: float = 0.0) -> None:
    """Same structure and ranks; every block's product U diag(sig) V^T and
    every leaf within tol * scale (Frobenius; scale defaults to the norm of
    the whole matrix); sig entries within sig_tol (default: tol) of the
    block's largest.  `allow` is an absolute allowance added to every bound:
    thresholded inverses (eps > 0) zero a column when its singular value is
    below eps-level, and two rounding paths may decide differently for a
    value right at the threshold, changing a block by at most about eps.

    Factor columns are compared through their products because columns
    whose singular value is negligible point in directions set by
    rounding, which differ between BLAS implementations."""
    if scale is None:
        scale = float(np.linalg.norm(tree.to_dense(want)))
    if sig_tol is None:
        sig_tol = tol
    assert type(got) is type(want), f"{where}: node type differs"
    if isinstance(want, tree.Dense):
        err = float(np.linalg.norm(got.d - want.d))
        assert err <= tol * scale + allow, f"{where}: leaf err {err / scale}"
    elif isinstance(want, tree.LowRank):
        assert got.rank == want.rank, f"{where}: rank {got.rank} != {want.rank}"
        if want.rank:
            pg = (got.u * got.sig) @ got.v.T
            pw = (want.u * want.sig) @ want.v.T
            err = float(np.linalg.norm(pg - pw))
            assert err <= tol * scale + allow, f"{where}: block err {err / scale}"
            smax = float(np.max(np.abs(want.sig)))
            serr = float(np.max(np.abs(got.sig - want.sig)))
            assert serr <= sig_tol * max(smax, 1e-300) + allow + 1e-300, \
                f"{where}: sig err {serr / smax}"
    else:
        for q in ("nw", "ne", "se", "sw"):
            compare_trees(getattr(got, q), getattr(want, q), tol, where + "." + q, scale, sig_tol,
                          allow)


def replay_prk(api, rec: dict, tol: float) -> None:
    t = matrix(rec)
    m = t.size
    u, v, s = rec["prk_u"], rec["prk_v"], rec["prk_s"]
    i = 0
    while f"prk{i}_cfg" in rec:
        k, al, ep = rec[f"prk{i}_cfg"]
        a = tree.to_c(t)
        try:
            api.geprk(m, int(k), float(al), u.reshape(-1, order="F").copy(), m,
                      v.reshape(-1, order="F").copy(), m, s.copy(), 1, a, float(ep))
            got = tree.from_c(a)
        finally:
            tree.free_c(a)
        want = tree.unflatten(rec[f"prk{i}_meta"], rec[f"prk{i}_data"])
        compare_trees(got, want, tol, f"prk{i}")
        i += 1


def replay_inv(api, rec: dict, tol: float, dense_tol: float, sig_tol: float | None = None) -> None:
    t = matrix(rec)
    m = t.size
    i = 0
    while f"inv{i}_cfg" in rec:
        ep, info_want = rec[f"inv{i}_cfg"]
        a = tree.to_c(t)
        b = tree.new_empty()
        try:
            info = api.geinv(m, a, b, float(ep))
            got = tree.from_c(b)
        finally:
            tree.free_c(a)
            tree.free_c(b)
        assert info == int(info_want), f"inv{i}: info {info} != {info_want}"
        want = tree.unflatten(rec[f"inv{i}_meta"], rec[f"inv{i}_data"])
        e = rel_err(tree.to_dense(got), tree.to_dense(want))
        assert e <= dense_tol, f"inv{i}: dense rel err {e}"
        compare_trees(got, want, tol, f"inv{i}", sig_tol=sig_tol, allow=2.0 * float(ep))
        i += 1
