"""Generate the golden vectors in tests/golden/*.npz from the reference.

Runs the reference's own C sources (built in place into
oracle/_ref/libdplr_ref.so by oracle/build_oracle.py --ref, linked to
scipy's OpenBLAS) on small seeded cases and stores inputs and outputs:

* trees compressed by the reference's dplrd2gep from dense kernels
  (1D exponential kernel; the 1/|i-j| matrix of the reference's own test
  driver test/testdplr.c:44-53 at a reduced size), plus a seeded random
  tree with uneven ranks, a rank-0 level and spare capacity;
* dplrgepmv (both ops; unit and non-unit strides; alpha == 0; beta == 0),
  dplrgepdmm (all four op combinations, padded leading dimensions),
  dplrgeprk, dplrgeinv (eps = 0 and eps > 0), dplrnz, dplrrnk.

The fixtures are replayed by tests/test_golden.py against the oracle
(CPU) and against the GPU library.  Re-run with
``python tests/golden/make_golden.py`` (needs the reference tree).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from dplr_gb300 import gen, tree  # noqa: E402
from oracle import build_oracle, pyoracle  # noqa: E402


def reference_api():
    build_oracle.build_reference()
    api = pyoracle.reference()
    if api is None:
        raise SystemExit("reference library unavailable (needs the reference sources)")
    return api


def d2gep(api, a: np.ndarray, eps: float, nlvl: int):
    """Compress with the reference's dplrd2gep (src/dplrd2p.c:186)."""
    import ctypes
    from dplr_gb300.tree import c_double_p
    m = a.shape[0]
    f = api.lib.dplrd2gep
    f.restype = None
    f.argtypes = [ctypes.c_int, c_double_p, ctypes.c_int, tree.PDPlrMtx, ctypes.c_double,
                  ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    b = tree.new_empty()
    info = ctypes.c_int(-99)
    af = np.asfortranarray(a)
    f(m, af.ctypes.data_as(c_double_p), m, b, eps, nlvl, ctypes.byref(info))
    assert info.value == 0, info.value
    out = tree.from_c(b)
    tree.free_c(b)
    return out


def record_case(api, name: str, t, eps_inv: float, seed: int) -> None:
    rng = np.random.default_rng(seed)
    m = t.size
    nlvl = tree.depth(t)
    rec: dict[str, np.ndarray] = {}
    meta, data = tree.flatten(t)
    rec["A_meta"], rec["A_data"] = meta, data

    a = tree.to_c(t)
    rec["nz"] = np.array([api.nz(m, a)])
    rec["rnk"] = np.array(api.rnk(m, a, nlvl))

    # dplrgepmv: (trans, alpha, beta, incx, incy)
    pmv_cases = [("N", 1.5, 0.5, 1, 1), ("T", -0.75, 2.0, 1, 1), ("N", 1.0, 0.0, 2, 3),
                 ("T", 0.5, 1.0, 3, 2), ("N", 0.0, 0.7, 1, 1), ("T", 0.0, 0.0, 1, 1)]
    for i, (tr, al, be, incx, incy) in enumerate(pmv_cases):
        x = rng.standard_normal(m * incx)
        y = rng.standard_normal(m * incy)
        rec[f"pmv{i}_cfg"] = np.array([ord(tr), al, be, incx, incy])
        rec[f"pmv{i}_x"], rec[f"pmv{i}_y0"] = x.copy(), y.copy()
        api.gepmv(tr, m, al, a, x, incx, be, y, incy)
        rec[f"pmv{i}_y"] = y

    # dplrgepdmm: (transa, transb, n, alpha, beta, pad_b, pad_c)
    pdmm_cases = [("N", "N", 5, 1.25, 0.0, 0, 0), ("T", "N", 4, -0.75, 0.25, 3, 1),
                  ("N", "T", 3, 0.5, 1.0, 2, 4), ("T", "T", 6, 2.0, -1.0, 1, 2),
                  ("N", "N", 2, 0.0, 0.5, 0, 0)]
    for i, (ta, tb, n, al, be, pb, pc) in enumerate(pdmm_cases):
        rows_b, cols_b = (m, n) if tb == "N" else (n, m)
        ldb, ldc = rows_b + pb, m + pc
        b = np.asfortranarray(rng.standard_normal((ldb, cols_b)))
        c = np.asfortranarray(rng.standard_normal((ldc, n)))
        rec[f"pdmm{i}_cfg"] = np.array([ord(ta), ord(tb), n, al, be, ldb, ldc])
        rec[f"pdmm{i}_B"], rec[f"pdmm{i}_C0"] = b.copy(order="F"), c.copy(order="F")
        api.gepdmm(ta, tb, m, n, al, a, b.reshape(-1, order="F"), ldb, be,
                   c.reshape(-1, order="F"), ldc)
        rec[f"pdmm{i}_C"] = c
    tree.free_c(a)

    # dplrgeprk on a fresh copy: A += alpha u diag(s) v^T
    k = 3
    u = np.asfortranarray(rng.standard_normal((m, k)))
    v = np.asfortranarray(rng.standard_normal((m, k)))
    s = np.abs(rng.standard_normal(k)) + 0.1
    for i, (al, ep) in enumerate([(0.8, 1e-10), (-1.3, 1e-3)]):
        a = tree.to_c(t)
        api.geprk(m, k, al, u.reshape(-1, order="F"), m, v.reshape(-1, order="F"), m, s, 1, a, ep)
        rec[f"prk{i}_cfg"] = np.array([k, al, ep])
        m2, d2 = tree.flatten(tree.from_c(a))
        rec[f"prk{i}_meta"], rec[f"prk{i}_data"] = m2, d2
        tree.free_c(a)
    rec["prk_u"], rec["prk_v"], rec["prk_s"] = u, v, s

    # dplrgeinv with eps = 0 and eps > 0
    for i, ep in enumerate([0.0, eps_inv]):
        a = tree.to_c(t)
        b = tree.new_empty()
        info = api.geinv(m, a, b, ep)
        rec[f"inv{i}_cfg"] = np.array([ep, info])
        m2, d2 = tree.flatten(tree.from_c(b))
        rec[f"inv{i}_meta"], rec[f"inv{i}_data"] = m2, d2
        tree.free_c(a)
        tree.free_c(b)

    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **rec)
    print(f"{name}: m={m} levels={nlvl} nnz={rec['nz'][0]} -> {os.path.getsize(path)} bytes")


def main() -> None:
    api = reference_api()
    # 1D exponential kernel, compressed by the reference (config-1 family).
    x = gen.sorted_uniform(256, seed=11)
    kern = gen.exp_kernel_1d(x, 0.1, 1e-2)
    record_case(api, "exp256", d2gep(api, kern, 1e-10, 3), 1e-10, seed=1)
    # The reference test driver's matrix (test/testdplr.c:44-53) at m=256.
    i = np.arange(256)
    d = np.abs(i[:, None] - i[None, :]).astype(float)
    inv_dist = np.where(d == 0, 0.0, 1.0 / np.where(d == 0, 1.0, d))
    record_case(api, "invdist256", d2gep(api, inv_dist, 1e-6, 3), 1e-6, seed=2)
    # Seeded random tree: uneven ranks, a rank-0 level, spare capacity.
    rt = gen.random_tree(256, 32, [7, 0, 5], seed=3, capacity_extra=2)
    record_case(api, "rand256", rt, 1e-8, seed=3)


if __name__ == "__main__":
    main()
