"""Generate tests/golden/ppmm/*.npz: dplrgeppmm outputs of the reference.

Runs the reference's own dplrgeppmm (src/dplrppmm.c:998), built into
oracle/_ref/libdplr_ref.so by oracle/build_oracle.py --ref, on seeded
trees of one structure (m = 128, three levels, leaves of 16): every
(transa, transb) with several (alpha, beta, eps), including alpha = 0,
beta = 0, negative scalars, rank-0 levels and a threshold large enough
to zero columns (the kernel trees: the first two scalar sets).  Each case stores C after the call (live columns, ranks
and capacities).  Re-run with ``python tests/golden/make_golden_ppmm.py``
(needs the reference tree).
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from dplr_gb300 import gen, tree  # noqa: E402
from dplr_gb300.tree import PDPlrMtx  # noqa: E402

OUT = os.path.join(HERE, "ppmm")
SCALARS = [(1.5, 0.5, 1e-10), (-0.75, -1.25, 1e-6), (1.0, 0.0, 1e-12), (0.0, 2.0, 1e-8),
           (0.5, 1.0, 1e3)]
OPS = [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")]


def trees(name: str):
    """(A, B, C) of one structure."""
    if name == "rand":
        a = gen.random_tree(128, 16, [6, 3, 0], seed=21, capacity_extra=1, diag_shift=4.0)
        b = gen.random_tree(128, 16, [4, 5, 2], seed=22, diag_shift=4.0)
        c = gen.random_tree(128, 16, [3, 0, 4], seed=23, capacity_extra=3, diag_shift=4.0)
        return a, b, c
    # compressed kernels (1D exponential, 1/|i-j|), C random
    x = gen.sorted_uniform(128, seed=12)
    a = gen.compress_dense(gen.exp_kernel_1d(x, 0.1, 1e-2), 1e-10, 3)
    i = np.arange(128)
    d = np.abs(i[:, None] - i[None, :]).astype(float)
    b = gen.compress_dense(np.where(d == 0, 0.0, 1.0 / np.where(d == 0, 1.0, d)), 1e-6, 3)
    c = gen.random_tree(128, 16, [2, 2, 2], seed=24, diag_shift=4.0)
    return a, b, c


def main() -> None:
    sys.path.insert(0, os.path.dirname(HERE))
    from oracle import build_oracle, pyoracle
    build_oracle.build_reference()
    api = pyoracle.reference()
    if api is None:
        raise SystemExit("reference library unavailable (needs the reference sources)")
    f = api.lib.dplrgeppmm
    f.restype = None
    f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                  PDPlrMtx, PDPlrMtx, ctypes.POINTER(ctypes.c_double), PDPlrMtx, ctypes.c_double]
    os.makedirs(OUT, exist_ok=True)
    for name in ("rand", "kern"):
        a, b, c = trees(name)
        rec = {}
        for key, t in (("A", a), ("B", b), ("C", c)):
            rec[f"{key}_meta"], rec[f"{key}_data"] = tree.flatten(t)
        ca, cb = tree.to_c(a), tree.to_c(b)
        for i, (ta, tb) in enumerate(OPS):
            for j, (al, be, ep) in enumerate(SCALARS):
                if name == "kern" and j > 1:
                    continue
                cc = tree.to_c(c)
                f(ta.encode(), tb.encode(), 128, ctypes.c_double(al), ca, cb, ctypes.c_double(be), cc, ep)
                rec[f"case{i}_{j}_cfg"] = np.array([ord(ta), ord(tb), al, be, ep])
                rec[f"case{i}_{j}_meta"], rec[f"case{i}_{j}_data"] = tree.flatten(tree.from_c(cc))
                tree.free_c(cc)
        tree.free_c(ca)
        tree.free_c(cb)
        path = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(path, **rec)
        print(f"{name}: {sum(k.endswith('_cfg') for k in rec)} cases -> {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
