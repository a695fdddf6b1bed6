"""Build recipe for the CPU oracle (test infrastructure only).

Two artefacts:

* ``oracle/_build/liboracle.so`` and ``oracle/_build/liboracle_loops.so``:
  the C restatement in ``dplr_oracle.c``, linked against scipy's bundled
  LP64 OpenBLAS when one is found (``liboracle.so``) and against the
  plain-loop BLAS in ``oblas_naive.c`` (``liboracle_loops.so``, always).
* ``oracle/_ref/libdplr_ref.so``: the reference's own C sources compiled
  where they lie (no copy), with every Fortran BLAS/LAPACK symbol renamed
  to scipy's ``scipy_``-prefixed export.  ``src/dplrreduce.c`` is left out
  because it needs the Fortran ``dortlr``/``ortlrini`` objects and no
  Fortran compiler is available.  Only built where the reference tree is
  present.

Run ``python oracle/build_oracle.py [--ref]``.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# The reference checkout: $DPLR_REFERENCE_ROOT, else a directory named
# "reference" beside the repository.  It exists only where the fixtures are
# made; the GPU machine has none and builds only the restatement.
REFERENCE_ROOT = os.environ.get(
    "DPLR_REFERENCE_ROOT",
    os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))

# Fortran BLAS/LAPACK symbols declared by the reference's lapackapi_netlib.h.
_RENAMED = ["dscal_", "dcopy_", "dnrm2_", "ddot_", "daxpy_", "dgemv_", "dgemm_",
            "dgesvd_", "dger_", "dgetri_", "dgetrf_"]
# Reference sources that compile without Fortran (all but dplrreduce.c).
_REF_SOURCES = ["dplrini.c", "dplrd2p.c", "dplrresizelr.c", "dplrp2d.c", "dplrscal.c",
                "dplrcpy.c", "dplraxpy.c", "dplrrnk.c", "dplrpmv.c", "dplrpdmm.c",
                "dplrprk.c", "dplrppmm.c", "dplrinv.c", "dplrnz.c", "dplrempty.c"]


def find_scipy_openblas() -> str | None:
    """Path of scipy's bundled OpenBLAS shared library, or None."""
    try:
        import scipy  # noqa: F401
    except Exception:
        return None
    site = os.path.dirname(os.path.dirname(os.path.abspath(sys.modules["scipy"].__file__)))
    hits = sorted(glob.glob(os.path.join(site, "scipy.libs", "libscipy_openblas*.so*")))
    return hits[0] if hits else None


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + res.stderr)


def _link_flags(lib: str) -> list[str]:
    return [lib, "-Wl,-rpath," + os.path.dirname(lib), "-lm"]


def build_oracle(verbose: bool = False) -> dict:
    """Compile the oracle libraries; returns their paths."""
    os.makedirs(BUILD, exist_ok=True)
    # no contraction of a*b+c into fma: the double-double checker relies
    # on exact TwoSum steps, and the restatement on the reference's rounding
    cflags = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-Wall", "-ffp-contract=off", "-pthread"]
    src = [os.path.join(HERE, f) for f in ("dplr_oracle.c", "dd_resid.c", "shape.c")]
    out = {}
    loops = os.path.join(BUILD, "liboracle_loops.so")
    _run(cflags + src + [os.path.join(HERE, "oblas_naive.c"), "-o", loops, "-lm"])
    out["loops"] = loops
    lib = find_scipy_openblas()
    if lib is not None:
        blas = os.path.join(BUILD, "liboracle.so")
        _run(cflags + src + [os.path.join(HERE, "oblas_scipy.c"), "-o", blas] + _link_flags(lib))
        out["blas"] = blas
    if verbose:
        print("oracle:", out)
    return out


def build_reference(verbose: bool = False) -> str | None:
    """Compile the reference C sources in place into oracle/_ref (here only)."""
    src_dir = os.path.join(REFERENCE_ROOT, "src")
    lib = find_scipy_openblas()
    if not os.path.isdir(src_dir) or lib is None:
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    out = os.path.join(REF_OUT, "libdplr_ref.so")
    renames = [f"-D{s}=scipy_{s}" for s in _RENAMED]
    srcs = [os.path.join(src_dir, s) for s in _REF_SOURCES]
    _run(["gcc", "-O2", "-fPIC", "-shared", "-w"] + renames + srcs + ["-o", out] + _link_flags(lib))
    if verbose:
        print("reference:", out)
    return out


if __name__ == "__main__":
    build_oracle(verbose=True)
    if "--ref" in sys.argv:
        build_reference(verbose=True)
