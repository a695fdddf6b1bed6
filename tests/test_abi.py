"""The C ABI: libdplr_gb300.so loads and exports every declared symbol,
and the ctypes mirror of DPlrMtx has the C layout.  No GPU needed."""
import ctypes
import os
import re
import subprocess

import pytest

from dplr_gb300 import tree

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in ("dplr.h", "dplr_gb300.h")]


def declared_symbols():
    names = []
    for h in HEADERS:
        text = open(h).read()
        names += re.findall(r"DPLR_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)
    return sorted(set(names))


def built_lib():
    from dplr_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        from dplr_gb300 import build
        build.build()
    return _native.LIB_PATH


def test_headers_declare_the_drop_in_entry_points():
    names = declared_symbols()
    for fn in ("dplrgepmv", "dplrgepdmm", "dplrgeinv", "dplrgeprk", "dplrreduce",
               "dplrini", "dplrclr", "dplrnz", "dplrrnk"):
        assert fn in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(built_lib())
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_struct_layout_matches_c():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "dplr.h"
int main(void){printf("%zu %zu %zu %zu %zu %zu\n", sizeof(DPlrMtx), offsetof(DPlrMtx, size),
  offsetof(DPlrMtx, dlr.rank), offsetof(DPlrMtx, dlr.u), offsetof(DPlrMtx, dlr.sig),
  offsetof(DPlrMtx, dh.sw)); return 0;}
'''
    tmp = os.path.join(ROOT, "_work")
    os.makedirs(tmp, exist_ok=True)
    c = os.path.join(tmp, "layout.c")
    exe = os.path.join(tmp, "layout")
    open(c, "w").write(src)
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
    out = [int(v) for v in subprocess.check_output([exe]).split()]
    D = tree.DPlrMtx
    assert out == [ctypes.sizeof(D), D.size.offset, D.body.offset + tree._LRPart.rank.offset,
                   D.body.offset + tree._LRPart.u.offset, D.body.offset + tree._LRPart.sig.offset,
                   D.body.offset + tree._HPart.sw.offset]


def test_structure_helpers_on_host():
    """dplrini/dplrinilr/dplrresizelr keep DPLR's semantics (no GPU)."""
    from dplr_gb300 import _native
    lib = _native.lib()
    a = tree.new_empty()
    lib.dplrinilr.argtypes = [ctypes.c_int, tree.PDPlrMtx, ctypes.c_int]
    lib.dplrresizelr.argtypes = [tree.PDPlrMtx, ctypes.c_int]
    lib.dplrinilr(8, a, 2)
    c = a.contents
    assert (c.type, c.size, c.dlr.rank, c.dlr.capacity) == (tree.PLR_LRMTX, 8, 0, 2)
    lib.dplrresizelr(a, 3)          # grows to max(3, 2*2) = 4
    assert a.contents.dlr.capacity == 4
    lib.dplrresizelr(a, 1)          # below capacity: no change
    assert a.contents.dlr.capacity == 4
    tree.free_c(a)
