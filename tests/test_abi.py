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


_LAYOUT_PROBE = r'''
#include <stdio.h>
#include <stddef.h>
#include "dplr.h"
int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(DPlrMtx),
  offsetof(DPlrMtx, type), offsetof(DPlrMtx, size), offsetof(DPlrMtx, dh.nw),
  offsetof(DPlrMtx, dh.ne), offsetof(DPlrMtx, dh.se), offsetof(DPlrMtx, dh.sw),
  offsetof(DPlrMtx, dd.d), offsetof(DPlrMtx, dlr.rank), offsetof(DPlrMtx, dlr.capacity),
  offsetof(DPlrMtx, dlr.u), offsetof(DPlrMtx, dlr.sig)); return 0;}
'''


def _layout(include_dir: str, tmp_path) -> list[int]:
    """sizeof/offsetof of DPlrMtx as a C compiler lays it out with the
    dplr.h found in include_dir."""
    c = tmp_path / "layout.c"
    exe = tmp_path / f"layout_{abs(hash(include_dir))}"
    c.write_text(_LAYOUT_PROBE)
    subprocess.check_call(["gcc", "-w", "-I", include_dir, str(c), "-o", str(exe)])
    return [int(v) for v in subprocess.check_output([str(exe)]).split()]


def test_struct_layout_matches_c(tmp_path):
    """The ctypes mirror has the layout of this repository's dplr.h."""
    out = _layout(os.path.join(ROOT, "include"), tmp_path)
    D, H, L = tree.DPlrMtx, tree._HPart, tree._LRPart
    b = D.body.offset
    assert out[0] == ctypes.sizeof(D)
    assert out[2] == D.size.offset
    assert out[3:7] == [b + H.nw.offset, b + H.ne.offset, b + H.se.offset, b + H.sw.offset]
    assert out[8:12] == [b + L.rank.offset, b + L.capacity.offset, b + L.u.offset, b + L.sig.offset]


def test_struct_layout_matches_the_reference_header(tmp_path):
    """dplr.h here and the reference's include/dplr.h (which pulls in
    include/dplr_internal.h:32-87) give DPlrMtx the same size and the same
    offsets for every member, so trees pass between the two unchanged."""
    from oracle.build_oracle import REFERENCE_ROOT
    ref_inc = os.path.join(REFERENCE_ROOT, "include")
    if not os.path.exists(os.path.join(ref_inc, "dplr_internal.h")):
        pytest.skip("reference headers not present on this machine")
    assert _layout(os.path.join(ROOT, "include"), tmp_path) == _layout(ref_inc, tmp_path)


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
