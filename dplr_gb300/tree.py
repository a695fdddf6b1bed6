"""Host-side mirror of DPLR's PLR matrix tree.

``DPlrMtx`` reproduces the C layout of ``include/dplr.h`` (DPLR
include/dplr_internal.h:32-87) for ctypes.  Python-side trees are plain
dataclasses (``Dense``, ``LowRank``, ``HNode``) that can be converted to
malloc-owned C trees (so C code may ``free``/``realloc`` them exactly as
DPLR's own routines do) and back, serialised to flat arrays, expanded to
dense, and measured (``nnz`` restates DPLR src/dplrnz.c:17-62).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Union

import numpy as np

PLR_UMTX, PLR_HMTX, PLR_DMTX, PLR_LRMTX = 0, 1, 2, 3

c_double_p = ctypes.POINTER(ctypes.c_double)


class DPlrMtx(ctypes.Structure):
    pass


class _HPart(ctypes.Structure):
    _fields_ = [("nw", ctypes.POINTER(DPlrMtx)), ("ne", ctypes.POINTER(DPlrMtx)),
                ("se", ctypes.POINTER(DPlrMtx)), ("sw", ctypes.POINTER(DPlrMtx))]


class _DPart(ctypes.Structure):
    _fields_ = [("d", c_double_p)]


class _LRPart(ctypes.Structure):
    _fields_ = [("rank", ctypes.c_int), ("capacity", ctypes.c_int),
                ("u", c_double_p), ("v", c_double_p), ("sig", c_double_p)]


class _Body(ctypes.Union):
    _fields_ = [("dh", _HPart), ("dd", _DPart), ("dlr", _LRPart)]


DPlrMtx._anonymous_ = ("body",)
DPlrMtx._fields_ = [("type", ctypes.c_int), ("size", ctypes.c_int), ("body", _Body)]

PDPlrMtx = ctypes.POINTER(DPlrMtx)

_libc = ctypes.CDLL(None)
_libc.malloc.restype = ctypes.c_void_p
_libc.malloc.argtypes = [ctypes.c_size_t]
_libc.free.restype = None
_libc.free.argtypes = [ctypes.c_void_p]


# --------------------------------------------------------------------------
# Python-side nodes
# --------------------------------------------------------------------------

@dataclass
class Dense:
    d: np.ndarray                      # m x m

    @property
    def size(self) -> int:
        return self.d.shape[0]


@dataclass
class LowRank:
    u: np.ndarray                      # n x rank
    sig: np.ndarray                    # rank
    v: np.ndarray                      # n x rank
    capacity: int | None = None        # >= rank; None means rank

    @property
    def size(self) -> int:
        return self.u.shape[0]

    @property
    def rank(self) -> int:
        return self.u.shape[1]


@dataclass
class HNode:
    nw: "Node"
    ne: LowRank
    se: "Node"
    sw: LowRank

    @property
    def size(self) -> int:
        return self.nw.size + self.se.size


Node = Union[Dense, HNode]


# --------------------------------------------------------------------------
# C conversion (malloc-owned, NaN in unused capacity like dplrinilr)
# --------------------------------------------------------------------------

def _malloc_doubles(count: int, values: np.ndarray | None = None) -> int:
    if count <= 0:
        return 0
    ptr = _libc.malloc(count * 8)
    if not ptr:
        raise MemoryError("malloc failed")
    buf = np.ctypeslib.as_array((ctypes.c_double * count).from_address(ptr))
    buf[:] = np.nan
    if values is not None:
        flat = np.asarray(values, dtype=np.float64).reshape(-1, order="F")
        buf[: flat.size] = flat
    return ptr


def _new_node() -> int:
    ptr = _libc.malloc(ctypes.sizeof(DPlrMtx))
    if not ptr:
        raise MemoryError("malloc failed")
    ctypes.memset(ptr, 0, ctypes.sizeof(DPlrMtx))
    return ptr


def _fill(ptr: int, node) -> None:
    c = DPlrMtx.from_address(ptr)
    if isinstance(node, Dense):
        m = node.size
        c.type, c.size = PLR_DMTX, m
        c.dd.d = ctypes.cast(_malloc_doubles(m * m, node.d), c_double_p)
    elif isinstance(node, LowRank):
        n, r = node.size, node.rank
        cap = r if node.capacity is None else max(node.capacity, r)
        c.type, c.size = PLR_LRMTX, n
        c.dlr.rank, c.dlr.capacity = r, cap
        c.dlr.u = ctypes.cast(_malloc_doubles(n * cap, node.u), c_double_p)
        c.dlr.v = ctypes.cast(_malloc_doubles(n * cap, node.v), c_double_p)
        c.dlr.sig = ctypes.cast(_malloc_doubles(cap, node.sig), c_double_p)
    elif isinstance(node, HNode):
        c.type, c.size = PLR_HMTX, node.size
        kids = []
        for child in (node.nw, node.ne, node.se, node.sw):
            kp = _new_node()
            _fill(kp, child)
            kids.append(ctypes.cast(kp, PDPlrMtx))
        c.dh.nw, c.dh.ne, c.dh.se, c.dh.sw = kids
    else:
        raise TypeError(f"unknown node {type(node)}")


def to_c(node: Node) -> PDPlrMtx:
    """Allocate a C tree (all buffers and structs from malloc)."""
    ptr = _new_node()
    _fill(ptr, node)
    return ctypes.cast(ptr, PDPlrMtx)


def new_empty() -> PDPlrMtx:
    """A malloc'd node in the dplrini state (type PLR_UMTX)."""
    return ctypes.cast(_new_node(), PDPlrMtx)


def _as_array(p, count: int) -> np.ndarray:
    if count == 0:
        return np.zeros(0)
    return np.ctypeslib.as_array(p, shape=(count,)).copy()


def from_c(p: PDPlrMtx) -> Node | LowRank:
    """Copy a C tree into Python nodes (live columns only)."""
    c = p.contents
    if c.type == PLR_DMTX:
        m = c.size
        return Dense(_as_array(c.dd.d, m * m).reshape(m, m, order="F"))
    if c.type == PLR_LRMTX:
        n, r = c.size, c.dlr.rank
        u = _as_array(c.dlr.u, n * r).reshape(n, r, order="F")
        v = _as_array(c.dlr.v, n * r).reshape(n, r, order="F")
        return LowRank(u, _as_array(c.dlr.sig, r), v, capacity=c.dlr.capacity)
    if c.type == PLR_HMTX:
        return HNode(from_c(c.dh.nw), from_c(c.dh.ne), from_c(c.dh.se), from_c(c.dh.sw))
    raise ValueError(f"node of type {c.type} cannot be read")


def free_c(p: PDPlrMtx) -> None:
    """Free buffers, child structs and the root struct of a C tree."""
    if not p:
        return
    addr = ctypes.cast(p, ctypes.c_void_p).value
    c = p.contents
    if c.type == PLR_DMTX:
        _libc.free(ctypes.cast(c.dd.d, ctypes.c_void_p))
    elif c.type == PLR_LRMTX:
        for q in (c.dlr.u, c.dlr.v, c.dlr.sig):
            _libc.free(ctypes.cast(q, ctypes.c_void_p))
    elif c.type == PLR_HMTX:
        for q in (c.dh.nw, c.dh.ne, c.dh.se, c.dh.sw):
            free_c(q)
    _libc.free(addr)


# --------------------------------------------------------------------------
# utilities on Python trees
# --------------------------------------------------------------------------

def to_dense(node: Node) -> np.ndarray:
    """Expand to a dense matrix (the meaning of DPLR src/dplrp2d.c:98)."""
    if isinstance(node, Dense):
        return node.d.copy()
    h = node.nw.size
    out = np.empty((node.size, node.size))
    out[:h, :h] = to_dense(node.nw)
    out[h:, h:] = to_dense(node.se)
    out[:h, h:] = (node.ne.u * node.ne.sig) @ node.ne.v.T
    out[h:, :h] = (node.sw.u * node.sw.sig) @ node.sw.v.T
    return out


def nnz(node: Node) -> int:
    """Stored entries, restating DPLR src/dplrnz.c:17-62."""
    if isinstance(node, Dense):
        return node.size * node.size
    return node.size * (node.ne.rank + node.sw.rank) + nnz(node.nw) + nnz(node.se)


def ranks_by_level(node: Node, out: list | None = None, level: int = 0) -> list:
    """Maximum off-diagonal rank per level (the meaning of src/dplrrnk.c:22)."""
    if out is None:
        out = []
    if isinstance(node, HNode):
        while len(out) <= level:
            out.append(0)
        out[level] = max(out[level], node.ne.rank, node.sw.rank)
        ranks_by_level(node.nw, out, level + 1)
        ranks_by_level(node.se, out, level + 1)
    return out


def depth(node: Node) -> int:
    return 0 if isinstance(node, Dense) else 1 + max(depth(node.nw), depth(node.se))


# --------------------------------------------------------------------------
# flat serialisation (pre-order nw, ne, se, sw)
# --------------------------------------------------------------------------

def flatten(node) -> tuple[np.ndarray, np.ndarray]:
    """(meta int64[n,4] = type,size,rank,capacity ; data float64) in pre-order."""
    meta, chunks = [], []

    def walk(nd):
        if isinstance(nd, Dense):
            meta.append((PLR_DMTX, nd.size, 0, 0))
            chunks.append(nd.d.reshape(-1, order="F"))
        elif isinstance(nd, LowRank):
            cap = nd.rank if nd.capacity is None else nd.capacity
            meta.append((PLR_LRMTX, nd.size, nd.rank, cap))
            chunks.extend([nd.u.reshape(-1, order="F"), nd.v.reshape(-1, order="F"), nd.sig])
        else:
            meta.append((PLR_HMTX, nd.size, 0, 0))
            for ch in (nd.nw, nd.ne, nd.se, nd.sw):
                walk(ch)

    walk(node)
    data = np.concatenate(chunks) if chunks else np.zeros(0)
    return np.asarray(meta, dtype=np.int64), data


def unflatten(meta: np.ndarray, data: np.ndarray):
    pos = {"i": 0, "o": 0}

    def take(count):
        o = pos["o"]
        pos["o"] += count
        return data[o:o + count]

    def walk():
        t, m, r, cap = (int(x) for x in meta[pos["i"]])
        pos["i"] += 1
        if t == PLR_DMTX:
            return Dense(take(m * m).reshape(m, m, order="F").copy())
        if t == PLR_LRMTX:
            u = take(m * r).reshape(m, r, order="F").copy()
            v = take(m * r).reshape(m, r, order="F").copy()
            return LowRank(u, take(r).copy(), v, capacity=cap)
        nw, ne, se, sw = walk(), walk(), walk(), walk()
        return HNode(nw, ne, se, sw)

    return walk()


def trees_close(a, b, rtol: float, atol: float = 0.0) -> bool:
    """Same structure, ranks and factors within tolerance (NaN-free)."""
    if type(a) is not type(b):
        return False
    if isinstance(a, Dense):
        return a.d.shape == b.d.shape and np.allclose(a.d, b.d, rtol=rtol, atol=atol)
    if isinstance(a, LowRank):
        return (a.u.shape == b.u.shape and np.allclose(a.u, b.u, rtol=rtol, atol=atol)
                and np.allclose(a.v, b.v, rtol=rtol, atol=atol)
                and np.allclose(a.sig, b.sig, rtol=rtol, atol=atol))
    return all(trees_close(x, y, rtol, atol) for x, y in
               ((a.nw, b.nw), (a.ne, b.ne), (a.se, b.se), (a.sw, b.sw)))
