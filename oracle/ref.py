"""numpy/ctypes front end of oracle/_ref/libref_shaders.so.

TEST INFRASTRUCTURE ONLY.  The library holds the reference's own shader
functions compiled as C++ on the CPU (oracle/ref_shaders.py builds it from a
reference checkout; oracle/ref_glue.cpp runs them).  Tests use it to pin the
oracle (oracle.cpp) stage by stage, and tests/golden/make_golden.py to write
reference-derived fixtures.  Variant names: `lit` applies no deviation patch,
`fix` all of them (the reference-intent contract), `lit_dK` all but DK.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import ref_shaders

_lib = None
OCTNODE_DTYPE = np.dtype([("children", "<i4", (8,)), ("corner", "<f4", (4,)), ("cell_size", "<f4"),
                          ("child_node_mask", "<i4"), ("child_leaf_mask", "<i4"), ("_pad", "<i4")])


def available() -> bool:
    return os.path.exists(ref_shaders.LIB_PATH)


def build(reference_root: str) -> str:
    return ref_shaders.build(reference_root)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("oracle/_ref/libref_shaders.so is not built (python oracle/ref_shaders.py <reference>)")
        L = ctypes.CDLL(ref_shaders.LIB_PATH)
        P, u32, i32, f32, i_ = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_float, ctypes.c_int
        for name in ref_shaders.VARIANTS:
            stage = ref_shaders.VARIANTS[name][0]
            fn = getattr(L, name)
            fn.restype, fn.argtypes = {
                "morton": (None, [P, u32, f32, f32, P]),
                "unique": (u32, [P, u32]),
                "tree": (None, [P, i32, P, P, P, P, P]),
                "edge": (None, [P, P, P, u32, i_]),
                "psum": (None, [P, u32, u32, P]),
                "octree": (None, [P, u32, P, P, P, P, P, P, P, P, f32, f32, i32, i_]),
            }[stage]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def _nz(a: np.ndarray, dtype) -> np.ndarray:
    """A non-empty contiguous buffer (ctypes needs a valid pointer for m = 0)."""
    a = np.ascontiguousarray(a, dtype=dtype)
    return a if a.size else np.zeros(1, dtype)


def _w64(dtype) -> bool:
    return np.dtype(dtype) == np.uint64


def morton32(pts: np.ndarray, min_coord: float = 0.0, rng: float = 1024.0) -> np.ndarray:
    """morton.comp:60-67 over float[n][4]."""
    pts = np.ascontiguousarray(pts, dtype=np.float32).reshape(-1, 4)
    keys = np.zeros(pts.shape[0], np.uint32)
    lib().ref_morton_lit(_p(pts), pts.shape[0], min_coord, rng, _p(keys))
    return keys


def unique(keys: np.ndarray):
    """unique.comp:31-49 in place; returns (the first u keys, u)."""
    k = np.array(keys, copy=True)
    fn = lib().ref_unique_w64 if _w64(k.dtype) else lib().ref_unique_lit
    u = int(fn(_p(k), k.size))
    return k[:u], u


def radix_tree(codes: np.ndarray, variant: str = "fix") -> dict:
    """build_radix_tree.comp over m = u - 1 nodes."""
    codes = np.ascontiguousarray(codes)
    m = max(codes.size - 1, 0)
    out = dict(prefix_n=np.zeros(max(m, 1), np.uint8), has_leaf_left=np.zeros(max(m, 1), np.uint8),
               has_leaf_right=np.zeros(max(m, 1), np.uint8), left_child=np.zeros(max(m, 1), np.int32),
               parent=np.zeros(max(m, 1), np.int32))
    name = f"ref_tree_{'w64_' if _w64(codes.dtype) else ''}{variant}"
    getattr(lib(), name)(_p(codes), m, _p(out["prefix_n"]), _p(out["has_leaf_left"]), _p(out["has_leaf_right"]),
                         _p(out["left_child"]), _p(out["parent"]))
    return {k: v[:m] for k, v in out.items()}


def edge_count(prefix_n: np.ndarray, parent: np.ndarray, key_bits: int, variant: str = "fix") -> np.ndarray:
    """edge_count.comp:30-41 over exactly m nodes."""
    m = prefix_n.size
    edge = np.zeros(max(m, 1), np.uint32)
    getattr(lib(), f"ref_edge_{variant}")(_p(_nz(prefix_n, np.uint8)), _p(_nz(parent, np.int32)), _p(edge), m,
                                          2 if key_bits == 32 else 1)
    return edge[:m]


def partial_sum(data: np.ndarray, first: int, last: int) -> np.ndarray:
    """partial_sum.comp:23-39: inclusive scan of data[first, last)."""
    data = _nz(data.view(np.int32) if data.dtype == np.uint32 else data, np.int32)
    out = np.zeros(max(last - first, 1), np.int32)
    lib().ref_psum_lit(_p(data), first, last, _p(out))
    return out[:last - first].view(np.uint32)


def node_offsets(edge: np.ndarray, u: int) -> np.ndarray:
    """main.rs:127-129: partial_sum(edge, 0, u) with edge[m] past the end (as 0, D4), then ps[0] = 0."""
    data = np.zeros(max(u, 1), np.uint32)
    data[:edge.size] = edge
    ps = partial_sum(data, 0, u)
    if u > 0:
        ps[0] = 0
    return ps


def octree(codes: np.ndarray, tree: dict, edge: np.ndarray, ps: np.ndarray, min_coord: float = 0.0,
           rng: float = 1024.0, variant: str = "fix") -> np.ndarray:
    """Root setup (main.rs:140-153), k_MakeOctNodes, then k_LinkLeafNodes (octree.comp:126-222)."""
    codes = np.ascontiguousarray(codes)
    u = codes.size
    m = max(u - 1, 0)
    o = 1 + (int(ps[u - 1]) if u > 1 else 0)
    nodes = np.zeros(o, OCTNODE_DTYPE)
    w64 = _w64(codes.dtype)
    name = f"ref_octree_{'w64_' if w64 else ''}{variant}"
    getattr(lib(), name)(_p(nodes), o, _p(_nz(ps, np.uint32)), _p(_nz(edge, np.uint32)), _p(codes),
                         _p(_nz(tree["prefix_n"], np.uint8)), _p(_nz(tree["parent"], np.int32)),
                         _p(_nz(tree["left_child"], np.int32)), _p(_nz(tree["has_leaf_left"], np.uint8)),
                         _p(_nz(tree["has_leaf_right"], np.uint8)), min_coord, rng, m, 1 if w64 else 2)
    return nodes


def build_octree(pts: np.ndarray, key_bits: int, min_coord: float = 0.0, rng: float = 1024.0) -> dict:
    """The commented pipeline of main.rs:60-170 through the reference's shaders.

    32-bit codes come from morton.comp; 64-bit codes (not in the reference)
    must be passed in as `pts` already encoded, i.e. pts is then a uint64 key
    array.  The sort is main.rs:85's stable sort by key; the payload (point
    index, kept for the first of each run) is this project's addition and is
    carried by numpy's stable argsort.
    """
    if key_bits == 32:
        keys = morton32(pts, min_coord, rng)
    else:
        keys = np.ascontiguousarray(pts, dtype=np.uint64)
    order = np.argsort(keys, kind="stable").astype(np.uint32)
    skeys = keys[order]
    ukeys, u = unique(skeys)
    first = np.ones(skeys.size, bool)
    first[1:] = skeys[1:] != skeys[:-1]
    idx = order[first][:u]
    tree = radix_tree(ukeys, "fix")
    edge = edge_count(tree["prefix_n"], tree["parent"], key_bits, "fix")
    ps = node_offsets(edge, u)
    nodes = octree(ukeys, tree, edge, ps, min_coord, rng, "fix")
    return dict(keys=ukeys, idx=idx, edge_count=edge, node_offsets=ps, nodes=nodes, n_unique=u,
                n_brt_nodes=max(u - 1, 0), n_oct_nodes=nodes.size, **tree)
