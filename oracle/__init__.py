"""numpy/ctypes front end of the CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg and reference arm, as the checker.  The product
library never imports it.  See oracle.h for what each function restates
(reference file:line) and for the parity status.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

LITERAL_D1 = 1 << 1
LITERAL_D2 = 1 << 2
LITERAL_D3 = 1 << 3
LITERAL_D6 = 1 << 6
LITERAL_D11 = 1 << 11
LITERAL_D16 = 1 << 16

OCTNODE_DTYPE = np.dtype(
    [
        ("children", "<i4", (8,)),
        ("corner", "<f4", (4,)),
        ("cell_size", "<f4"),
        ("child_node_mask", "<i4"),
        ("child_leaf_mask", "<i4"),
        ("_pad", "<i4"),
    ]
)
assert OCTNODE_DTYPE.itemsize == 64


def build(verbose: bool = False) -> str:
    """Compile oracle.cpp into oracle/_build/liboracle.so (g++, no cmake)."""
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if verbose:
        print(out.stdout)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        u32, i32, f32, i_ = ctypes.c_uint32, ctypes.c_int32, ctypes.c_float, ctypes.c_int
        sig = {
            "orc_morton32": (None, [P, u32, f32, f32, P]),
            "orc_morton64": (None, [P, u32, f32, f32, P]),
            "orc_morton32_to_xyz": (None, [P, u32, f32, f32]),
            "orc_morton64_to_xyz": (None, [P, ctypes.c_uint64, f32, f32]),
            "orc_global_hist_u32": (None, [P, u32, i_, P, u32]),
            "orc_global_hist_u64": (None, [P, u32, i_, P]),
            "orc_sort_pairs_u32": (None, [P, P, u32, i_]),
            "orc_sort_pairs_u64": (None, [P, P, u32, i_]),
            "orc_unique_u32": (u32, [P, P, u32]),
            "orc_unique_u64": (u32, [P, P, u32]),
            "orc_radix_tree_u32": (u32, [P, i32, P, P, P, P, P, u32]),
            "orc_radix_tree_u64": (u32, [P, i32, P, P, P, P, P, u32]),
            "orc_edge_count": (None, [P, P, u32, i_, P, u32]),
            "orc_prefix_sum": (u32, [P, u32, P]),
            "orc_octree_u32": (u32, [P, u32, P, P, P, P, P, P, P, f32, f32, P, u32, P, P]),
            "orc_octree_u64": (u32, [P, u32, P, P, P, P, P, P, P, f32, f32, P, u32, P, P]),
            "orc_validate_octree": (i_, [P, u32, u32, f32]),
            "orc_build_octree": (i_, [P, u32, f32, f32, i_, P, P, P, P, P, P, P, P, P, P, P, u32, i_, P]),
            "orc_max_threads": (i_, []),
            "orc_pwl_loss_grad": (ctypes.c_double, [P, u32, P, P, i_, P]),
            "orc_pwl_buckets": (None, [P, u32, P, P, i_, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def key_dtype(key_bits: int):
    return np.uint32 if key_bits == 32 else np.uint64


def unused_bits(key_bits: int) -> int:
    """A = W - 3B: always-zero high bits of a Morton code in its word."""
    return 2 if key_bits == 32 else 1


def max_threads() -> int:
    return int(lib().orc_max_threads())


def morton(pts: np.ndarray, key_bits: int, min_coord: float = 0.0, rng: float = 1024.0) -> np.ndarray:
    pts = np.ascontiguousarray(pts, dtype=np.float32).reshape(-1, 4)
    n = pts.shape[0]
    keys = np.empty(n, dtype=key_dtype(key_bits))
    fn = lib().orc_morton32 if key_bits == 32 else lib().orc_morton64
    fn(_p(pts), n, min_coord, rng, _p(keys))
    return keys


def morton_to_xyz(code: int, key_bits: int, min_coord: float = 0.0, rng: float = 1024.0) -> np.ndarray:
    out = np.empty(4, dtype=np.float32)
    fn = lib().orc_morton32_to_xyz if key_bits == 32 else lib().orc_morton64_to_xyz
    fn(_p(out), int(code), min_coord, rng)
    return out


def global_hist(keys: np.ndarray, passes: int, flags: int = 0) -> np.ndarray:
    keys = np.ascontiguousarray(keys)
    hist = np.zeros(passes * 256, dtype=np.uint32)
    if keys.dtype == np.uint32:
        lib().orc_global_hist_u32(_p(keys), keys.size, passes, _p(hist), flags)
    else:
        lib().orc_global_hist_u64(_p(keys), keys.size, passes, _p(hist))
    return hist.reshape(passes, 256)


def sort_pairs(keys: np.ndarray, vals: np.ndarray, threads: int = 1):
    k = np.array(keys, copy=True)
    v = np.array(vals, dtype=np.uint32, copy=True)
    fn = lib().orc_sort_pairs_u32 if k.dtype == np.uint32 else lib().orc_sort_pairs_u64
    fn(_p(k), _p(v), k.size, threads)
    return k, v


def unique(keys: np.ndarray, vals: np.ndarray | None = None):
    k = np.array(keys, copy=True)
    v = None if vals is None else np.array(vals, dtype=np.uint32, copy=True)
    fn = lib().orc_unique_u32 if k.dtype == np.uint32 else lib().orc_unique_u64
    u = fn(_p(k), None if v is None else _p(v), k.size)
    return k[:u], (None if v is None else v[:u]), int(u)


def radix_tree(codes: np.ndarray, flags: int = 0):
    codes = np.ascontiguousarray(codes)
    m = max(codes.size - 1, 0)
    prefix_n = np.zeros(m, np.uint8)
    hll = np.zeros(m, np.uint8)
    hlr = np.zeros(m, np.uint8)
    left = np.zeros(m, np.int32)
    parent = np.zeros(m, np.int32)
    fn = lib().orc_radix_tree_u32 if codes.dtype == np.uint32 else lib().orc_radix_tree_u64
    multi = fn(_p(codes), m, _p(prefix_n), _p(hll), _p(hlr), _p(left), _p(parent), flags)
    return dict(prefix_n=prefix_n, has_leaf_left=hll, has_leaf_right=hlr, left_child=left, parent=parent,
                multi_parent=int(multi))


def edge_count(prefix_n: np.ndarray, parent: np.ndarray, key_bits: int, flags: int = 0) -> np.ndarray:
    m = prefix_n.size
    edge = np.zeros(m, np.uint32)
    lib().orc_edge_count(_p(prefix_n), _p(parent), m, unused_bits(key_bits), _p(edge), flags)
    return edge


def prefix_sum(edge: np.ndarray, u: int) -> np.ndarray:
    ps = np.zeros(u, np.uint32)
    if u > 0:
        e = np.ascontiguousarray(edge, dtype=np.uint32)
        if e.size == 0:
            e = np.zeros(1, np.uint32)
        lib().orc_prefix_sum(_p(e), u, _p(ps))
    return ps


def octree(codes, tree, edge, ps, min_coord=0.0, rng=1024.0, flags=0):
    u = codes.size
    o = 1 + (int(ps[u - 1]) if u > 1 else 0) if u > 0 else 0
    nodes = np.zeros(max(o, 1), OCTNODE_DTYPE)
    conflicts = ctypes.c_uint32(0)
    caps = ctypes.c_uint32(0)
    fn = lib().orc_octree_u32 if codes.dtype == np.uint32 else lib().orc_octree_u64
    dummy8 = np.zeros(1, np.uint8)
    dummy32 = np.zeros(1, np.int32)
    dummyu = np.zeros(1, np.uint32)

    def nz(a, d):
        return a if a.size else d

    got = fn(_p(codes), u, _p(nz(tree["prefix_n"], dummy8)), _p(nz(tree["has_leaf_left"], dummy8)),
             _p(nz(tree["has_leaf_right"], dummy8)), _p(nz(tree["left_child"], dummy32)),
             _p(nz(tree["parent"], dummy32)), _p(nz(edge, dummyu)), _p(nz(ps, dummyu)), min_coord, rng,
             _p(nodes), flags, ctypes.byref(conflicts), ctypes.byref(caps))
    assert got in (o, 0), (got, o)
    return nodes[:got], int(conflicts.value), int(caps.value)


def validate_octree(nodes: np.ndarray, u: int, rng: float = 1024.0) -> int:
    nodes = np.ascontiguousarray(nodes)
    buf = nodes if nodes.size else np.zeros(1, OCTNODE_DTYPE)
    return int(lib().orc_validate_octree(_p(buf), nodes.size, u, rng))


STAGES = ("morton", "sort", "unique", "radix_tree", "edge_count", "prefix_sum", "octree")


def build_octree(pts: np.ndarray, key_bits: int, min_coord=0.0, rng=1024.0, flags=0, threads=1):
    """Whole path on the CPU.  Returns (outputs dict, stage wall times in ms)."""
    pts = np.ascontiguousarray(pts, dtype=np.float32).reshape(-1, 4)
    n = pts.shape[0]
    nn = max(n, 1)
    keys = np.zeros(nn, key_dtype(key_bits))
    idx = np.zeros(nn, np.uint32)
    prefix_n = np.zeros(nn, np.uint8)
    hll = np.zeros(nn, np.uint8)
    hlr = np.zeros(nn, np.uint8)
    left = np.zeros(nn, np.int32)
    parent = np.zeros(nn, np.int32)
    edge = np.zeros(nn, np.uint32)
    ps = np.zeros(nn, np.uint32)
    nodes = np.zeros(nn + 1, OCTNODE_DTYPE)
    counts = np.zeros(3, np.uint32)
    stage_ms = np.zeros(8, np.float64)
    t0 = time.perf_counter()
    bad = lib().orc_build_octree(_p(pts), n, min_coord, rng, key_bits, _p(keys), _p(idx), _p(prefix_n), _p(hll),
                                 _p(hlr), _p(left), _p(parent), _p(edge), _p(ps), _p(nodes), _p(counts), flags,
                                 threads, _p(stage_ms))
    total_ms = (time.perf_counter() - t0) * 1e3
    u, m, o = (int(c) for c in counts)
    out = dict(keys=keys[:u], idx=idx[:u], prefix_n=prefix_n[:m], has_leaf_left=hll[:m], has_leaf_right=hlr[:m],
               left_child=left[:m], parent=parent[:m], edge_count=edge[:m], node_offsets=ps[:u], nodes=nodes[:o],
               n_unique=u, n_brt_nodes=m, n_oct_nodes=o, conflicts=int(bad))
    times = dict(zip(STAGES, stage_ms[:7].tolist()))
    times["total"] = total_ms
    return out, times


def pwl_loss_grad(sample: np.ndarray, knots: np.ndarray, heights: np.ndarray):
    """Loss and gradient of the learned-bucket CDF model (double precision)."""
    sample = np.ascontiguousarray(sample, dtype=np.uint64)
    knots = np.ascontiguousarray(knots, dtype=np.uint64)
    heights = np.ascontiguousarray(heights, dtype=np.float32)
    B = knots.size - 1
    grad = np.zeros(B + 1, np.float64)
    loss = lib().orc_pwl_loss_grad(_p(sample), sample.size, _p(knots), _p(heights), B, _p(grad))
    return float(loss), grad


def pwl_buckets(keys: np.ndarray, knots: np.ndarray, heights: np.ndarray) -> np.ndarray:
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    knots = np.ascontiguousarray(knots, dtype=np.uint64)
    heights = np.ascontiguousarray(heights, dtype=np.float32)
    out = np.zeros(keys.size, np.uint32)
    lib().orc_pwl_buckets(_p(keys), keys.size, _p(knots), _p(heights), knots.size - 1, _p(out))
    return out
