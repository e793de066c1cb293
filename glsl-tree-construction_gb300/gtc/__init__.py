"""Python driver of the GB300-native octree-construction library (libgtc.so).

Thin ctypes layer over the C ABI in include/gtc.h.  Device buffers are torch
CUDA tensors (plumbing only: allocation and streams); every computation runs
in libgtc.so's CUDA kernels.  Operators mirror the reference's stage functions
(radixsort-vulkan/src/*.rs): compute_morton, histogram, radix_sort, unique,
build_radix_tree, edge_count, partial_sum, build_octree.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _build, _lib
from ._lib import OctreeBuffers

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "TIMEOUT", 5: "OVERFLOW_FALLBACK",
          6: "UNSUPPORTED", 7: "CAPACITY"}
OP_SORT_PAIRS, OP_UNIQUE, OP_PARTIAL_SUM, OP_BUILD_OCTREE, OP_GLOBAL_HISTOGRAM = 1, 2, 3, 4, 5
STAGES = ("morton", "histogram", "onesweep", "unique", "radix_tree", "prefix_sum", "octree", "learned", "run_fixup")

OCTNODE_DTYPE = np.dtype([("children", "<i4", (8,)), ("corner", "<f4", (4,)), ("cell_size", "<f4"),
                          ("child_node_mask", "<i4"), ("child_leaf_mask", "<i4"), ("_pad", "<i4")])


class GtcError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"gtc status {status} ({STATUS.get(status, '?')}): {msg}")


def build(**kw) -> str:
    return _build.build(**kw)


def lib():
    return _lib.load()


def _torch():
    import torch

    return torch


def _ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


def _stream(stream=None) -> int:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


class Context:
    """A libgtc context bound to one CUDA device (gtc_create / gtc_destroy)."""

    def __init__(self, device: int = 0):
        self.L = lib()
        h = ctypes.c_void_p()
        s = self.L.gtc_create(ctypes.byref(h), device)
        if s != 0:
            raise GtcError(s, "gtc_create failed (no CUDA device?)")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.L.gtc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- status ------------------------------------------------------------
    def check(self, status: int):
        if status != 0:
            raise GtcError(status, (self.L.gtc_last_error(self.h) or b"").decode())

    def device_status(self, stream=None) -> int:
        """Synchronise and return (and clear) the device status; raises on error."""
        s = self.L.gtc_device_status(self.h, _stream(stream))
        self.check(s)
        return s

    def device_status_code(self, stream=None) -> int:
        return self.L.gtc_device_status(self.h, _stream(stream))

    def set_spin_limit(self, polls: int):
        """Poll budget of this context's bounded device waits (0: the default)."""
        self.check(self.L.gtc_set_spin_limit(self.h, polls))

    def debug_skip_first_tile(self):
        """The next sort_pairs hands out tile tickets from 1 (tile 0 never
        publishes; its look-backs time out).  For tests of the timeout path."""
        self.check(self.L.gtc_debug_skip_first_tile(self.h))

    def set_profiling(self, on: bool):
        self.check(self.L.gtc_set_profiling(self.h, 1 if on else 0))

    def stage_times(self, reset: bool = True) -> dict:
        ms = (ctypes.c_float * len(STAGES))()
        n = (ctypes.c_uint32 * len(STAGES))()
        self.check(self.L.gtc_stage_times(self.h, ms, n, 1 if reset else 0))
        return {STAGES[i]: (ms[i], n[i]) for i in range(len(STAGES))}

    def workspace_size(self, op: int, n: int, key_bits: int) -> int:
        b = ctypes.c_size_t()
        self.check(self.L.gtc_workspace_size(self.h, op, n, key_bits, ctypes.byref(b)))
        return b.value

    def workspace(self, op: int, n: int, key_bits: int):
        torch = _torch()
        nbytes = self.workspace_size(op, n, key_bits)
        return torch.empty(max(nbytes, 256), dtype=torch.uint8, device=f"cuda:{self.device}")

    # -- stage operators (device tensors, current torch stream) ------------
    def morton(self, pts, key_bits: int, min_coord: float = 0.0, rng: float = 1024.0, with_idx: bool = True):
        torch = _torch()
        n = pts.shape[0]
        kd = torch.int32 if key_bits == 32 else torch.int64
        keys = torch.empty(n, dtype=kd, device=pts.device)
        idx = torch.empty(n, dtype=torch.int32, device=pts.device) if with_idx else None
        fn = self.L.gtc_morton32 if key_bits == 32 else self.L.gtc_morton64
        self.check(fn(self.h, _ptr(pts), _ptr(keys), _ptr(idx), n, min_coord, rng, _stream()))
        return keys, idx

    def global_histogram(self, keys, begin_bit: int, end_bit: int, ws=None):
        torch = _torch()
        passes = (end_bit - begin_bit + 7) // 8
        hist = torch.empty(passes * 256, dtype=torch.int32, device=keys.device)
        fn = self.L.gtc_global_histogram_u32 if keys.element_size() == 4 else self.L.gtc_global_histogram_u64
        self.check(fn(self.h, _ptr(keys), keys.numel(), begin_bit, end_bit, _ptr(hist), _ptr(ws),
                      0 if ws is None else ws.numel(), _stream()))
        return hist.view(passes, 256)

    def sort_pairs(self, keys, vals=None, begin_bit: int = 0, end_bit: int | None = None, ws=None,
                   keys_alt=None, vals_alt=None):
        """Stable onesweep sort in place (result in keys / vals)."""
        torch = _torch()
        n = keys.numel()
        end_bit = keys.element_size() * 8 if end_bit is None else end_bit
        keys_alt = torch.empty_like(keys) if keys_alt is None else keys_alt
        if vals is not None and vals_alt is None:
            vals_alt = torch.empty_like(vals)
        fn = self.L.gtc_sort_pairs_u32 if keys.element_size() == 4 else self.L.gtc_sort_pairs_u64
        self.check(fn(self.h, _ptr(keys), _ptr(vals), _ptr(keys_alt), _ptr(vals_alt), n, begin_bit, end_bit,
                      _ptr(ws), 0 if ws is None else ws.numel(), _stream()))
        return keys, vals

    def unique(self, keys, vals=None, ws=None):
        """In-place unique; returns the device count tensor (1 element)."""
        torch = _torch()
        cnt = torch.zeros(1, dtype=torch.int32, device=keys.device)
        fn = self.L.gtc_unique_u32 if keys.element_size() == 4 else self.L.gtc_unique_u64
        self.check(fn(self.h, _ptr(keys), _ptr(vals), keys.numel(), _ptr(cnt), _ptr(ws),
                      0 if ws is None else ws.numel(), _stream()))
        return cnt

    def radix_tree(self, codes, n_brt_nodes: int, with_edge: bool = False):
        torch = _torch()
        m = n_brt_nodes
        dev = codes.device
        out = dict(prefix_n=torch.zeros(max(m, 1), dtype=torch.uint8, device=dev),
                   has_leaf_left=torch.zeros(max(m, 1), dtype=torch.uint8, device=dev),
                   has_leaf_right=torch.zeros(max(m, 1), dtype=torch.uint8, device=dev),
                   left_child=torch.zeros(max(m, 1), dtype=torch.int32, device=dev),
                   parent=torch.zeros(max(m, 1), dtype=torch.int32, device=dev))
        if with_edge:
            out["edge_count"] = torch.zeros(max(m, 1), dtype=torch.int32, device=dev)
        fn = self.L.gtc_build_radix_tree_u32 if codes.element_size() == 4 else self.L.gtc_build_radix_tree_u64
        self.check(fn(self.h, _ptr(codes), m, _ptr(out["prefix_n"]), _ptr(out["has_leaf_left"]),
                      _ptr(out["has_leaf_right"]), _ptr(out["left_child"]), _ptr(out["parent"]),
                      _ptr(out.get("edge_count")), _stream()))
        return {k: v[:m] for k, v in out.items()}

    def edge_count(self, prefix_n, parent, key_bits: int):
        torch = _torch()
        m = prefix_n.numel()
        edge = torch.zeros(max(m, 1), dtype=torch.int32, device=prefix_n.device)
        self.check(self.L.gtc_edge_count(self.h, _ptr(prefix_n), _ptr(parent), _ptr(edge), m, key_bits, _stream()))
        return edge[:m]

    def partial_sum(self, data, first: int, last: int, ws=None):
        torch = _torch()
        out = torch.zeros(max(last - first, 1), dtype=torch.int32, device=data.device)
        self.check(self.L.gtc_partial_sum_u32(self.h, _ptr(data), first, last, _ptr(out), _ptr(ws),
                                              0 if ws is None else ws.numel(), _stream()))
        return out[: last - first]

    def node_offsets(self, edge, n_brt_nodes: int, ws=None):
        torch = _torch()
        ps = torch.zeros(n_brt_nodes + 1, dtype=torch.int32, device=edge.device)
        o = torch.zeros(1, dtype=torch.int32, device=edge.device)
        self.check(self.L.gtc_node_offsets(self.h, _ptr(edge), n_brt_nodes, _ptr(ps), _ptr(o), _ptr(ws),
                                           0 if ws is None else ws.numel(), _stream()))
        return ps, o

    def make_octree(self, codes, tree, edge, ps, n_oct: int, min_coord=0.0, rng=1024.0, link=True):
        torch = _torch()
        m = tree["prefix_n"].numel()
        nodes = torch.zeros((max(n_oct, 1), 16), dtype=torch.int32, device=codes.device)
        k64 = codes.element_size() == 8
        mk = self.L.gtc_make_octree_u64 if k64 else self.L.gtc_make_octree_u32
        self.check(mk(self.h, _ptr(nodes), max(n_oct, 1), _ptr(ps), _ptr(edge), _ptr(codes), _ptr(tree["prefix_n"]),
                      _ptr(tree["parent"]), min_coord, rng, m, _ptr(tree["has_leaf_left"]),
                      _ptr(tree["has_leaf_right"]), _ptr(tree["left_child"]), _stream()))
        if link:
            lk = self.L.gtc_link_octree_u64 if k64 else self.L.gtc_link_octree_u32
            self.check(lk(self.h, _ptr(nodes), max(n_oct, 1), _ptr(ps), _ptr(edge), _ptr(codes),
                          _ptr(tree["prefix_n"]), _ptr(tree["parent"]), m, _ptr(tree["has_leaf_left"]),
                          _ptr(tree["has_leaf_right"]), _ptr(tree["left_child"]), _stream()))
        return nodes[:n_oct]

    # -- sort variant table (autotuner) ------------------------------------
    def gather_points(self, pts, idx, count: int | None = None):
        """Points in payload order: out[i] = pts[idx[i]] (float4 [count, 4])."""
        torch = _torch()
        count = idx.numel() if count is None else count
        out = torch.empty((count, 4), dtype=torch.float32, device=pts.device)
        self.check(self.L.gtc_gather_points(self.h, _ptr(pts), pts.shape[0], _ptr(idx), count, _ptr(out),
                                            _stream()))
        return out

    def sort_variants(self):
        out = []
        for v in range(self.L.gtc_sort_num_variants()):
            t, k = ctypes.c_int(), ctypes.c_int()
            self.check(self.L.gtc_sort_variant_shape(v, ctypes.byref(t), ctypes.byref(k)))
            out.append((t.value, k.value))
        return out

    def set_sort_digit_bits(self, key_bits: int, db: int):
        """Pin the sort's digit width (6..8 bits; -1 unpins)."""
        self.check(self.L.gtc_sort_set_digit_bits(key_bits, db))

    def get_sort_digit_bits(self, key_bits: int, bits: int, n: int) -> int:
        return self.L.gtc_sort_get_digit_bits(key_bits, bits, n)

    def set_sort_variant(self, key_bits: int, v: int):
        self.check(self.L.gtc_sort_set_variant(key_bits, v))

    def get_sort_variant(self, key_bits: int) -> int:
        return int(self.L.gtc_sort_get_variant(key_bits))

    def autotune_sort(self, key_bits: int, n: int, begin_bit: int = 0, end_bit: int | None = None, keys=None,
                      reps: int = 3) -> dict:
        """Time every onesweep variant on n keys (the given device keys, or
        seeded uniform ones) and cache the fastest for this shape.  Returns
        {"best": variant, "ms": [per-variant best time]}."""
        end_bit = key_bits if end_bit is None else end_bit
        nv = self.L.gtc_sort_num_variants()
        times = (ctypes.c_float * nv)()
        dtimes = (ctypes.c_float * 3)()
        best = ctypes.c_int(-1)
        bdb = ctypes.c_int(-1)
        self.check(self.L.gtc_autotune_sort_ex(self.h, key_bits, begin_bit, end_bit, n, _ptr(keys), reps,
                                               ctypes.byref(best), times, ctypes.byref(bdb), dtimes))
        big = 3.0e38  # widths that do not fit the bit range report FLT_MAX
        return {"best": best.value, "ms": [float(t) for t in times], "digit_bits": bdb.value,
                "digit_ms": {6 + i: (float(dtimes[i]) if dtimes[i] < big else None) for i in range(3)}}


def autotune_lookup(key_bits: int, bits: int, n: int) -> int:
    """The autotuned onesweep variant for a sort of that shape, or -1."""
    return int(lib().gtc_autotune_lookup(key_bits, bits, n))


def autotune_lookup_digit_bits(key_bits: int, bits: int, n: int) -> int:
    return lib().gtc_autotune_lookup_digit_bits(key_bits, bits, n)


def autotune_save(path: str):
    if lib().gtc_autotune_save(path.encode()) != 0:
        raise GtcError(1, f"cannot write {path}")


def autotune_load(path: str):
    if lib().gtc_autotune_load(path.encode()) != 0:
        raise GtcError(1, f"cannot read {path}")


def autotune_clear():
    lib().gtc_autotune_clear()


LITERAL_D2 = 1 << 2  # gtc_edge_count: depth = prefix_n / 3 (edge_count.comp:34)
LITERAL_D6 = 1 << 6  # leaf links leave child_leaf_mask at 0 (octree.comp:27-30)


def set_literal(flags: int):
    """Process-wide literal-mode switches (LITERAL_D2 | LITERAL_D6; 0 = the
    corrected forms)."""
    st = lib().gtc_set_literal(flags)
    if st != 0:
        raise GtcError(st, f"unknown literal flags {flags:#x}")


def get_literal() -> int:
    return int(lib().gtc_get_literal())


def export_le(path: str, data, append: bool = False):
    """Write a host or device array to `path` as little-endian elements of its
    own width (the reference's write_u32::<LittleEndian> dump)."""
    a = data.cpu().numpy() if hasattr(data, "cpu") else np.asarray(data)
    a = np.ascontiguousarray(a)
    width = a.dtype.itemsize
    st = lib().gtc_export_le(path.encode(), a.ctypes.data if a.size else None, a.size, width, int(append))
    if st != 0:
        raise GtcError(st, f"cannot write {path}")


STAGE_BUFFERS = ("keys", "idx", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent", "edge_count",
                 "node_offsets", "nodes")


def export_build(res, directory: str) -> dict:
    """Every stage buffer of a build as `<name>.bin` (little-endian words of
    each buffer's element width; nodes as 16 32-bit words per node), cut to
    the live lengths (u keys and payloads, m tree entries, u node offsets, o
    nodes).  Returns {name: path}."""
    import os

    os.makedirs(directory, exist_ok=True)
    u, m, o = res.n_unique, res.n_brt_nodes, res.n_oct_nodes
    live = {"keys": u, "idx": u, "prefix_n": m, "has_leaf_left": m, "has_leaf_right": m, "left_child": m,
            "parent": m, "edge_count": m, "node_offsets": u, "nodes": o}
    out = {}
    for name in STAGE_BUFFERS:
        t = getattr(res, name)
        a = t.cpu().numpy() if hasattr(t, "cpu") else np.asarray(t)
        a = a.reshape(-1, 16)[: live[name]] if name == "nodes" else a.reshape(-1)[: live[name]]
        path = os.path.join(directory, name + ".bin")
        export_le(path, a)
        out[name] = path
    return out


@dataclass
class OctreeResult:
    keys: object
    idx: object
    prefix_n: object
    has_leaf_left: object
    has_leaf_right: object
    left_child: object
    parent: object
    edge_count: object
    node_offsets: object
    nodes: object  # int32 [o, 16] view of gtc_octnode
    n_unique: int
    n_brt_nodes: int
    n_oct_nodes: int


class OctreePlan:
    """Resident buffers for repeated builds of up to n_max points: the fused
    stream-ordered pipeline (gtc_build_octree) with no allocation per call,
    optionally captured once into a CUDA graph and replayed."""

    def __init__(self, ctx: Context, n_max: int, key_bits: int, nodes_capacity: int | None = None):
        torch = _torch()
        self.ctx, self.n_max, self.key_bits = ctx, n_max, key_bits
        dev = f"cuda:{ctx.device}"
        n = max(n_max, 1)
        kd = torch.int32 if key_bits == 32 else torch.int64
        self.keys = torch.empty(n, dtype=kd, device=dev)
        self.idx = torch.empty(n, dtype=torch.int32, device=dev)
        self.prefix_n = torch.empty(n, dtype=torch.uint8, device=dev)
        self.hll = torch.empty(n, dtype=torch.uint8, device=dev)
        self.hlr = torch.empty(n, dtype=torch.uint8, device=dev)
        self.left = torch.empty(n, dtype=torch.int32, device=dev)
        self.parent = torch.empty(n, dtype=torch.int32, device=dev)
        self.edge = torch.empty(n, dtype=torch.int32, device=dev)
        self.ps = torch.empty(n, dtype=torch.int32, device=dev)
        self.nodes_capacity = nodes_capacity or (n + 1024)
        self.nodes = torch.empty((self.nodes_capacity, 16), dtype=torch.int32, device=dev)
        self.counts = torch.zeros(4, dtype=torch.int32, device=dev)
        self.ws = ctx.workspace(OP_BUILD_OCTREE, n, key_bits)
        self.bufs = OctreeBuffers(_ptr(self.keys), _ptr(self.idx), _ptr(self.prefix_n), _ptr(self.hll),
                                  _ptr(self.hlr), _ptr(self.left), _ptr(self.parent), _ptr(self.edge),
                                  _ptr(self.ps), _ptr(self.nodes), self.nodes_capacity, _ptr(self.counts))
        self.graph = None

    def launch(self, pts, n: int | None = None, min_coord=0.0, rng=1024.0, stream=None):
        n = pts.shape[0] if n is None else n
        assert n <= self.n_max
        self.ctx.check(self.ctx.L.gtc_build_octree(self.ctx.h, _ptr(pts), n, min_coord, rng, self.key_bits,
                                                   ctypes.byref(self.bufs), _ptr(self.ws), self.ws.numel(),
                                                   _stream(stream)))

    def capture(self, pts, n: int | None = None, min_coord=0.0, rng=1024.0):
        """Capture the whole pipeline for `pts` into a CUDA graph."""
        torch = _torch()
        self.launch(pts, n, min_coord, rng)  # warm-up (sets kernel attributes)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            g.capture_begin()
            self.launch(pts, n, min_coord, rng, stream=s)
            g.capture_end()
        torch.cuda.synchronize()
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def counts_host(self):
        c = self.counts.cpu().numpy()
        return int(c[0]), int(c[1]), int(c[2])

    def result(self) -> OctreeResult:
        u, m, o = self.counts_host()
        self.ctx.device_status()
        return OctreeResult(self.keys[:u], self.idx[:u], self.prefix_n[:m], self.hll[:m], self.hlr[:m],
                            self.left[:m], self.parent[:m], self.edge[:m], self.ps[:u], self.nodes[:o], u, m, o)


@dataclass
class CloudResult:
    """One cloud of a batched build: the same fields as OctreeResult, as
    views into the batch's buffers (cloud-local indices)."""
    keys: object
    idx: object
    prefix_n: object
    has_leaf_left: object
    has_leaf_right: object
    left_child: object
    parent: object
    edge_count: object
    node_offsets: object
    nodes: object
    n_unique: int
    n_brt_nodes: int
    n_oct_nodes: int


class BatchPlan:
    """Resident buffers for batched builds (gtc_build_octree_batched): up to
    n_max points in up to clouds_max clouds, 32-bit codes.  offsets is a
    device uint32 tensor of n_clouds + 1 non-decreasing point offsets."""

    def __init__(self, ctx: Context, n_max: int, clouds_max: int, nodes_capacity: int | None = None):
        torch = _torch()
        self.ctx, self.n_max, self.clouds_max = ctx, n_max, clouds_max
        dev = f"cuda:{ctx.device}"
        n = max(n_max, 1)
        i32, u8 = torch.int32, torch.uint8
        self.keys = torch.empty(n, dtype=i32, device=dev)
        self.idx = torch.empty(n, dtype=i32, device=dev)
        self.prefix_n = torch.empty(n, dtype=u8, device=dev)
        self.hll = torch.empty(n, dtype=u8, device=dev)
        self.hlr = torch.empty(n, dtype=u8, device=dev)
        self.left = torch.empty(n, dtype=i32, device=dev)
        self.parent = torch.empty(n, dtype=i32, device=dev)
        self.edge = torch.empty(n, dtype=i32, device=dev)
        self.ps = torch.empty(n, dtype=i32, device=dev)
        self.nodes_capacity = nodes_capacity or (n + clouds_max + 1024)
        self.nodes = torch.empty((self.nodes_capacity, 16), dtype=i32, device=dev)
        self.key_offset = torch.zeros(clouds_max + 1, dtype=i32, device=dev)
        self.node_offset = torch.zeros(clouds_max + 1, dtype=i32, device=dev)
        self.cloud_counts = torch.zeros((clouds_max, 3), dtype=i32, device=dev)
        b = ctypes.c_size_t(0)
        ctx.check(ctx.L.gtc_batched_workspace_size(n_max, clouds_max, ctypes.byref(b)))
        self.ws = torch.empty(max(b.value, 256), dtype=torch.uint8, device=dev)
        self.bufs = _lib.BatchBuffers(_ptr(self.keys), _ptr(self.idx), _ptr(self.prefix_n), _ptr(self.hll),
                                      _ptr(self.hlr), _ptr(self.left), _ptr(self.parent), _ptr(self.edge),
                                      _ptr(self.ps), _ptr(self.nodes), self.nodes_capacity, _ptr(self.key_offset),
                                      _ptr(self.node_offset), _ptr(self.cloud_counts))
        self.graph = None
        self.n_clouds = 0

    def launch(self, pts, offsets, n_total: int | None = None, min_coord=0.0, rng=1024.0, stream=None):
        n_clouds = offsets.shape[0] - 1
        n_total = pts.shape[0] if n_total is None else n_total
        assert 1 <= n_clouds <= self.clouds_max and n_total <= self.n_max
        self.n_clouds = n_clouds
        self.ctx.check(self.ctx.L.gtc_build_octree_batched(
            self.ctx.h, _ptr(pts), _ptr(offsets), n_clouds, n_total, min_coord, rng, ctypes.byref(self.bufs),
            _ptr(self.ws), self.ws.numel(), _stream(stream)))

    def autotune(self, pts, offsets, n_total: int | None = None, min_coord=0.0, rng=1024.0, reps: int = 3) -> dict:
        """Time every batched onesweep shape on this batch and cache the
        fastest for its size; returns {"best": variant, "ms": [per-variant best
        build time]}.  Leaves the outputs of the last timed build."""
        n_clouds = offsets.shape[0] - 1
        n_total = pts.shape[0] if n_total is None else n_total
        assert 1 <= n_clouds <= self.clouds_max and n_total <= self.n_max
        self.n_clouds = n_clouds
        nv = self.ctx.L.gtc_batched_num_variants()
        times = (ctypes.c_float * nv)()
        best = ctypes.c_int(-1)
        self.ctx.check(self.ctx.L.gtc_autotune_batched(
            self.ctx.h, _ptr(pts), _ptr(offsets), n_clouds, n_total, min_coord, rng, ctypes.byref(self.bufs),
            _ptr(self.ws), self.ws.numel(), reps, ctypes.byref(best), times))
        return {"best": best.value, "ms": [float(t) for t in times]}

    def capture(self, pts, offsets, n_total: int | None = None, min_coord=0.0, rng=1024.0):
        """Capture the whole batched pipeline into one CUDA graph."""
        torch = _torch()
        self.launch(pts, offsets, n_total, min_coord, rng)  # warm-up (sets kernel attributes)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            g.capture_begin()
            self.launch(pts, offsets, n_total, min_coord, rng, stream=s)
            g.capture_end()
        torch.cuda.synchronize()
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def host_offsets(self):
        """(key_offset, node_offset, cloud_counts) as numpy arrays."""
        S = self.n_clouds
        return (self.key_offset[:S + 1].cpu().numpy().astype(np.int64),
                self.node_offset[:S + 1].cpu().numpy().astype(np.int64),
                self.cloud_counts[:S].cpu().numpy().astype(np.int64))

    def clouds(self) -> list:
        """Per-cloud results (raises on a device error, e.g. node capacity)."""
        self.ctx.device_status()
        ko, no, cc = self.host_offsets()
        out = []
        for c in range(self.n_clouds):
            u, m, o = (int(x) for x in cc[c])
            k0, n0 = int(ko[c]), int(no[c])
            out.append(CloudResult(self.keys[k0:k0 + u], self.idx[k0:k0 + u], self.prefix_n[k0:k0 + m],
                                   self.hll[k0:k0 + m], self.hlr[k0:k0 + m], self.left[k0:k0 + m],
                                   self.parent[k0:k0 + m], self.edge[k0:k0 + m], self.ps[k0:k0 + u],
                                   self.nodes[n0:n0 + o], u, m, o))
        return out


def batched_variants() -> list:
    """(threads, keys per thread) of every batched onesweep variant."""
    L = lib()
    out = []
    for v in range(L.gtc_batched_num_variants()):
        t, k = ctypes.c_int(), ctypes.c_int()
        if L.gtc_batched_variant_shape(v, ctypes.byref(t), ctypes.byref(k)) != 0:
            raise GtcError(1, "gtc_batched_variant_shape")
        out.append((t.value, k.value))
    return out


def batched_set_variant(v: int):
    """Pin one batched onesweep shape for every batched build (-1 unpins)."""
    if lib().gtc_batched_set_variant(v) != 0:
        raise GtcError(1, f"no batched variant {v}")


def batched_get_variant(n_total: int) -> int:
    return lib().gtc_batched_get_variant(n_total)


def autotune_lookup_batched(n_total: int) -> int:
    return lib().gtc_autotune_lookup_batched(n_total)


def build_octree_batched(ctx: Context, pts, offsets, min_coord=0.0, rng=1024.0) -> list:
    """One batched build of the clouds pts[offsets[c]:offsets[c+1]] (device
    tensors); returns per-cloud results, re-running once with a larger node
    array if the first guess was too small."""
    n_clouds = offsets.shape[0] - 1
    plan = BatchPlan(ctx, pts.shape[0], n_clouds)
    plan.launch(pts, offsets, min_coord=min_coord, rng=rng)
    total_nodes = int(plan.node_offset[n_clouds].item())
    if total_nodes > plan.nodes_capacity:
        ctx.device_status_code()
        plan = BatchPlan(ctx, pts.shape[0], n_clouds, nodes_capacity=total_nodes)
        plan.launch(pts, offsets, min_coord=min_coord, rng=rng)
    return plan.clouds()


OP_LEARNED_SORT = 6
LEARNED_FLAGS = {1: "overflow", 2: "order", 4: "non-monotone model"}


class LearnedModel:
    """Learned-bucket CDF model (gtc_learned_model_*): piecewise linear with
    `buckets` segments, trained on the GPU from a sample of sorted keys."""

    def __init__(self, ctx: Context, buckets: int):
        self.ctx = ctx
        h = ctypes.c_void_p()
        ctx.check(ctx.L.gtc_learned_model_create(ctx.h, buckets, ctypes.byref(h)))
        self.h = h
        self.buckets = buckets

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.gtc_learned_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        """(knots u64[B+1], heights f32[B+1]) as host numpy arrays."""
        kn = np.zeros(self.buckets + 1, np.uint64)
        hy = np.zeros(self.buckets + 1, np.float32)
        self.ctx.check(self.ctx.L.gtc_learned_model_export(self.h, kn.ctypes.data_as(ctypes.c_void_p),
                                                           hy.ctypes.data_as(ctypes.c_void_p)))
        return kn, hy

    def train(self, sorted_keys, stride: int = 100, iters: int = 600, lr: float = 0.05) -> float:
        """Knots at the quantiles of every stride-th key of sorted_keys, heights
        from the key-space uniform CDF, then `iters` Adam steps on the heights
        (learning rate decaying from lr to lr / 10^4).  Returns the final loss."""
        torch = _torch()
        loss = torch.zeros(1, dtype=torch.float32, device=sorted_keys.device)
        self.ctx.check(self.ctx.L.gtc_learned_train_u64(self.ctx.h, self.h, _ptr(sorted_keys), sorted_keys.numel(),
                                                        stride, iters, lr, _ptr(loss), _stream()))
        return float(loss.item())

    def gradient(self, sorted_keys, stride: int = 100, init: bool = True):
        torch = _torch()
        g = torch.zeros(self.buckets + 1, dtype=torch.float32, device=sorted_keys.device)
        loss = torch.zeros(1, dtype=torch.float32, device=sorted_keys.device)
        self.ctx.check(self.ctx.L.gtc_learned_gradient_u64(self.ctx.h, self.h, _ptr(sorted_keys),
                                                           sorted_keys.numel(), stride, 1 if init else 0, _ptr(g),
                                                           _ptr(loss), _stream()))
        return g, float(loss.item())

    def histogram(self, keys):
        torch = _torch()
        c = torch.zeros(self.buckets, dtype=torch.int32, device=keys.device)
        self.ctx.check(self.ctx.L.gtc_learned_histogram_u64(self.ctx.h, self.h, _ptr(keys), keys.numel(), _ptr(c),
                                                            _stream()))
        return c

    def autotune(self, keys, vals=None, ws=None, keys_out=None, vals_out=None, reps: int = 3) -> dict:
        """Time every grouping-pass shape on these keys and cache the fastest
        for n; returns {"best": variant, "ms": [per-variant best sort time]}."""
        torch = _torch()
        n = keys.numel()
        keys_out = torch.empty_like(keys) if keys_out is None else keys_out
        vals_out = torch.empty(n, dtype=torch.int32, device=keys.device) if vals_out is None else vals_out
        ws = self.ctx.workspace(OP_LEARNED_SORT, n, 64) if ws is None else ws
        flags = torch.zeros(1, dtype=torch.int32, device=keys.device)
        nv = self.ctx.L.gtc_learned_num_variants()
        times = (ctypes.c_float * nv)()
        best = ctypes.c_int(-1)
        self.ctx.check(self.ctx.L.gtc_autotune_learned(self.ctx.h, self.h, _ptr(keys), _ptr(vals), _ptr(keys_out),
                                                       _ptr(vals_out), n, _ptr(ws), ws.numel(), _ptr(flags), reps,
                                                       ctypes.byref(best), times))
        return {"best": best.value, "ms": [float(t) for t in times]}

    def sort(self, keys, vals=None, ws=None, keys_out=None, vals_out=None):
        """Out-of-place learned sort; returns (keys_out, vals_out, flags tensor)."""
        torch = _torch()
        n = keys.numel()
        keys_out = torch.empty_like(keys) if keys_out is None else keys_out
        vals_out = torch.empty(n, dtype=torch.int32, device=keys.device) if vals_out is None else vals_out
        ws = self.ctx.workspace(OP_LEARNED_SORT, n, 64) if ws is None else ws
        flags = torch.zeros(1, dtype=torch.int32, device=keys.device)
        self.ctx.check(self.ctx.L.gtc_learned_sort_u64(self.ctx.h, self.h, _ptr(keys), _ptr(vals), _ptr(keys_out),
                                                       _ptr(vals_out), n, _ptr(ws), ws.numel(), _ptr(flags), _stream()))
        return keys_out, vals_out, flags


def learned_variants() -> list:
    """(threads, keys per thread) of every learned grouping-pass variant."""
    L = lib()
    out = []
    for v in range(L.gtc_learned_num_variants()):
        t, k = ctypes.c_int(), ctypes.c_int()
        if L.gtc_learned_variant_shape(v, ctypes.byref(t), ctypes.byref(k)) != 0:
            raise GtcError(1, "gtc_learned_variant_shape")
        out.append((t.value, k.value))
    return out


def learned_set_variant(v: int):
    """Pin one grouping-pass shape for every learned sort (-1 unpins)."""
    if lib().gtc_learned_set_variant(v) != 0:
        raise GtcError(1, f"no learned variant {v}")


def learned_get_variant(n: int) -> int:
    return lib().gtc_learned_get_variant(n)


def autotune_lookup_learned(n: int) -> int:
    return lib().gtc_autotune_lookup_learned(n)


def learned_buckets_for(n: int) -> int:
    """Bucket count for n keys: 2^12, raised to the next power of two while the
    average bucket would exceed 4096 keys (the on-chip bucket sort holds at
    most 8192), capped at 16384."""
    b = 4096
    while n / b > 4096 and b < 16384:
        b *= 2
    return b


def build_octree(ctx: Context, pts, key_bits: int, min_coord=0.0, rng=1024.0) -> OctreeResult:
    plan = OctreePlan(ctx, pts.shape[0], key_bits)
    plan.launch(pts, min_coord=min_coord, rng=rng)
    u, m, o = plan.counts_host()
    if o > plan.nodes_capacity:
        ctx.device_status_code()
        plan = OctreePlan(ctx, pts.shape[0], key_bits, nodes_capacity=o)
        plan.launch(pts, min_coord=min_coord, rng=rng)
    return plan.result()


def nodes_to_numpy(nodes) -> np.ndarray:
    """int32 [o, 16] device/host tensor -> structured gtc_octnode array."""
    a = nodes.cpu().numpy() if hasattr(nodes, "cpu") else np.asarray(nodes)
    return np.ascontiguousarray(a).view(OCTNODE_DTYPE).reshape(-1)
