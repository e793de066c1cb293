"""The reference-signature host shims (gtc_ref_*, csrc/compat.cpp) through the
C ABI with host arrays, in the Rust parameter order of the functions they
replace, against the oracle and the reference-derived fixtures:

  compute_morton      morton.rs:76-83       histogram       histogram.rs:38
  radix_sort          radixsort.rs:36       unique          unique.rs:37
  build_radix_tree    build_radix_tree.rs:34-43
  edge_count          edge_count.rs:41-47   partial_sum     partial_sum.rs:43
  build_octree        octree.rs:73-87       morton32_to_xyz morton.rs:43

Chained in main.rs:60-170's order they rebuild the reference fixture
(tests/golden/ref_pipeline_32.npz) byte for byte.  The edge cases are the
reference's own: n = 0, 1 and 2 points, all-equal keys (one unique key, a
tree of no nodes, an octree of the root alone).
"""
import ctypes
import os

import numpy as np
import pytest

from gtc import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None and a.size else None


@pytest.fixture(scope="module")
def L(gtc_mod):
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return gtc_mod.lib()


# ---- one shim at a time ----------------------------------------------------
def compute_morton(L, pts):
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 4)
    keys = np.zeros(max(pts.shape[0], 1), np.uint32)
    assert L.gtc_ref_compute_morton(_p(pts), _p(keys), pts.shape[0], 0.0, 1024.0, 256) == 0
    return keys[:pts.shape[0]]


def radix_sort(L, keys):
    out = np.zeros(max(keys.size, 1), np.uint32)
    assert L.gtc_ref_radix_sort(_p(keys), keys.size, _p(out), 1) == 0
    return out[:keys.size]


def unique(L, keys):
    buf = np.array(keys, np.uint32, copy=True)
    u = L.gtc_ref_unique(_p(buf), buf.size)
    return buf[:u], u


def build_radix_tree(L, codes):
    m = max(codes.size - 1, 0)
    out = {f: np.zeros(max(m, 1), dt) for f, dt in (("prefix_n", np.uint8), ("has_leaf_left", np.uint8),
                                                       ("has_leaf_right", np.uint8), ("left_child", np.int32),
                                                       ("parent", np.int32))}
    assert L.gtc_ref_build_radix_tree(m, _p(codes), _p(out["prefix_n"]), _p(out["has_leaf_left"]),
                                      _p(out["has_leaf_right"]), _p(out["left_child"]), _p(out["parent"]), 256) == 0
    return {k: v[:m] for k, v in out.items()}


def edge_count(L, tree):
    m = tree["prefix_n"].size
    edge = np.zeros(max(m, 1), np.uint32)
    assert L.gtc_ref_edge_count(_p(tree["prefix_n"]), _p(tree["parent"]), _p(edge), m, 256) == 0
    return edge[:m]


def partial_sum(L, data, first, last):
    out = np.zeros(max(last - first, 1), np.uint32)
    assert L.gtc_ref_partial_sum(_p(data), first, last, _p(out)) == 0
    return out[:last - first]


def node_offsets(L, edge, u):
    # main.rs:127-129: partial_sum(edge, 0, n_unique), then [0] = 0; the
    # element past the m edge counts reads as 0 (D4).
    data = np.zeros(u, np.uint32)
    data[:edge.size] = edge
    ps = partial_sum(L, data, 0, u)
    ps[0] = 0
    return ps


def build_octree(L, codes, tree, edge, ps):
    m = tree["prefix_n"].size
    o = 1 + (int(ps[m]) if m > 0 else 0)
    nodes = np.zeros((o, 16), np.int32)
    assert L.gtc_ref_build_octree(_p(nodes), _p(ps), _p(edge), _p(codes), _p(tree["prefix_n"]), _p(tree["parent"]),
                                  0.0, 1024.0, m, _p(tree["has_leaf_left"]), _p(tree["has_leaf_right"]),
                                  _p(tree["left_child"]), 256) == 0
    return nodes


# ---- tests -------------------------------------------------------------------
def test_reference_fixture_through_the_shims(L):
    """main.rs:60-170 driven through the shims reproduces the reference
    shaders' outputs (ref_pipeline_32.npz) for every stage."""
    fx = dict(np.load(os.path.join(GOLDEN, "ref_pipeline_32.npz")))
    keys = compute_morton(L, fx["pts"])
    skeys = radix_sort(L, keys)
    np.testing.assert_array_equal(skeys, np.sort(keys))
    codes, u = unique(L, skeys)
    np.testing.assert_array_equal(codes, fx["keys"])
    tree = build_radix_tree(L, codes)
    for f in ("prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent"):
        np.testing.assert_array_equal(tree[f], fx[f], err_msg=f)
    edge = edge_count(L, tree)
    np.testing.assert_array_equal(edge, fx["edge_count"])
    ps = node_offsets(L, edge, u)
    np.testing.assert_array_equal(ps, fx["node_offsets"])
    nodes = build_octree(L, codes, tree, edge, ps)
    np.testing.assert_array_equal(nodes, fx["nodes"])


@pytest.mark.parametrize("n", [0, 1, 2, 1000, 1 << 16])
def test_compute_morton(L, oracle, n):
    pts = W.config1_points(n, seed=11) if n else np.zeros((0, 4), np.float32)
    np.testing.assert_array_equal(compute_morton(L, pts), oracle.morton(pts, 32))


@pytest.mark.parametrize("n", [0, 1, 2, 777, 1 << 20])
def test_radix_sort_and_histogram(L, oracle, n):
    keys = W.config3_keys(n, 32, seed=3) if n else np.zeros(0, np.uint32)
    np.testing.assert_array_equal(radix_sort(L, keys), np.sort(keys))
    hist = np.zeros(1024, np.uint32)
    assert L.gtc_ref_histogram(keys.size, _p(keys), _p(hist)) == 0
    np.testing.assert_array_equal(hist.reshape(4, 256), oracle.global_hist(keys, 4))


def test_histogram_of_the_recorded_run(L, oracle):
    """test_radix_sort's keys 10,000,000..1 (main.rs:189-190): the corrected
    histogram, equal to the reference's recorded dump on the three passes its
    mask bug leaves alone (output.txt:7684-8707, less its constant 9n)."""
    n = 10_000_000
    keys = np.arange(n, 0, -1, dtype=np.uint32)
    hist = np.zeros(1024, np.uint32)
    assert L.gtc_ref_histogram(n, _p(keys), _p(hist)) == 0
    rec = np.array([int(x) for x in open(os.path.join(GOLDEN, "ref_global_hist.txt")) if x.strip() and
                    not x.startswith("#")], np.int64).reshape(4, 256)
    h = hist.reshape(4, 256).astype(np.int64)
    for p in (0, 2, 3):
        assert (rec[p, 1:] - 9 * n == h[p, 1:]).all() and h[p, 0] == 0


@pytest.mark.parametrize("case", ["empty", "one", "all_equal", "runs"])
def test_unique(L, oracle, case):
    keys = {"empty": np.zeros(0, np.uint32), "one": np.array([7], np.uint32),
            "all_equal": np.full(5000, 12345, np.uint32),
            "runs": np.sort(W.config3_keys(300_000, 32, seed=5) >> np.uint32(18))}[case]
    got, u = unique(L, keys)
    exp, _, u_exp = oracle.unique(keys)
    assert u == u_exp
    np.testing.assert_array_equal(got, exp)


@pytest.mark.parametrize("n_pts", [1, 2, 3, 9, 1 << 12, 1 << 18])
def test_tree_edges_offsets_octree(L, oracle, n_pts):
    """The tree, edge count, offsets and octree shims against the oracle, from
    one point (u = 1: no tree nodes, the root alone) up."""
    codes = np.unique(oracle.morton(W.uniform_points(n_pts, seed=n_pts), 32))
    u = codes.size
    tree = build_radix_tree(L, codes)
    exp_tree = oracle.radix_tree(codes)
    for f in ("prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent"):
        np.testing.assert_array_equal(tree[f], exp_tree[f], err_msg=f)
    edge = edge_count(L, tree)
    np.testing.assert_array_equal(edge, oracle.edge_count(exp_tree["prefix_n"], exp_tree["parent"], 32))
    ps = node_offsets(L, edge, u)
    np.testing.assert_array_equal(ps, oracle.prefix_sum(edge, u))
    nodes = build_octree(L, codes, tree, edge, ps)
    exp_nodes, conflicts, _ = oracle.octree(codes, exp_tree, edge, ps)
    assert conflicts == 0
    np.testing.assert_array_equal(nodes, exp_nodes.view(np.int32).reshape(-1, 16))


def test_all_equal_points_build_the_root_alone(L, oracle):
    pts = np.repeat(W.uniform_points(1, seed=4), 64, axis=0)
    codes, u = unique(L, radix_sort(L, compute_morton(L, pts)))
    assert u == 1
    tree = build_radix_tree(L, codes)
    assert tree["prefix_n"].size == 0
    nodes = build_octree(L, codes, tree, np.zeros(0, np.uint32), node_offsets(L, np.zeros(0, np.uint32), 1))
    exp, _ = oracle.build_octree(pts, 32)
    np.testing.assert_array_equal(nodes, exp["nodes"].view(np.int32).reshape(-1, 16))


@pytest.mark.parametrize("first,last", [(0, 0), (0, 1), (5, 5), (3, 1000), (0, 1 << 20), (17, (1 << 20) - 3)])
def test_partial_sum(L, first, last):
    data = (W.config3_keys(1 << 20, 32, seed=9) & np.uint32(1023)).astype(np.uint32)
    got = partial_sum(L, data, first, last)
    np.testing.assert_array_equal(got, np.cumsum(data[first:last], dtype=np.uint64).astype(np.uint32))
