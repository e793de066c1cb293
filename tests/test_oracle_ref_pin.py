"""Pins the oracle to the reference's own shader code, stage by stage.

oracle/_ref/libref_shaders.so holds the reference's GLSL function bodies
(vulkan/radixsort-vulkan/shader/{morton,unique,build_radix_tree,edge_count,
partial_sum,octree}.comp) compiled unchanged as C++ on the CPU, run as one
serial invocation, with named text patches for the deviation rows
(oracle/ref_shaders.py).  Every stage of the oracle is compared with it byte
for byte on the same inputs:

* the corrected oracle (flags 0) against the `fix` build (all D-patches);
* each literal switch ORC_LITERAL_DK against the build that leaves exactly
  that deviation unpatched (`lit_dK`), and ORC_LITERAL_D1 | D16 against the
  unpatched tree shader;
* the 64-bit oracle against the shaders with 64-bit codes substituted (W64).

The library is built here from the reference checkout; where neither the
library nor the checkout exists (the GPU host), these tests skip and
tests/test_oracle.py checks the oracle against the committed fixtures that
tests/golden/make_golden.py wrote from this library.
"""
import numpy as np
import pytest

from gtc import workloads as W

INPUTS = {
    "uniform_4k": lambda: W.uniform_points(1 << 12, seed=0),
    "uniform_16k": lambda: W.uniform_points(1 << 14, seed=1),
    "uniform_64k": lambda: W.config1_points(1 << 16, seed=0),
    "clustered_16k": lambda: W.gaussian_mixture_points(1 << 14, 8, 2.0, noise=0.02, seed=2),
    "dense_8k": lambda: W.gaussian_mixture_points(1 << 13, 2, 0.3, seed=3),
    "duplicates_8k": lambda: _grid_points(1 << 13, 8, seed=4),
    "corners_8": lambda: _corner_points(),
    "two_points": lambda: W.uniform_points(2, seed=5),
    "one_point": lambda: W.uniform_points(1, seed=8),
    "all_equal": lambda: np.repeat(W.uniform_points(1, seed=9), 1000, axis=0),
    "outlier_last": lambda: _outlier_points(),
}


def _grid_points(n, cells, seed):
    # many repeated codes: coordinates snapped to a coarse grid
    p = W.uniform_points(n, seed=seed)
    step = np.float32(1024.0 / cells)
    p[:, :3] = np.floor(p[:, :3] / step) * step
    return p


def _corner_points():
    c = np.array([[x, y, z] for x in (100.0, 900.0) for y in (100.0, 900.0) for z in (100.0, 900.0)], np.float32)
    p = np.ones((8, 4), np.float32)
    p[:, :3] = c
    return p


def _outlier_points():
    # the top split falls at the last key: every point in the low octant but one
    p = W.uniform_points(2000, seed=6)
    p[:, :3] *= np.float32(0.4)
    p[-1, :3] = np.float32(1000.0)
    return p


@pytest.fixture(scope="module")
def ref():
    from oracle import ref as R
    from oracle import ref_shaders

    root = ref_shaders.default_reference_root()
    if root is not None:
        R.build(root)
    if not R.available():
        pytest.skip("no reference checkout and no oracle/_ref build on this machine")
    return R


def _codes(oracle, pts, key_bits):
    keys = oracle.morton(pts, key_bits)
    return np.unique(keys)  # sorted distinct codes


def _same_tree(a, b):
    for f in ("prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent"):
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


def _node_words(nodes):
    return np.ascontiguousarray(nodes).view(np.int32).reshape(-1, 16)[:, :15]


@pytest.mark.parametrize("name", list(INPUTS))
def test_morton32_matches_shader(oracle, ref, name):
    pts = INPUTS[name]()
    np.testing.assert_array_equal(oracle.morton(pts, 32), ref.morton32(pts))


def test_morton32_wrap_matches_shader(oracle, ref):
    # exactly `range` above min quantises to 2^10, which the shader's mask wraps to 0
    p = np.ones((3, 4), np.float32)
    p[0, :3] = [1024.0, 512.0, 0.0]
    p[1, :3] = [0.0, 1023.9999, 1024.0]
    p[2, :3] = [3.0, 2.5, 7.75]
    np.testing.assert_array_equal(oracle.morton(p, 32), ref.morton32(p))


@pytest.mark.parametrize("key_bits", [32, 64])
@pytest.mark.parametrize("name", list(INPUTS))
def test_unique_matches_shader(oracle, ref, name, key_bits):
    keys = np.sort(oracle.morton(INPUTS[name](), key_bits), kind="stable")
    k_orc, _, u_orc = oracle.unique(keys)
    k_ref, u_ref = ref.unique(keys)
    assert u_orc == u_ref
    np.testing.assert_array_equal(k_orc, k_ref)


@pytest.mark.parametrize("key_bits", [32, 64])
@pytest.mark.parametrize("name", list(INPUTS))
def test_radix_tree_matches_shader(oracle, ref, name, key_bits):
    codes = _codes(oracle, INPUTS[name](), key_bits)
    fixed = oracle.radix_tree(codes)
    assert fixed["multi_parent"] == 0
    _same_tree(fixed, ref.radix_tree(codes, "fix"))
    # the unpatched shader: uint8_t direction (D1) and l = n - 1 at the root (D16)
    lit = oracle.radix_tree(codes, oracle.LITERAL_D1 | oracle.LITERAL_D16)
    _same_tree(lit, ref.radix_tree(codes, "lit"))
    if key_bits == 32:
        _same_tree(oracle.radix_tree(codes, oracle.LITERAL_D1), ref.radix_tree(codes, "lit_d1"))
        _same_tree(oracle.radix_tree(codes, oracle.LITERAL_D16), ref.radix_tree(codes, "lit_d16"))


def test_literal_tree_deviations_show(oracle, ref):
    # D1: the literal direction is +1 everywhere, so nodes that Karras builds
    # leftwards come out wrong; D16 only changes the tree when the top split
    # falls at the last key.
    codes = _codes(oracle, INPUTS["uniform_16k"](), 32)
    fixed = ref.radix_tree(codes, "fix")
    lit_d1 = ref.radix_tree(codes, "lit_d1")
    assert (fixed["left_child"] != lit_d1["left_child"]).any()
    _same_tree(ref.radix_tree(codes, "lit_d16"), fixed)
    out = _codes(oracle, INPUTS["outlier_last"](), 32)
    assert (ref.radix_tree(out, "lit_d16")["left_child"] != ref.radix_tree(out, "fix")["left_child"]).any()


@pytest.mark.parametrize("key_bits", [32, 64])
@pytest.mark.parametrize("name", list(INPUTS))
def test_edge_count_and_offsets_match_shader(oracle, ref, name, key_bits):
    codes = _codes(oracle, INPUTS[name](), key_bits)
    tree = oracle.radix_tree(codes)
    e_orc = oracle.edge_count(tree["prefix_n"], tree["parent"], key_bits)
    np.testing.assert_array_equal(e_orc, ref.edge_count(tree["prefix_n"], tree["parent"], key_bits, "fix"))
    np.testing.assert_array_equal(oracle.edge_count(tree["prefix_n"], tree["parent"], key_bits, oracle.LITERAL_D2),
                                  ref.edge_count(tree["prefix_n"], tree["parent"], key_bits, "lit"))
    u = codes.size
    np.testing.assert_array_equal(oracle.prefix_sum(e_orc, u), ref.node_offsets(e_orc, u))


@pytest.mark.parametrize("key_bits", [32, 64])
@pytest.mark.parametrize("name", list(INPUTS))
def test_octree_matches_shader(oracle, ref, name, key_bits):
    codes = _codes(oracle, INPUTS[name](), key_bits)
    tree = oracle.radix_tree(codes)
    edge = oracle.edge_count(tree["prefix_n"], tree["parent"], key_bits)
    ps = oracle.prefix_sum(edge, codes.size)
    nodes, conflicts, caps = oracle.octree(codes, tree, edge, ps)
    assert conflicts == 0 and caps == 0
    assert oracle.validate_octree(nodes, codes.size) == 0
    got = ref.octree(codes, tree, edge, ps, variant="fix")
    np.testing.assert_array_equal(_node_words(nodes), _node_words(got))


@pytest.mark.parametrize("name", ["uniform_4k", "clustered_16k", "duplicates_8k", "corners_8", "outlier_last"])
def test_octree_literal_switches_match_shader(oracle, ref, name):
    codes = _codes(oracle, INPUTS[name](), 32)
    tree = oracle.radix_tree(codes)
    u = codes.size
    edge = oracle.edge_count(tree["prefix_n"], tree["parent"], 32)
    ps = oracle.prefix_sum(edge, u)
    fixed = ref.octree(codes, tree, edge, ps, variant="fix")
    # D6: SetLeaf clears a bit of a zero mask; only the leaf masks change.
    d6, _, _ = oracle.octree(codes, tree, edge, ps, flags=oracle.LITERAL_D6)
    ref_d6 = ref.octree(codes, tree, edge, ps, variant="lit_d6")
    np.testing.assert_array_equal(_node_words(d6), _node_words(ref_d6))
    assert (ref_d6["child_leaf_mask"] == 0).all()
    diff = _node_words(ref_d6) != _node_words(fixed)
    assert not diff[:, :14].any()  # children, corner, cell size, node mask
    # D3: slots from the inclusive scan, overlapping ranges.
    d3, _, _ = oracle.octree(codes, tree, edge, ps, flags=oracle.LITERAL_D3)
    np.testing.assert_array_equal(_node_words(d3), _node_words(ref.octree(codes, tree, edge, ps, variant="lit_d3")))
    # D2: literal depth in edge counts, offsets and the octree together.  The
    # literal link shifts a code by 30 - 3 * (prefix_n / 3 + 1), a negative
    # count (undefined) for prefix lengths of 30 and 31, so the literal form
    # is compared only on inputs where no prefix length reaches 30.
    if tree["prefix_n"].max() >= 30:
        return
    e2 = oracle.edge_count(tree["prefix_n"], tree["parent"], 32, oracle.LITERAL_D2)
    ps2 = oracle.prefix_sum(e2, u)
    d2, _, _ = oracle.octree(codes, tree, e2, ps2, flags=oracle.LITERAL_D2)
    np.testing.assert_array_equal(_node_words(d2), _node_words(ref.octree(codes, tree, e2, ps2, variant="lit_d2")))


@pytest.mark.parametrize("key_bits", [32, 64])
@pytest.mark.parametrize("name", ["uniform_64k", "clustered_16k", "duplicates_8k", "two_points", "one_point",
                                  "all_equal"])
def test_whole_path_matches_shaders(oracle, ref, name, key_bits):
    """main.rs:60-170's order through the shaders vs the oracle's fused build."""
    pts = INPUTS[name]()
    exp, _ = oracle.build_octree(pts, key_bits)
    got = ref.build_octree(pts if key_bits == 32 else oracle.morton(pts, 64), key_bits)
    assert (got["n_unique"], got["n_brt_nodes"], got["n_oct_nodes"]) == \
        (exp["n_unique"], exp["n_brt_nodes"], exp["n_oct_nodes"])
    for f in ("keys", "idx", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent", "edge_count",
              "node_offsets"):
        np.testing.assert_array_equal(exp[f], got[f], err_msg=f)
    np.testing.assert_array_equal(_node_words(exp["nodes"]), _node_words(got["nodes"]))


# ---- committed reference-derived fixtures (run on every machine) ----------
REF_FIELDS = ("keys", "idx", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent", "edge_count",
              "node_offsets")


def load_ref_fixture(key_bits):
    import os

    path = os.path.join(os.path.dirname(__file__), "golden", f"ref_pipeline_{key_bits}.npz")
    return dict(np.load(path))


@pytest.mark.parametrize("key_bits", [32, 64])
def test_oracle_matches_reference_fixture(oracle, key_bits):
    """The oracle's fused build against the reference shaders' outputs that
    tests/golden/make_golden.py recorded (ref_pipeline_{32,64}.npz)."""
    fx = load_ref_fixture(key_bits)
    exp, _ = oracle.build_octree(fx["pts"], key_bits)
    assert exp["n_unique"] == fx["keys"].size and exp["n_oct_nodes"] == fx["nodes"].shape[0]
    for f in REF_FIELDS:
        np.testing.assert_array_equal(exp[f], fx[f], err_msg=f)
    np.testing.assert_array_equal(exp["nodes"].view(np.int32).reshape(-1, 16), fx["nodes"])
