"""The oracle on its own: known answers, invariants, deviation switches and
regression against the committed vectors (tests/golden/oracle_small_*.npz)."""
import os

import numpy as np
import pytest

from gtc import workloads as W

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def pts_of(xyz):
    xyz = np.asarray(xyz, np.float32).reshape(-1, 3)
    p = np.ones((xyz.shape[0], 4), np.float32)
    p[:, :3] = xyz
    return p


# ------------------------------------------------------------------ morton --
def spread3(v, bits):
    out = 0
    for b in range(bits):
        out |= ((v >> b) & 1) << (3 * b)
    return out


@pytest.mark.parametrize("key_bits,B", [(32, 10), (64, 21)])
def test_morton_known_answers(oracle, key_bits, B):
    rng = np.random.default_rng(1)
    q = rng.integers(0, 1 << B, size=(200, 3))
    scale = float(1 << B)
    # cell centres, exactly representable: (q + 0.5) / 2^B * 1024
    xyz = ((q + 0.5) / scale * 1024.0).astype(np.float32)
    keys = oracle.morton(pts_of(xyz), key_bits)
    for k, (x, y, z) in zip(keys, q):
        assert int(k) == spread3(int(x), B) | (spread3(int(y), B) << 1) | (spread3(int(z), B) << 2)


def test_morton_wrap_and_saturation(oracle):
    # (x - min) / range * 1024 == 1024 wraps to cell 0 (mask), negatives and NaN -> 0 (D17)
    p = pts_of([[1024.0, 0.0, 0.0], [-5.0, 0.0, 0.0], [np.nan, 0.0, 0.0], [1023.999, 1023.999, 1023.999]])
    k = oracle.morton(p, 32)
    assert k[0] == 0 and k[1] == 0 and k[2] == 0
    assert k[3] == (1 << 30) - 1


@pytest.mark.parametrize("key_bits,B", [(32, 10), (64, 21)])
def test_decode_corner(oracle, key_bits, B):
    code = spread3(5, B) | (spread3(7, B) << 1) | (spread3(9, B) << 2)
    c = oracle.morton_to_xyz(code, key_bits, 0.0, 1024.0)
    s = 1024.0 / (1 << B)
    assert np.allclose(c, [5 * s, 7 * s, 9 * s, 1.0], rtol=0, atol=0)


# -------------------------------------------------------------------- sort --
@pytest.mark.parametrize("dtype", [np.uint32, np.uint64])
@pytest.mark.parametrize("threads", [1, 4])
def test_sort_is_stable(oracle, dtype, threads):
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 50, size=200_000).astype(dtype)
    vals = np.arange(keys.size, dtype=np.uint32)
    k, v = oracle.sort_pairs(keys, vals, threads=threads)
    order = np.argsort(keys, kind="stable")
    assert (k == keys[order]).all() and (v == order.astype(np.uint32)).all()


def test_unique_keeps_first(oracle):
    keys = np.array([1, 1, 2, 2, 2, 5, 9, 9], np.uint32)
    vals = np.arange(8, dtype=np.uint32)
    k, v, u = oracle.unique(keys, vals)
    assert u == 4 and k.tolist() == [1, 2, 5, 9] and v.tolist() == [0, 2, 5, 6]
    assert oracle.unique(np.zeros(0, np.uint32))[2] == 0


# -------------------------------------------------------------- radix tree --
def test_radix_tree_small_known(oracle):
    # 4 codes; the true tree: root [0,3] splits at 1 (bit 29 vs 28 ...)
    codes = np.array([0b0001, 0b0010, 0b0100, 0b0101], np.uint32)
    t = oracle.radix_tree(codes)
    assert t["multi_parent"] == 0
    assert t["prefix_n"].tolist() == [29, 30, 31]
    assert t["left_child"].tolist() == [1, 0, 2]
    assert t["has_leaf_left"].tolist() == [0, 1, 1]
    assert t["has_leaf_right"].tolist() == [0, 1, 1]
    assert t["parent"].tolist() == [0, 0, 0]


def test_d16_last_key_outlier(oracle):
    # top split falls at the last key: the literal root range (l = m - 1)
    # leaves key 3 without a parent and gives node 1 two parents.
    codes = np.array([0, 1, 2, 1 << 29], np.uint32)
    good = oracle.radix_tree(codes)
    lit = oracle.radix_tree(codes, oracle.LITERAL_D16)
    assert good["multi_parent"] == 0
    assert good["prefix_n"][0] == 2 and good["left_child"][0] == 2 and good["has_leaf_right"][0] == 1
    assert lit["multi_parent"] > 0 or lit["prefix_n"][0] != good["prefix_n"][0]


def _tree_is_binary_radix_tree(codes, t):
    m = codes.size - 1
    children_internal = np.zeros(m, np.int64)
    leaf_seen = np.zeros(m + 1, np.int64)
    for i in range(m):
        g = t["left_child"][i]
        for side, flag in ((0, t["has_leaf_left"][i]), (1, t["has_leaf_right"][i])):
            if flag:
                leaf_seen[g + side] += 1
            else:
                children_internal[g + side] += 1
                assert t["parent"][g + side] == i
    assert (children_internal[1:] == 1).all() and children_internal[0] == 0
    assert (leaf_seen == 1).all()


@pytest.mark.parametrize("key_bits", [32, 64])
def test_radix_tree_structure_random(oracle, key_bits):
    pts = W.gaussian_mixture_points(3000, 3, 20.0, noise=0.1, seed=5)
    k = oracle.morton(pts, key_bits)
    ks, _ = oracle.sort_pairs(k, np.arange(k.size, dtype=np.uint32))
    ku, _, u = oracle.unique(ks)
    t = oracle.radix_tree(ku)
    assert t["multi_parent"] == 0
    _tree_is_binary_radix_tree(ku, t)
    lit = oracle.radix_tree(ku, oracle.LITERAL_D1)
    assert lit["multi_parent"] > 0  # D1: the uint8 direction races


# ------------------------------------------------------------------ octree --
@pytest.mark.parametrize("key_bits", [32, 64])
def test_octree_valid_no_conflicts(oracle, key_bits):
    pts = W.uniform_points(1 << 15, seed=11)
    out, _ = oracle.build_octree(pts, key_bits)
    assert out["conflicts"] == 0
    assert oracle.validate_octree(out["nodes"], out["n_unique"]) == 0
    assert out["n_oct_nodes"] == 1 + int(out["edge_count"].sum())


def test_literal_switches_break_octree(oracle):
    pts = W.uniform_points(1 << 14, seed=2)
    for flag in (oracle.LITERAL_D2, oracle.LITERAL_D3):
        out, _ = oracle.build_octree(pts, 32, flags=flag)
        assert out["conflicts"] > 0
    out, _ = oracle.build_octree(pts, 32, flags=oracle.LITERAL_D6)
    assert out["conflicts"] == 0
    assert all(int(m) == 0 for m in out["nodes"]["child_leaf_mask"])  # SetLeaf clears a zero mask


def test_octree_corner_cases(oracle):
    # u = 0
    out, _ = oracle.build_octree(np.zeros((0, 4), np.float32), 32)
    assert out["n_oct_nodes"] == 0
    # u = 1 (D18): all points in one cell
    out, _ = oracle.build_octree(pts_of([[3.0, 4.0, 5.0]] * 7), 32)
    assert out["n_unique"] == 1 and out["n_oct_nodes"] == 1
    assert out["nodes"][0]["cell_size"] == 1024.0 and int(out["nodes"][0]["child_node_mask"]) == 0
    # u = 2: one radix node, both leaves under the root
    out, _ = oracle.build_octree(pts_of([[1.0, 1.0, 1.0], [900.0, 900.0, 900.0]]), 32)
    assert out["n_unique"] == 2 and out["n_oct_nodes"] == 1
    assert int(out["nodes"][0]["child_leaf_mask"]) == (1 << 0) | (1 << 7)
    assert oracle.validate_octree(out["nodes"], 2) == 0


def test_eight_corner_cells(oracle):
    # one point in each of the 8 top-level cells: a root with 8 leaves
    xyz = [[x, y, z] for z in (10.0, 600.0) for y in (10.0, 600.0) for x in (10.0, 600.0)]
    out, _ = oracle.build_octree(pts_of(xyz), 32)
    assert out["n_unique"] == 8 and out["n_oct_nodes"] == 1
    assert int(out["nodes"][0]["child_leaf_mask"]) == 0xFF
    assert sorted(out["nodes"][0]["children"].tolist()) == list(range(8))


def test_pwl_gradient_finite_differences(oracle):
    """The learned-model gradient of the oracle (the checker of the GPU
    backward kernel) agrees with central finite differences of its loss."""
    rng = np.random.default_rng(3)
    sample = np.sort(rng.integers(0, 1 << 62, size=5000, dtype=np.uint64))
    B = 16
    q = (np.arange(B + 1) * (sample.size - 1) // B)
    kn = sample[q].copy()
    kn[0] = 0
    kn[-1] = np.uint64(2**64 - 1)
    y = np.sort(rng.random(B + 1).astype(np.float32))
    loss, g = oracle.pwl_loss_grad(sample, kn, y)
    for k in range(B + 1):
        h = 1e-3
        yp, ym = y.astype(np.float64).copy(), y.astype(np.float64).copy()
        yp[k] += h
        ym[k] -= h
        lp, _ = oracle.pwl_loss_grad(sample, kn, yp.astype(np.float32))
        lm, _ = oracle.pwl_loss_grad(sample, kn, ym.astype(np.float32))
        # float32 heights: the perturbation is representable to ~1e-7 relative
        fd = (lp - lm) / (np.float32(y[k] + h) - np.float32(y[k] - h))
        assert abs(fd - g[k]) <= 1e-3 * max(abs(g[k]), 1e-3), (k, fd, g[k])


@pytest.mark.parametrize("key_bits", [32, 64])
def test_oracle_matches_committed_vectors(oracle, key_bits):
    g = np.load(os.path.join(GOLDEN, f"oracle_small_{key_bits}.npz"))
    out, _ = oracle.build_octree(g["pts"], key_bits)
    for k in ("keys", "idx", "prefix_n", "has_leaf_left", "has_leaf_right", "left_child", "parent", "edge_count",
              "node_offsets"):
        assert np.array_equal(out[k], g[k]), k
    assert np.array_equal(out["nodes"].view(np.int32).reshape(-1, 16), g["nodes"])
