"""Literal-mode switches against the oracle's literal forms, point gather in
payload order, and the stage-buffer export of a real build."""
import os

import numpy as np
import pytest

from gtc import workloads as W

pytestmark = pytest.mark.gpu


def dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t, dt):
    return t.cpu().numpy().view(dt)


@pytest.fixture
def literal(gtc_mod):
    yield gtc_mod.set_literal
    gtc_mod.set_literal(0)


@pytest.mark.parametrize("key_bits", [32, 64])
def test_literal_d2_edge_count(ctx, oracle, literal, key_bits, gtc_mod):
    pts = W.config1_points(1 << 18)
    k = oracle.morton(pts, key_bits)
    ks, _ = oracle.sort_pairs(k, np.arange(k.size, dtype=np.uint32), threads=4)
    codes, _, u = oracle.unique(ks)
    t = ctx.radix_tree(dev(codes), u - 1)
    literal(gtc_mod.LITERAL_D2)
    got = host(ctx.edge_count(t["prefix_n"], t["parent"], key_bits), np.uint32)
    e = oracle.radix_tree(codes)
    exp = oracle.edge_count(e["prefix_n"], e["parent"], key_bits, flags=oracle.LITERAL_D2)
    assert np.array_equal(got, exp)
    assert not np.array_equal(exp, oracle.edge_count(e["prefix_n"], e["parent"], key_bits))


@pytest.mark.parametrize("key_bits", [32, 64])
def test_literal_d6_fused_build(ctx, oracle, literal, key_bits, gtc_mod):
    import gtc
    import torch

    pts = W.config1_points(1 << 18)
    literal(gtc_mod.LITERAL_D6)
    res = gtc.build_octree(ctx, torch.from_numpy(pts).cuda(), key_bits)
    exp, _ = oracle.build_octree(pts, key_bits, flags=oracle.LITERAL_D6, threads=8)
    got = gtc.nodes_to_numpy(res.nodes)
    assert res.n_oct_nodes == exp["n_oct_nodes"]
    assert np.array_equal(got.view(np.int32), exp["nodes"].view(np.int32))
    assert (got["child_leaf_mask"] == 0).all() and (got["children"] != 0).any()


def test_literal_d6_stage_make_and_link(ctx, oracle, literal, gtc_mod):
    pts = W.config1_points(1 << 16)
    k = oracle.morton(pts, 32)
    ks, _ = oracle.sort_pairs(k, np.arange(k.size, dtype=np.uint32), threads=4)
    codes, _, u = oracle.unique(ks)
    e = oracle.radix_tree(codes)
    edge = oracle.edge_count(e["prefix_n"], e["parent"], 32)
    ps = oracle.prefix_sum(edge, u)
    enodes, conflicts, _ = oracle.octree(codes, e, edge, ps, flags=oracle.LITERAL_D6)
    assert conflicts == 0
    tree = {kk: dev(v) for kk, v in e.items() if kk != "multi_parent"}
    literal(gtc_mod.LITERAL_D6)
    gn = ctx.make_octree(dev(codes), tree, dev(edge), dev(ps), enodes.size)
    got = host(gn.contiguous(), np.int32).reshape(-1, 16)
    assert np.array_equal(got, enodes.view(np.int32).reshape(-1, 16))
    assert (enodes["child_leaf_mask"] == 0).all()


def test_gather_points_in_payload_order(ctx):
    rng = np.random.default_rng(9)
    pts = np.ones((300_001, 4), np.float32)
    pts[:, :3] = rng.random((300_001, 3)).astype(np.float32) * 1024
    idx = rng.permutation(300_001).astype(np.uint32)[:250_000]
    out = ctx.gather_points(dev(pts), dev(idx))
    assert np.array_equal(out.cpu().numpy(), pts[idx])


def test_export_build_files_match_buffers(ctx, tmp_path):
    import gtc
    import torch

    pts = W.config1_points(1 << 16)
    res = gtc.build_octree(ctx, torch.from_numpy(pts).cuda(), 32)
    paths = gtc.export_build(res, str(tmp_path))
    u, m, o = res.n_unique, res.n_brt_nodes, res.n_oct_nodes
    assert np.array_equal(np.fromfile(paths["keys"], "<u4"), host(res.keys, np.uint32)[:u])
    assert np.array_equal(np.fromfile(paths["parent"], "<i4"), host(res.parent, np.int32)[:m])
    assert np.array_equal(np.fromfile(paths["prefix_n"], "<u1"), host(res.prefix_n, np.uint8)[:m])
    nodes = np.fromfile(paths["nodes"], "<i4").reshape(-1, 16)
    assert nodes.shape[0] == o and np.array_equal(nodes, res.nodes.cpu().numpy()[:o])
    assert os.path.getsize(paths["node_offsets"]) == 4 * u
