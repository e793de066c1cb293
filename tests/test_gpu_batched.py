"""Parity of the batched build (gtc_build_octree_batched) with the oracle:
every cloud of a batch must equal the oracle's single-cloud 32-bit build of
that cloud alone, buffer for buffer and node for node (cloud-local indices)."""
import numpy as np
import pytest

from gtc import workloads as W

pytestmark = pytest.mark.gpu


def _p(xyz):
    xyz = np.asarray(xyz, np.float32).reshape(-1, 3)
    out = np.ones((xyz.shape[0], 4), np.float32)
    out[:, :3] = xyz
    return out


def _batch(clouds):
    sizes = [c.shape[0] for c in clouds]
    offsets = np.zeros(len(clouds) + 1, np.uint32)
    offsets[1:] = np.cumsum(sizes)
    pts = np.concatenate(clouds) if sum(sizes) else np.zeros((0, 4), np.float32)
    return np.ascontiguousarray(pts, np.float32), offsets


def _check_cloud(gtc, oracle, res, pts_c, tag):
    exp, _ = oracle.build_octree(pts_c, 32, threads=8)
    assert exp["conflicts"] == 0
    assert (res.n_unique, res.n_brt_nodes, res.n_oct_nodes) == (exp["n_unique"], exp["n_brt_nodes"],
                                                                 exp["n_oct_nodes"]), tag
    pairs = [("keys", res.keys, np.uint32), ("idx", res.idx, np.uint32), ("prefix_n", res.prefix_n, np.uint8),
             ("has_leaf_left", res.has_leaf_left, np.uint8), ("has_leaf_right", res.has_leaf_right, np.uint8),
             ("left_child", res.left_child, np.int32), ("parent", res.parent, np.int32),
             ("edge_count", res.edge_count, np.uint32), ("node_offsets", res.node_offsets, np.uint32)]
    for name, t, dt in pairs:
        got = t.cpu().numpy().view(dt)
        assert np.array_equal(got, exp[name]), (tag, name)
    got_nodes = gtc.nodes_to_numpy(res.nodes)
    assert np.array_equal(got_nodes.view(np.int32), exp["nodes"].view(np.int32)), (tag, "nodes")


def _run_batch(ctx, oracle, pts, offsets, tag):
    import gtc
    import torch

    tp = torch.from_numpy(pts).cuda() if pts.shape[0] else torch.zeros((0, 4), dtype=torch.float32, device="cuda")
    to = torch.from_numpy(offsets.view(np.int32)).cuda()
    results = gtc.build_octree_batched(ctx, tp, to)
    assert len(results) == offsets.size - 1
    for c in range(offsets.size - 1):
        s, e = int(offsets[c]), int(offsets[c + 1])
        _check_cloud(gtc, oracle, results[c], pts[s:e], f"{tag}/cloud{c}")
    return results


@pytest.mark.parametrize("variant", [0, 1, 3], ids=["512x12", "256x16", "512x8"])
def test_batched_edge_cases(ctx, oracle, variant):
    clouds = [
        np.zeros((0, 4), np.float32),                       # empty first cloud
        _p([[1.0, 2.0, 3.0]]),                              # one point
        _p([[1.0, 2.0, 3.0], [700.0, 2.0, 3.0]]),           # two points
        _p([[5.5, 6.5, 7.5]] * 5000),                       # one distinct code
        W.uniform_points(12_345, seed=3),                   # ragged last tile
        np.zeros((0, 4), np.float32),                       # runs of empty clouds
        np.zeros((0, 4), np.float32),
        np.repeat(W.uniform_points(3000, seed=4), 7, axis=0),  # duplicates
        W.gaussian_mixture_points(70_000, 1, 0.05, seed=6),  # dense cluster: long equal runs
        _p([[1024.0, 0.0, 0.0], [0.0, 1023.99, 0.0], [0.0, 0.0, 0.0], [512.0, 512.0, 512.0]]),
        _p([[float(i) * 0.25, 1.0, 1.0] for i in range(4096)]),
        W.uniform_points(6144, seed=9),                     # exactly one sort tile
        W.uniform_points(6145, seed=10),                    # one tile + one key
        _p([[9.0, 9.0, 9.0]]),                              # one point, last cloud
        np.zeros((0, 4), np.float32),                       # empty last cloud
        W.uniform_points(4096, seed=11),                    # exactly one tile of the 4096-key shapes
        W.uniform_points(4097, seed=12),
    ]
    pts, offsets = _batch(clouds)
    import gtc

    gtc.batched_set_variant(variant)  # the tile shape also decides how the clouds are cut
    try:
        _run_batch(ctx, oracle, pts, offsets, f"edge/v{variant}")
    finally:
        gtc.batched_set_variant(-1)


@pytest.mark.parametrize("tree_method", [1, 0], ids=["window", "karras"])
def test_batched_config4_reduced(ctx, oracle, gtc_mod, tree_method):
    """64 clouds, sizes log-uniform in [1K, 100K], alternately uniform and
    8-cluster Gaussian (the batched workload's shape at reduced size), with
    both radix tree kernels."""
    L = gtc_mod.lib()
    assert L.gtc_tree_set_method(tree_method) == 0
    try:
        pts, offsets = W.config4_clouds(64, seed=1, lo=1000, hi=100_000)
        _run_batch(ctx, oracle, pts, offsets, "config4-reduced")
    finally:
        L.gtc_tree_set_method(1)


def test_batched_config4_full(ctx, oracle):
    """The full batched workload: 512 clouds, sizes log-uniform in [1K, 1M]
    (about 83M points); every cloud is checked against the oracle's build of
    that cloud alone, buffer for buffer and node for node.  The oracle builds
    run on a thread pool (ctypes releases the GIL), after every GPU result is
    on the host."""
    import concurrent.futures as cf
    import os

    import gtc
    import torch

    pts, offsets = W.config4_clouds(512, seed=0)
    tp = torch.from_numpy(pts).cuda()
    to = torch.from_numpy(offsets.view(np.int32)).cuda()
    results = gtc.build_octree_batched(ctx, tp, to)
    assert len(results) == 512
    fields = [("keys", np.uint32), ("idx", np.uint32), ("prefix_n", np.uint8), ("has_leaf_left", np.uint8),
              ("has_leaf_right", np.uint8), ("left_child", np.int32), ("parent", np.int32),
              ("edge_count", np.uint32), ("node_offsets", np.uint32)]
    got = []
    for res in results:
        g = {name: getattr(res, name).cpu().numpy().view(dt) for name, dt in fields}
        g["nodes"] = gtc.nodes_to_numpy(res.nodes).view(np.int32)
        g["counts"] = (res.n_unique, res.n_brt_nodes, res.n_oct_nodes)
        got.append(g)
    del results, tp, to

    def check(c):
        s, e = int(offsets[c]), int(offsets[c + 1])
        exp, _ = oracle.build_octree(pts[s:e], 32, threads=1)
        g = got[c]
        if exp["conflicts"] != 0:
            return f"cloud {c}: oracle conflicts"
        if g["counts"] != (exp["n_unique"], exp["n_brt_nodes"], exp["n_oct_nodes"]):
            return f"cloud {c}: counts {g['counts']}"
        for name, _ in fields:
            if not np.array_equal(g[name], exp[name]):
                return f"cloud {c}: {name}"
        if not np.array_equal(g["nodes"], exp["nodes"].view(np.int32)):
            return f"cloud {c}: nodes"
        return None

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        bad = [r for r in ex.map(check, range(512)) if r]
    assert not bad, bad[:10]


def test_batched_graph_replay(ctx, oracle):
    import gtc
    import torch

    pts, offsets = W.config4_clouds(24, seed=5, lo=100, hi=50_000)
    tp = torch.from_numpy(pts).cuda()
    to = torch.from_numpy(offsets.view(np.int32)).cuda()
    plan = gtc.BatchPlan(ctx, pts.shape[0], offsets.size - 1)
    plan.capture(tp, to)
    for _ in range(3):
        plan.replay()
    torch.cuda.synchronize()
    for c, res in enumerate(plan.clouds()):
        s, e = int(offsets[c]), int(offsets[c + 1])
        _check_cloud(gtc, oracle, res, pts[s:e], f"graph/cloud{c}")


def test_batched_all_empty(ctx):
    import gtc
    import torch

    plan = gtc.BatchPlan(ctx, 16, 3)
    offsets = torch.zeros(4, dtype=torch.int32, device="cuda")
    plan.launch(torch.zeros((0, 4), dtype=torch.float32, device="cuda"), offsets, n_total=0)
    ko, no, cc = plan.host_offsets()
    assert not ko.any() and not no.any() and not cc.any()
    assert [r.n_unique for r in plan.clouds()] == [0, 0, 0]


def test_batched_node_capacity_reported(ctx):
    """A node array that is too small is reported as a capacity error; the
    kernels store nothing past it."""
    import gtc
    import torch

    pts, offsets = _batch([W.uniform_points(5000, seed=1), W.uniform_points(7000, seed=2)])
    tp = torch.from_numpy(pts).cuda()
    to = torch.from_numpy(offsets.view(np.int32)).cuda()
    plan = gtc.BatchPlan(ctx, pts.shape[0], 2, nodes_capacity=100)
    plan.launch(tp, to)
    with pytest.raises(gtc.GtcError) as ei:
        plan.ctx.device_status()
    assert ei.value.status == 7
    big = gtc.BatchPlan(ctx, pts.shape[0], 2)
    big.launch(tp, to)
    assert int(big.node_offset[2].item()) > 100
    big.clouds()


@pytest.mark.parametrize("offs", [[0, 100, 50, 200], [0, 100, 150, 199], [5, 100, 150, 200]])
def test_batched_bad_device_offsets(ctx, offs):
    """Offsets that do not partition [0, n_total) are caught on the device:
    the status reads INVALID_ARG and the batch reports no codes, no nodes."""
    import gtc
    import torch

    pts = torch.from_numpy(W.uniform_points(200, seed=1)).cuda()
    plan = gtc.BatchPlan(ctx, 200, 3)
    plan.launch(pts, torch.tensor(offs, dtype=torch.int32, device="cuda"), n_total=200)
    with pytest.raises(gtc.GtcError) as ei:
        ctx.device_status()
    assert ei.value.status == 1
    ko, no, cc = plan.host_offsets()
    assert not ko.any() and not no.any() and not cc.any()


def test_batched_rejects_bad_args(ctx):
    import gtc
    import torch

    plan = gtc.BatchPlan(ctx, 64, 2)
    pts = torch.zeros((64, 4), dtype=torch.float32, device="cuda")
    offsets = torch.tensor([0, 32, 64], dtype=torch.int32, device="cuda")
    # Points not 16-byte aligned: refused on the host before any launch.
    with pytest.raises(gtc.GtcError) as ei:
        plan.launch(pts.view(-1)[1:], offsets, n_total=64)
    assert ei.value.status == 1


def test_every_batched_variant_identical_and_tuned(ctx, oracle):
    """Every compiled tile shape of the segmented onesweep gives the same
    batch, byte for byte (each cloud also against the oracle under a
    non-default shape); the autotuner times them all on the batch and its pick
    is what an unpinned build uses."""
    import gtc
    import torch

    gtc.autotune_clear()
    pts_np, offs_np = W.config4_clouds(48, seed=11)
    pts = torch.from_numpy(pts_np).cuda()
    offs = torch.from_numpy(offs_np.view(np.int32)).cuda()
    n = pts_np.shape[0]
    plan = gtc.BatchPlan(ctx, n, 48)
    ref = None
    try:
        for v in range(len(gtc.batched_variants())):
            gtc.batched_set_variant(v)
            plan.launch(pts, offs)
            torch.cuda.synchronize()
            ctx.device_status()
            got = [t.clone() for t in (plan.keys, plan.idx, plan.parent, plan.edge, plan.nodes, plan.node_offset)]
            if ref is None:
                ref = got
                continue
            for a, b in zip(ref, got):
                assert torch.equal(a, b), v
        for c, res in enumerate(plan.clouds()):  # the last (non-default) shape, against the oracle
            s, e = int(offs_np[c]), int(offs_np[c + 1])
            if c % 4 == 0:
                _check_cloud(gtc, oracle, res, pts_np[s:e], f"variant{v}/cloud{c}")
    finally:
        gtc.batched_set_variant(-1)
    r = plan.autotune(pts, offs, reps=2)
    assert len(r["ms"]) == len(gtc.batched_variants()) and all(0 < t < 1e4 for t in r["ms"])
    assert gtc.autotune_lookup_batched(n) == r["best"] == gtc.batched_get_variant(n)
    plan.launch(pts, offs)
    torch.cuda.synchronize()
    assert torch.equal(plan.nodes, ref[4]) and torch.equal(plan.keys, ref[0])
    gtc.autotune_clear()
