"""End-to-end parity of the fused pipeline (gtc_build_octree) with the oracle:
every stage buffer and every octree node, byte for byte."""
import numpy as np
import pytest

from gtc import workloads as W

pytestmark = pytest.mark.gpu


def _cmp(res, exp, key_bits, tag=""):
    import gtc

    kd = np.uint32 if key_bits == 32 else np.uint64
    assert (res.n_unique, res.n_brt_nodes, res.n_oct_nodes) == (exp["n_unique"], exp["n_brt_nodes"],
                                                                 exp["n_oct_nodes"]), tag
    pairs = [("keys", res.keys, kd), ("idx", res.idx, np.uint32), ("prefix_n", res.prefix_n, np.uint8),
             ("has_leaf_left", res.has_leaf_left, np.uint8), ("has_leaf_right", res.has_leaf_right, np.uint8),
             ("left_child", res.left_child, np.int32), ("parent", res.parent, np.int32),
             ("edge_count", res.edge_count, np.uint32), ("node_offsets", res.node_offsets, np.uint32)]
    for name, t, dt in pairs:
        got = t.cpu().numpy().view(dt)
        assert np.array_equal(got, exp[name]), (tag, name)
    got_nodes = gtc.nodes_to_numpy(res.nodes)
    assert np.array_equal(got_nodes.view(np.int32), exp["nodes"].view(np.int32)), (tag, "nodes")


def _run(ctx, oracle, pts, key_bits, tag):
    import gtc
    import torch

    res = gtc.build_octree(ctx, torch.from_numpy(pts).cuda(), key_bits)
    exp, _ = oracle.build_octree(pts, key_bits, threads=8)
    assert exp["conflicts"] == 0
    _cmp(res, exp, key_bits, tag)
    assert oracle.validate_octree(gtc.nodes_to_numpy(res.nodes), res.n_unique) == 0


@pytest.mark.parametrize("key_bits", [32, 64])
def test_config1_uniform_2p20(ctx, oracle, key_bits):
    _run(ctx, oracle, W.config1_points(), key_bits, "config1")


def test_config2_clustered_10m(ctx, oracle):
    _run(ctx, oracle, W.config2_points(), 64, "config2")


@pytest.mark.parametrize("key_bits", [32, 64])
def test_many_duplicates_3m(ctx, oracle, key_bits):
    """3M points in a few tight clusters: most Morton codes repeat, so unique
    compacts heavily (its resident segment form runs at this size), and the
    node-offset scan sees long runs of nodes."""
    pts = W.gaussian_mixture_points(3_000_000, 4, 1.5, noise=0.01, seed=23)
    _run(ctx, oracle, pts, key_bits, "dups")


def _cube_points(cubes, per_cube, seed):
    """Points in cubes of side 2^-13 of the domain (8 low bits of each 21-bit
    axis): the 64-bit codes of one cube agree in their top 39 bits, above
    bit 24, and split into two runs of codes equal above bit 23, the bits the
    sort leaves to its run fixup.  With per_cube = 0 each cube gets 5..60
    points."""
    g = np.random.Generator(np.random.PCG64(seed))
    side = 1024.0 / (1 << 13)
    corners = np.floor(g.random((cubes, 3)) * (1 << 13)) * side
    counts = np.full(cubes, per_cube) if per_cube else g.integers(5, 61, cubes)
    xyz = np.repeat(corners, counts, axis=0) + g.random((int(counts.sum()), 3)) * side
    out = np.ones((xyz.shape[0], 4), np.float32)
    out[:, :3] = np.minimum(xyz, 1023.99).astype(np.float32)
    return out[g.permutation(out.shape[0])]


def _box_runs(lengths, seed):
    """One box of 2^8 x 2^8 x 2^7 finest cells per length (the x and y low
    8 bits and the z low 7 bits free, at distinct box positions): the 64-bit
    codes of a box agree in exactly bits 23..62, so each box is one run of
    that many distinct keys for the run fixup, in shuffled input order."""
    g = np.random.Generator(np.random.PCG64(seed))
    nb = len(lengths)
    bx = g.choice(1 << 13, nb, replace=False)
    by = g.integers(0, 1 << 13, nb)
    bz = g.integers(0, 1 << 14, nb)
    parts = []
    for b, n_box in enumerate(lengths):
        cells = g.choice(256 * 256 * 128, n_box, replace=False)
        cx = bx[b] * 256 + (cells & 255)
        cy = by[b] * 256 + ((cells >> 8) & 255)
        cz = bz[b] * 128 + (cells >> 16)
        parts.append((np.stack([cx, cy, cz], 1).astype(np.float64) + 0.5) * (1024.0 / (1 << 21)))
    xyz = np.concatenate(parts)
    out = np.ones((xyz.shape[0], 4), np.float32)
    out[:, :3] = xyz  # exact: cell centres are multiples of 2^-12 below 1024
    return out[g.permutation(out.shape[0])]


def test_run_fixup_lengths(ctx, oracle):
    """Runs of exactly the lengths where the run fixup changes path (one lane
    up to 8 keys, a warp up to 31, counting passes from 32) and around the
    2,048-key chunks its blocks own, three of each: 12 of them cross a chunk
    boundary."""
    lengths = (list(range(2, 13)) + [16, 30, 31, 32, 33, 34, 63, 64, 65, 100, 2047, 2048, 2049, 4100]) * 3
    pts = _box_runs(lengths, seed=41)
    codes = oracle.morton(pts, 64).view(np.uint64)
    high = np.sort(codes) >> np.uint64(23)
    edges = np.diff(np.concatenate(([0], (high[1:] == high[:-1]).astype(np.int8), [0])))
    runs = np.flatnonzero(edges == -1) - np.flatnonzero(edges == 1) + 1
    assert sorted(runs.tolist()) == sorted(lengths)  # the construction holds
    _run(ctx, oracle, pts, 64, "fixup_lengths")


@pytest.mark.parametrize("key_bits", [32, 64])
def test_edge_cases(ctx, oracle, key_bits):
    def p(xyz):
        xyz = np.asarray(xyz, np.float32).reshape(-1, 3)
        out = np.ones((xyz.shape[0], 4), np.float32)
        out[:, :3] = xyz
        return out

    cases = {
        "n1": p([[1.0, 2.0, 3.0]]),
        "n2": p([[1.0, 2.0, 3.0], [700.0, 2.0, 3.0]]),
        "all_equal": p([[5.5, 6.5, 7.5]] * 5000),
        # one run of a million equal codes: the run fixup's long path finds it in order
        "all_equal_1m": p(np.tile([[5.5, 6.5, 7.5]], (1 << 20, 1))),
        "corners": p([[x, y, z] for z in (10.0, 600.0) for y in (10.0, 600.0) for x in (10.0, 600.0)]),
        "boundary": p([[1024.0, 0.0, 0.0], [0.0, 1023.99, 0.0], [0.0, 0.0, 0.0], [512.0, 512.0, 512.0]]),
        "duplicates": np.repeat(W.uniform_points(3000, seed=4), 7, axis=0),
        "line": p([[float(i) * 0.25, 1.0, 1.0] for i in range(4096)]),
        "ragged": W.uniform_points(123_457, seed=8),
        "dense_cluster": W.gaussian_mixture_points(200_000, 1, 0.05, seed=6),
        # 64-bit codes that agree above bit 23 form runs the sort leaves to its
        # run fixup: two runs of about 50K keys (the long path, three counting
        # passes, across many tiles) and 4,000 runs of about 2..30 keys (lane,
        # warp and long paths at tile edges).
        "one_cell_run": _cube_points(1, 100_000, seed=31),
        "many_cell_runs": _cube_points(2_000, 0, seed=32),
    }
    for tag, pts in cases.items():
        _run(ctx, oracle, np.ascontiguousarray(pts), key_bits, tag)


def test_empty_input(ctx):
    import gtc
    import torch

    plan = gtc.OctreePlan(ctx, 16, 32)
    plan.launch(torch.zeros((0, 4), dtype=torch.float32, device="cuda"), n=0)
    assert plan.counts_host() == (0, 0, 0)


def test_graph_replay_matches_direct(ctx, oracle):
    import gtc
    import torch

    pts = W.gaussian_mixture_points(500_000, 8, 10.0, noise=0.05, seed=12)
    tp = torch.from_numpy(pts).cuda()
    plan = gtc.OctreePlan(ctx, pts.shape[0], 64)
    plan.capture(tp)
    for _ in range(3):
        plan.replay()
    torch.cuda.synchronize()
    exp, _ = oracle.build_octree(pts, 64, threads=8)
    _cmp(plan.result(), exp, 64, "graph")


def test_host_buffer_entry_point(ctx, oracle):
    import ctypes

    pts = W.config1_points(1 << 18)
    exp, _ = oracle.build_octree(pts, 32)
    nodes = np.zeros(exp["n_oct_nodes"] + 16, oracle.OCTNODE_DTYPE)
    counts = np.zeros(3, np.uint32)
    s = ctx.L.gtc_build_octree_host(ctx.h, pts.ctypes.data_as(ctypes.c_void_p), pts.shape[0], 0.0, 1024.0, 32,
                                    nodes.ctypes.data_as(ctypes.c_void_p), nodes.size,
                                    counts.ctypes.data_as(ctypes.c_void_p))
    ctx.check(s)
    assert tuple(counts) == (exp["n_unique"], exp["n_brt_nodes"], exp["n_oct_nodes"])
    assert np.array_equal(nodes[: counts[2]].view(np.int32), exp["nodes"].view(np.int32))


def test_host_entry_point_pinned_buffers(ctx, oracle):
    """Page-locked points take the direct path (the Morton pass reads them in
    host memory); same result, and a node buffer that is too small is
    reported with the counts still set."""
    import ctypes

    L = ctx.L
    pts = W.config2_points(1 << 19, seed=3)
    exp, _ = oracle.build_octree(pts, 64, threads=8)
    o = exp["n_oct_nodes"]
    hp, hn = ctypes.c_void_p(), ctypes.c_void_p()
    ctx.check(L.gtc_host_alloc(ctypes.byref(hp), pts.nbytes))
    ctx.check(L.gtc_host_alloc(ctypes.byref(hn), (o + 16) * 64))
    try:
        ctypes.memmove(hp, pts.ctypes.data, pts.nbytes)
        counts = np.zeros(3, np.uint32)
        cp = counts.ctypes.data_as(ctypes.c_void_p)
        ctx.check(L.gtc_build_octree_host(ctx.h, hp, pts.shape[0], 0.0, 1024.0, 64, hn, o + 16, cp))
        assert tuple(counts) == (exp["n_unique"], exp["n_brt_nodes"], o)
        got = np.ctypeslib.as_array((ctypes.c_int32 * (o * 16)).from_address(hn.value)).reshape(o, 16)
        assert np.array_equal(got, exp["nodes"].view(np.int32).reshape(o, 16))
        counts[:] = 0
        s = L.gtc_build_octree_host(ctx.h, hp, pts.shape[0], 0.0, 1024.0, 64, hn, o // 2, cp)
        assert s == 7  # GTC_ERR_CAPACITY
        assert int(counts[2]) == o
        ctx.device_status()  # the context stays usable
    finally:
        L.gtc_host_free(hp)
        L.gtc_host_free(hn)


def test_host_entry_point_queued(ctx, oracle):
    """Three clouds queued back to back through gtc_build_octree_host_async
    (two device buffer sets in flight, 64- and 32-bit codes), each into its
    own page-locked buffers: every one equals the oracle.  A node buffer that
    is too small is reported by the wait, with the counts set, and the
    context stays usable."""
    import ctypes

    L = ctx.L
    jobs = [(W.config2_points(1 << 19, seed=11), 64), (W.config2_points(1 << 19, seed=12), 64),
            (W.uniform_points(300_001, seed=13), 32)]
    exps = [oracle.build_octree(p, kb, threads=8)[0] for p, kb in jobs]
    bufs = []
    try:
        for (p, _), e in zip(jobs, exps):
            hp, hn, hc = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
            ctx.check(L.gtc_host_alloc(ctypes.byref(hp), p.nbytes))
            ctx.check(L.gtc_host_alloc(ctypes.byref(hn), (e["n_oct_nodes"] + 8) * 64))
            ctx.check(L.gtc_host_alloc(ctypes.byref(hc), 16))
            ctypes.memmove(hp, p.ctypes.data, p.nbytes)
            bufs.append((hp, hn, hc))
        for (hp, hn, hc), (p, kb), e in zip(bufs, jobs, exps):
            ctx.check(L.gtc_build_octree_host_async(ctx.h, hp, p.shape[0], 0.0, 1024.0, kb, hn,
                                                    e["n_oct_nodes"] + 8, hc))
        ctx.check(L.gtc_build_octree_host_wait(ctx.h))
        for (hp, hn, hc), e in zip(bufs, exps):
            c = np.ctypeslib.as_array((ctypes.c_uint32 * 3).from_address(hc.value))
            o = e["n_oct_nodes"]
            assert tuple(int(x) for x in c) == (e["n_unique"], e["n_brt_nodes"], o)
            got = np.ctypeslib.as_array((ctypes.c_int32 * (o * 16)).from_address(hn.value)).reshape(o, 16)
            assert np.array_equal(got, e["nodes"].view(np.int32).reshape(o, 16))
        hp, hn, hc = bufs[0]
        o = exps[0]["n_oct_nodes"]
        ctx.check(L.gtc_build_octree_host_async(ctx.h, hp, jobs[0][0].shape[0], 0.0, 1024.0, 64, hn, o // 2, hc))
        assert L.gtc_build_octree_host_wait(ctx.h) == 7  # GTC_ERR_CAPACITY
        c = np.ctypeslib.as_array((ctypes.c_uint32 * 3).from_address(hc.value))
        assert int(c[2]) == o
        ctx.device_status()
        # Pageable buffers are refused (GTC_ERR_INVALID_ARG) before anything is queued; counts only
        # (no node buffer) and n = 0 are accepted.
        pageable = np.ascontiguousarray(jobs[0][0])
        assert L.gtc_build_octree_host_async(ctx.h, pageable.ctypes.data_as(ctypes.c_void_p), pageable.shape[0],
                                             0.0, 1024.0, 64, hn, o + 8, hc) == 1
        ctx.check(L.gtc_build_octree_host_async(ctx.h, hp, jobs[0][0].shape[0], 0.0, 1024.0, 64, None, 0, hc))
        ctx.check(L.gtc_build_octree_host_async(ctx.h, hp, 0, 0.0, 1024.0, 64, hn, o + 8, bufs[1][2]))
        ctx.check(L.gtc_build_octree_host_wait(ctx.h))
        assert tuple(int(x) for x in c) == (exps[0]["n_unique"], exps[0]["n_brt_nodes"], o)
        c1 = np.ctypeslib.as_array((ctypes.c_uint32 * 3).from_address(bufs[1][2].value))
        assert tuple(int(x) for x in c1) == (0, 0, 0)
    finally:
        for b in bufs:
            for x in b:
                L.gtc_host_free(x)


def test_deterministic_across_runs(ctx):
    import gtc
    import torch

    pts = torch.from_numpy(W.config2_points(2_000_000, seed=5)).cuda()
    a = gtc.build_octree(ctx, pts, 64)
    b = gtc.build_octree(ctx, pts, 64)
    assert torch.equal(a.nodes, b.nodes) and torch.equal(a.keys, b.keys) and torch.equal(a.idx, b.idx)


@pytest.mark.parametrize("key_bits", [32, 64])
def test_reference_fixture(ctx, key_bits):
    """The CUDA build against the reference's own shaders' outputs
    (tests/golden/ref_pipeline_{32,64}.npz, recorded from the shader code
    compiled on the CPU, in main.rs:60-170's order), byte for byte."""
    import os

    import gtc
    import torch

    fx = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", f"ref_pipeline_{key_bits}.npz")))
    res = gtc.build_octree(ctx, torch.from_numpy(fx["pts"]).cuda(), key_bits)
    kd = np.uint32 if key_bits == 32 else np.uint64
    assert (res.n_unique, res.n_oct_nodes) == (fx["keys"].size, fx["nodes"].shape[0])
    for name, t, dt in [("keys", res.keys, kd), ("idx", res.idx, np.uint32), ("prefix_n", res.prefix_n, np.uint8),
                        ("has_leaf_left", res.has_leaf_left, np.uint8),
                        ("has_leaf_right", res.has_leaf_right, np.uint8), ("left_child", res.left_child, np.int32),
                        ("parent", res.parent, np.int32), ("edge_count", res.edge_count, np.uint32),
                        ("node_offsets", res.node_offsets, np.uint32)]:
        assert np.array_equal(t.cpu().numpy().view(dt), fx[name]), name
    assert np.array_equal(gtc.nodes_to_numpy(res.nodes).view(np.int32).reshape(-1, 16), fx["nodes"])
