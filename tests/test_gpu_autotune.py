"""The autotuner on the GPU: every variant is timed, the fastest is cached
for the shape, and sorts that pick it up stay bit-exact."""
import math

import numpy as np
import pytest

from gtc import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture()
def tuned(ctx, gtc_mod):
    gtc_mod.autotune_clear()
    yield ctx
    gtc_mod.autotune_clear()


def test_autotune_uniform_u32(tuned, gtc_mod):
    import torch

    ctx = tuned
    n = 1 << 20
    r = ctx.autotune_sort(32, n, 0, 30, reps=2)
    nv = len(ctx.sort_variants())
    assert 0 <= r["best"] < nv
    assert all(0.0 < t < 1e3 and math.isfinite(t) for t in r["ms"])
    assert r["ms"][r["best"]] == min(r["ms"])
    assert gtc_mod.autotune_lookup(32, 30, n) == r["best"]
    keys = (W.config3_keys(n, 32, seed=3) >> np.uint32(2)).astype(np.uint32)
    k, v = ctx.sort_pairs(torch.from_numpy(keys.view(np.int32)).cuda(),
                          torch.arange(n, dtype=torch.int32, device="cuda"), 0, 30)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k.cpu().numpy().view(np.uint32), keys[order])
    assert np.array_equal(v.cpu().numpy().view(np.uint32), order.astype(np.uint32))
    ctx.device_status()


def test_autotune_on_callers_morton_keys_feeds_the_pipeline(tuned, gtc_mod, oracle):
    """Tuning on the workload's own 64-bit Morton codes caches a variant for
    the pipeline's sort shape (63 bits); the octree build then runs with it
    and still matches the oracle."""
    import torch

    pts = W.gaussian_mixture_points(1_500_000, 16, 4.0, noise=0.02, seed=21)
    tp = torch.from_numpy(pts).cuda()
    codes, _ = ctx_morton(tuned, tp)
    r = tuned.autotune_sort(64, pts.shape[0], 0, 63, keys=codes, reps=2)
    assert gtc_mod.autotune_lookup(64, 63, pts.shape[0]) == r["best"]
    res = gtc_mod.build_octree(tuned, tp, 64)
    exp, _ = oracle.build_octree(pts, 64, threads=8)
    assert res.n_oct_nodes == exp["n_oct_nodes"]
    assert np.array_equal(res.keys.cpu().numpy().view(np.uint64), exp["keys"])
    assert np.array_equal(gtc_mod.nodes_to_numpy(res.nodes).view(np.int32), exp["nodes"].view(np.int32))


def ctx_morton(ctx, tp):
    return ctx.morton(tp, 64, with_idx=False)


def test_pinned_variant_overrides_the_tuned_one(tuned, gtc_mod):
    ctx = tuned
    assert gtc_mod.lib().gtc_autotune_record(32, 32, 4096, 1, 0.01) == 0
    ctx.set_sort_variant(32, 2)
    try:
        assert ctx.get_sort_variant(32) == 2
    finally:
        ctx.set_sort_variant(32, -1)
    assert gtc_mod.autotune_lookup(32, 32, 4096) == 1
