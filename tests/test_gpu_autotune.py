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


def test_every_digit_width_sorts_stably(ctx):
    """The sort at 6-, 7- and 8-bit digits (pinned), over full 32-bit keys and
    64-bit keys' low 48 bits and the pipeline's bits 23..62, on uniform and
    low-entropy keys: the same stable order as numpy.  A width that does not
    fit a 64-bit key's full range in 8 passes is ignored, and that sort stays
    exact."""
    import torch

    try:
        for db in (6, 7, 8):
            for kb, lo, hi in ((32, 0, 32), (64, 0, 48), (64, 23, 63), (64, 0, 64)):
                ctx.set_sort_digit_bits(kb, db)
                bits = hi - lo
                exp_db = db if (bits + db - 1) // db <= 8 else 8
                assert ctx.get_sort_digit_bits(kb, bits, 1 << 20) == exp_db
                for words in (0, 2):
                    n = 700_001
                    keys = W.config3_keys(n, kb, and_words=words, seed=db * 7 + words)
                    kd = np.int32 if kb == 32 else np.int64
                    if hi - lo < kb:  # keep only the sorted range's bits
                        keys = keys & ((np.uint64(1) << np.uint64(hi)) - np.uint64(1)).astype(keys.dtype)
                    order = np.argsort(keys >> keys.dtype.type(lo), kind="stable")
                    tk = torch.from_numpy(keys.view(kd)).cuda()
                    tv = torch.arange(n, dtype=torch.int32, device="cuda")
                    k, v = ctx.sort_pairs(tk, tv, lo, hi)
                    assert np.array_equal(v.cpu().numpy().view(np.uint32), order.astype(np.uint32)), (db, kb, lo, hi)
                    assert np.array_equal(k.cpu().numpy().view(keys.dtype), keys[order]), (db, kb, lo, hi)
    finally:
        ctx.set_sort_digit_bits(32, -1)
        ctx.set_sort_digit_bits(64, -1)


def test_tuner_times_digit_widths(ctx, gtc_mod):
    """The tuner times the best variant at 6 and 7 bits too (where they fit),
    caches the fastest width, and the sort of that shape then uses it."""
    import torch

    gtc_mod.autotune_clear()
    n = 1 << 20
    keys = torch.from_numpy(W.config3_keys(n, 32, seed=3).view(np.int32)).cuda()
    r = ctx.autotune_sort(32, n, 0, 32, keys=keys, reps=2)
    assert set(r["digit_ms"]) == {6, 7, 8} and all(t is not None and t > 0 for t in r["digit_ms"].values())
    assert r["digit_bits"] == min(r["digit_ms"], key=r["digit_ms"].get)
    assert gtc_mod.autotune_lookup_digit_bits(32, 32, n) == r["digit_bits"] == ctx.get_sort_digit_bits(32, 32, n)
    r64 = ctx.autotune_sort(64, n, 0, 64, reps=1)
    assert r64["digit_ms"][6] is None and r64["digit_ms"][7] is None and r64["digit_bits"] == 8
    gtc_mod.autotune_clear()
