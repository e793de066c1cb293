"""Learned-bucket sort (gtc_learned_*): GPU training gradients against the
oracle, output bit-exact against the stable sort, fallback on a shifted
distribution, and what training gains: the same model before training is
equal-width bucketing of the key range."""
import numpy as np
import pytest

from gtc import workloads as W

pytestmark = pytest.mark.gpu


def _keys(oracle, n, seed, shifted=False):
    return oracle.morton(W.config5_points(n, seed=seed, shifted=shifted), 64)


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()


def _trained(ctx, oracle, gtc_mod, n_prior=2_000_000, buckets=1024, iters=600):
    prior = np.sort(_keys(oracle, n_prior, seed=1))
    model = gtc_mod.LearnedModel(ctx, buckets)
    model.train(_dev(prior), stride=100, iters=iters)
    return model, prior


def test_gradient_matches_oracle(ctx, oracle, gtc_mod):
    prior = np.sort(_keys(oracle, 1_000_000, seed=1))
    model = gtc_mod.LearnedModel(ctx, 512)
    sample = prior[::100]
    for init in (True, False):
        g, loss = model.gradient(_dev(prior), stride=100, init=init)
        kn, hy = model.params()
        eloss, eg = oracle.pwl_loss_grad(sample, kn, hy)
        got = g.cpu().numpy().astype(np.float64)
        scale = np.abs(eg).max()
        assert np.allclose(got, eg, rtol=2e-3, atol=2e-3 * scale), (init, np.abs(got - eg).max(), scale)
        assert abs(loss - eloss) <= 1e-3 * max(eloss, 1e-12) + 1e-9
        if init:
            model.train(_dev(prior), stride=100, iters=20)


def test_training_reduces_loss_and_keeps_monotone(ctx, oracle, gtc_mod):
    prior = np.sort(_keys(oracle, 1_000_000, seed=1))
    model = gtc_mod.LearnedModel(ctx, 512)
    _, loss0 = model.gradient(_dev(prior), stride=100, init=True)
    loss1 = model.train(_dev(prior), stride=100, iters=200)
    assert loss1 < loss0
    kn, hy = model.params()
    assert np.all(np.diff(hy) >= 0) and hy[0] == 0 and hy[-1] == 1
    assert np.all(np.diff(kn.astype(np.float64)) >= 0)


@pytest.mark.parametrize("buckets", [1024, 16384])
def test_buckets_match_oracle(ctx, oracle, gtc_mod, buckets):
    """The GPU bucket line and the oracle's agree key for key (both FP32,
    operation for operation)."""
    model, _ = _trained(ctx, oracle, gtc_mod, n_prior=4_000_000, buckets=buckets, iters=200)
    keys = _keys(oracle, 1_000_000, seed=2)
    kn, hy = model.params()
    exp = np.bincount(oracle.pwl_buckets(keys, kn, hy), minlength=buckets)
    got = model.histogram(_dev(keys)).cpu().numpy()
    assert np.array_equal(got.astype(np.int64), exp)


@pytest.mark.parametrize("n", [1, 1000, 777_777, 4_000_000])
def test_learned_sort_bit_exact(ctx, oracle, gtc_mod, n):
    model, _ = _trained(ctx, oracle, gtc_mod, buckets=1024 if n < 4_000_000 else 4096)
    keys = _keys(oracle, n, seed=2)
    vals = np.arange(n, dtype=np.uint32)[::-1].copy()  # a payload that is not the index
    import torch

    tv = torch.from_numpy(vals.view(np.int32)).cuda()
    ko, vo, flags = model.sort(_dev(keys), tv)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(ko.cpu().numpy().view(np.uint64), keys[order])
    assert np.array_equal(vo.cpu().numpy().view(np.uint32), vals[order])
    ctx.device_status()
    if n >= 1000:
        assert int(flags.item()) == 0, gtc_mod.LEARNED_FLAGS


def test_learned_matches_onesweep(ctx, oracle, gtc_mod):
    import torch

    model, _ = _trained(ctx, oracle, gtc_mod, buckets=4096)
    keys = _dev(_keys(oracle, 6_000_000, seed=3))
    ko, vo, flags = model.sort(keys)
    k2, v2 = keys.clone(), torch.arange(keys.numel(), dtype=torch.int32, device="cuda")
    ctx.sort_pairs(k2, v2, 0, 64)
    assert int(flags.item()) == 0
    assert torch.equal(ko, k2) and torch.equal(vo, v2)


def test_shifted_distribution_falls_back(ctx, oracle, gtc_mod):
    model, _ = _trained(ctx, oracle, gtc_mod, buckets=1024)
    keys = _keys(oracle, 3_000_000, seed=4, shifted=True)
    ko, vo, flags = model.sort(_dev(keys))
    assert int(flags.item()) & 1  # overflow: the model does not fit the shifted mixture
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(ko.cpu().numpy().view(np.uint64), keys[order])
    assert np.array_equal(vo.cpu().numpy().view(np.uint32), order.astype(np.uint32))


def test_duplicates_and_equal_keys(ctx, oracle, gtc_mod):
    model, _ = _trained(ctx, oracle, gtc_mod, buckets=1024)
    base = _keys(oracle, 200_000, seed=5)
    rng = np.random.default_rng(0)
    dup = np.concatenate([base, base[rng.integers(0, base.size, 50_000)]])  # short runs of equal keys
    rng.shuffle(dup)
    same = np.full(100_000, base[17], np.uint64)  # one long run: falls back, still exact
    for keys, must_fall_back in ((dup, False), (same, True)):
        ko, vo, flags = model.sort(_dev(keys))
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(ko.cpu().numpy().view(np.uint64), keys[order])
        assert np.array_equal(vo.cpu().numpy().view(np.uint32), order.astype(np.uint32))
        assert (int(flags.item()) != 0) == must_fall_back


def test_wrapped_bucket_counter(ctx, oracle, gtc_mod):
    """The count kernel keeps 16-bit per-CTA counters.  12M copies of one
    key put about 79K keys of one bucket into every CTA: the counter wraps.
    The histogram entry point must still be exact (the CTA counts again) and
    the sort must flag the overflow and come out exact through the fallback."""
    model, _ = _trained(ctx, oracle, gtc_mod, buckets=1024)
    base = _keys(oracle, 500_000, seed=6)
    keys = np.concatenate([np.full(12_000_000, base[3], np.uint64), base])
    np.random.default_rng(1).shuffle(keys)
    kn, hy = model.params()
    exp = np.bincount(oracle.pwl_buckets(keys, kn, hy), minlength=1024)
    got = model.histogram(_dev(keys)).cpu().numpy()
    assert np.array_equal(got.astype(np.int64), exp)
    ko, vo, flags = model.sort(_dev(keys))
    assert int(flags.item()) & 1
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(ko.cpu().numpy().view(np.uint64), keys[order])
    assert np.array_equal(vo.cpu().numpy().view(np.uint32), order.astype(np.uint32))


def test_training_gain_over_the_untrained_model(ctx, oracle, gtc_mod):
    """What training gains, on the learned workload's keys (64-component
    mixture, 8M keys, 2^11 buckets; the model fitted to a 1% sample of a prior
    run's sorted keys).  Before training the heights are the key-space uniform
    CDF, i.e. equal-width buckets of the key range: clustered Morton codes pile
    into a few buckets, the largest far above the on-chip capacity, and the
    sort falls back to the plain onesweep.  After training the largest bucket
    stays within 2.5x the mean, nothing falls back, and both outputs are
    byte-equal to the stable onesweep."""
    import torch

    n, B = 8_000_000, 2048
    prior = _dev(np.sort(_keys(oracle, n, seed=1)))
    keys = _dev(_keys(oracle, n, seed=2))
    model = gtc_mod.LearnedModel(ctx, B)
    model.gradient(prior, stride=100, init=True)  # knots fitted, heights untrained
    untrained = model.histogram(keys).cpu().numpy()
    ko0, vo0, f0 = model.sort(keys)
    model.train(prior, stride=100)
    trained = model.histogram(keys).cpu().numpy()
    ko1, vo1, f1 = model.sort(keys)
    mean = n / B
    assert untrained.max() / mean > 20.0
    assert trained.max() / mean < 2.5
    assert int(f0.item()) & 1 and int(f1.item()) == 0
    k2, v2 = keys.clone(), torch.arange(n, dtype=torch.int32, device="cuda")
    ctx.sort_pairs(k2, v2, 0, 64)
    assert torch.equal(ko0, k2) and torch.equal(vo0, v2)
    assert torch.equal(ko1, k2) and torch.equal(vo1, v2)


def test_config5_full_64m(ctx, gtc_mod):
    """The learned-bucket workload at its stated size: 2^26 (64M) u64 Morton
    keys of the 64-component mixture (sigma 0.3-3% of the domain, Dirichlet(1)
    weights, 5% noise).  The model is trained on a 1% sample of a prior run's
    sorted keys (the same mixture, another seed).  The output must be
    byte-equal to the plain onesweep (gtc_sort_pairs_u64, stable, all 64
    bits) without the fallback; the shifted mixture must set the fallback
    flag and still come out byte-equal."""
    import torch

    n = 1 << 26

    def keys_of(seed, shifted=False):
        pts = torch.from_numpy(W.config5_points(n, seed=seed, shifted=shifted)).cuda()
        k, _ = ctx.morton(pts, 64, with_idx=False)
        del pts
        return k

    prior = keys_of(1)
    ctx.sort_pairs(prior, None, 0, 64)
    B = gtc_mod.learned_buckets_for(n)
    model = gtc_mod.LearnedModel(ctx, B)
    model.train(prior, stride=100)
    del prior
    for seed, shifted in ((2, False), (3, True)):
        keys = keys_of(seed, shifted)
        ko, vo, flags = model.sort(keys)
        k2, v2 = keys.clone(), torch.arange(n, dtype=torch.int32, device="cuda")
        ctx.sort_pairs(k2, v2, 0, 64)
        fl = int(flags.item())
        assert (fl != 0) == shifted, (shifted, fl, gtc_mod.LEARNED_FLAGS)
        assert torch.equal(ko, k2) and torch.equal(vo, v2)
        ctx.device_status()
        del keys, ko, vo, k2, v2
    model.close()


def test_every_learned_variant_identical_and_tuned(ctx, oracle, gtc_mod):
    """Every grouping-pass shape gives byte-identical learned sorts (equal to
    the stable onesweep); the autotuner times them all and an unpinned sort
    then uses its pick."""
    import torch

    gtc_mod.autotune_clear()
    model, _ = _trained(ctx, oracle, gtc_mod, buckets=4096)
    keys = _dev(_keys(oracle, 3_000_000, seed=6))
    n = keys.numel()
    k2, v2 = keys.clone(), torch.arange(n, dtype=torch.int32, device="cuda")
    ctx.sort_pairs(k2, v2, 0, 64)
    try:
        for v in range(len(gtc_mod.learned_variants())):
            gtc_mod.learned_set_variant(v)
            ko, vo, flags = model.sort(keys)
            assert int(flags.item()) == 0, v
            assert torch.equal(ko, k2) and torch.equal(vo, v2), v
    finally:
        gtc_mod.learned_set_variant(-1)
    r = model.autotune(keys, reps=2)
    assert len(r["ms"]) == len(gtc_mod.learned_variants()) and all(0 < t < 1e4 for t in r["ms"])
    assert gtc_mod.autotune_lookup_learned(n) == r["best"] == gtc_mod.learned_get_variant(n)
    ko, vo, flags = model.sort(keys)
    assert torch.equal(ko, k2) and torch.equal(vo, v2)
    gtc_mod.autotune_clear()
