"""Sort-only sweep (the sort-only configuration: n = 2^16 .. 2^28 in powers
of 4; u32 and u64 keys with u32 values = original index; keys uniform or the
AND of 1-4 independent uniform words).  Up to 2^20 keys the result is compared
with numpy's stable argsort; above that, on the device, by size-independent
properties: ascending keys, equal keys in input order, every output key equal
to the input key its payload names, and the payload a permutation."""
import numpy as np
import pytest

from gtc import workloads as W

pytestmark = pytest.mark.gpu


def _device_keys(n, key_bits, and_words, seed):
    import torch

    g = torch.Generator(device="cuda").manual_seed(seed)
    words = max(and_words, 1)
    k = None
    for _ in range(words):
        lo = torch.randint(0, 1 << 32, (n,), dtype=torch.int64, device="cuda", generator=g)
        w = lo
        if key_bits == 64:
            hi = torch.randint(0, 1 << 32, (n,), dtype=torch.int64, device="cuda", generator=g)
            w = (hi << 32) | lo
        k = w if k is None else (k & w)
    return k.to(torch.int32) if key_bits == 32 else k


def _check_properties(k_in, k_out, v_out, key_bits):
    import torch

    n = k_in.numel()
    if key_bits == 32:
        ki = k_in.to(torch.int64) & 0xFFFFFFFF
        ko = k_out.to(torch.int64) & 0xFFFFFFFF
    else:  # unsigned order as signed order: flip the top bit
        sign = torch.tensor(-(1 << 63), dtype=torch.int64, device=k_in.device)
        ki = k_in ^ sign
        ko = k_out ^ sign
    v = v_out.to(torch.int64)
    assert bool((v >= 0).all()) and bool((v < n).all())
    assert bool((ko[1:] >= ko[:-1]).all()), "keys not ascending"
    eq = ko[1:] == ko[:-1]
    assert bool((v[1:][eq] > v[:-1][eq]).all()), "equal keys out of input order"
    assert bool((ki[v] == ko).all()), "an output key differs from the input key its payload names"
    assert bool((torch.bincount(v, minlength=n) == 1).all()), "payload is not a permutation"


@pytest.mark.parametrize("key_bits", [32, 64])
@pytest.mark.parametrize("and_words", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("n", [1 << 16, 1 << 18, 1 << 20])
def test_sweep_exact(ctx, key_bits, and_words, n):
    import torch

    keys = W.config3_keys(n, key_bits, and_words, seed=n + and_words)
    kd = np.uint32 if key_bits == 32 else np.uint64
    td = torch.int32 if key_bits == 32 else torch.int64
    tk = torch.from_numpy(keys.view(np.int32 if key_bits == 32 else np.int64)).cuda()
    tv = torch.arange(n, dtype=torch.int32, device="cuda")
    ctx.sort_pairs(tk, tv)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(tk.cpu().numpy().view(kd), keys[order])
    assert np.array_equal(tv.cpu().numpy().view(np.uint32), order.astype(np.uint32))
    assert tk.dtype == td


@pytest.mark.parametrize("key_bits,n,and_words", [
    (32, 1 << 22, 0), (32, 1 << 22, 4), (64, 1 << 22, 2),
    (32, 1 << 24, 0), (32, 1 << 24, 3), (64, 1 << 24, 0), (64, 1 << 24, 1),
    (32, 1 << 26, 0), (64, 1 << 26, 0), (64, 1 << 26, 4),
    (32, 1 << 28, 0), (32, 1 << 28, 2), (64, 1 << 28, 0),
])
def test_sweep_large_properties(ctx, key_bits, n, and_words):
    import torch

    k_in = _device_keys(n, key_bits, and_words, seed=1000 + n % 977 + and_words)
    k = k_in.clone()
    v = torch.arange(n, dtype=torch.int32, device="cuda")
    ctx.sort_pairs(k, v)
    _check_properties(k_in, k, v, key_bits)
    ctx.device_status()
