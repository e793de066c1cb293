"""The bounded device waits run out, report and leave the context usable.

gtc_debug_skip_first_tile makes the next sort hand out its last pass's tile
tickets from 1, so that pass's tile 0 never runs and never publishes its
digit counts:
every look-back that reaches it (spin_descriptor in the production onesweep
kernel) polls its budget, records GTC_ERR_TIMEOUT in the status word and
returns.  With a budget of 1,000 polls (gtc_set_spin_limit) that takes
milliseconds.  Nothing faults and nothing hangs: the waits are bounded by
construction, and the sort writes only in-bounds positions (a tile's writes
for a digit stay inside that digit's range of the global histogram; a
timed-out look-back only lowers its offset within it).  Afterwards the
default budget is restored and the same context sorts exactly."""
import numpy as np
import pytest

from gtc import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("key_bits", [32, 64])
def test_lookback_timeout_is_reported_and_recovered(ctx, gtc_mod, key_bits):
    import torch

    n = 1 << 20
    keys_np = W.config3_keys(n, key_bits, seed=12)
    kd = np.int32 if key_bits == 32 else np.int64
    src = torch.from_numpy(keys_np.view(kd)).cuda()
    ctx.device_status()  # start from a clean status word
    ctx.set_spin_limit(1000)
    try:
        ctx.debug_skip_first_tile()
        k = src.clone()
        v = torch.arange(n, dtype=torch.int32, device="cuda")
        ctx.sort_pairs(k, v)
        with pytest.raises(gtc_mod.GtcError) as ei:
            ctx.device_status()
        assert ei.value.status == 4  # GTC_ERR_TIMEOUT
    finally:
        ctx.set_spin_limit(0)
    assert ctx.device_status() == 0  # the status word was cleared by the read
    k = src.clone()
    v = torch.arange(n, dtype=torch.int32, device="cuda")
    ctx.sort_pairs(k, v)
    assert ctx.device_status() == 0
    order = np.argsort(keys_np, kind="stable")
    assert np.array_equal(k.cpu().numpy().view(keys_np.dtype), keys_np[order])
    assert np.array_equal(v.cpu().numpy().view(np.uint32), order.astype(np.uint32))


def test_short_budget_without_a_lost_tile_still_sorts(ctx):
    """A budget of 10^5 polls is far above what a healthy look-back needs."""
    import torch

    n = 1 << 22
    keys_np = W.config3_keys(n, 32, seed=13)
    k = torch.from_numpy(keys_np.view(np.int32)).cuda()
    ctx.set_spin_limit(100_000)
    try:
        ctx.sort_pairs(k, None)
        assert ctx.device_status() == 0
    finally:
        ctx.set_spin_limit(0)
    assert np.array_equal(k.cpu().numpy().view(np.uint32), np.sort(keys_np))
