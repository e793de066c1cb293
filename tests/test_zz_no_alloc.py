"""gtc_sort_pairs_u32_noalloc: the sort for callers that cannot allocate
device memory where they sort (the allocator synchronises the device, or
their own allocator owns it).  It keeps its scratch in a fixed array inside
the library; this checks, through the C ABI, that two calls in a row give
exactly what the workspace-taking gtc_sort_pairs_u32 gives, and that sizes
beyond the array's limit are refused.

Collected last on purpose: a failure here stops a `-x` run only after every
other test has run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 4_194_304


def _ref_sort(ctx, keys, vals, torch):
    """The existing entry point, with a caller-owned workspace."""
    import gtc

    k, v = keys.clone(), vals.clone()
    ka, va = torch.empty_like(k), torch.empty_like(v)
    ws = ctx.workspace(gtc.OP_SORT_PAIRS, k.numel(), 32)
    s = ctx.L.gtc_sort_pairs_u32(ctx.h, k.data_ptr(), v.data_ptr(), ka.data_ptr(), va.data_ptr(), k.numel(), 0, 32,
                                 ws.data_ptr(), ws.numel(), torch.cuda.current_stream().cuda_stream)
    ctx.check(s)
    return k, v


def _noalloc_sort(ctx, keys, vals, torch, begin=0, end=32):
    k, v = keys.clone(), vals.clone()
    ka, va = torch.empty_like(k), torch.empty_like(v)
    s = ctx.L.gtc_sort_pairs_u32_noalloc(ctx.h, k.data_ptr(), v.data_ptr(), ka.data_ptr(), va.data_ptr(),
                                         k.numel(), begin, end, torch.cuda.current_stream().cuda_stream)
    ctx.check(s)
    return k, v


def test_noalloc_sort_matches_workspace_sort_twice(ctx):
    import torch

    rng = np.random.default_rng(2024)
    # Two calls in a row; the second is smaller, so stale scratch from the
    # first call would show up as wrong output.
    for n, hi in ((MAX_KEYS - 3, 1 << 32), (1_000_003, 1 << 12)):
        keys = torch.from_numpy(rng.integers(0, hi, size=n, dtype=np.uint64).astype(np.uint32).view(np.int32)).cuda()
        vals = torch.arange(n, dtype=torch.int32, device="cuda")
        rk, rv = _ref_sort(ctx, keys, vals, torch)
        nk, nv = _noalloc_sort(ctx, keys, vals, torch)
        ctx.device_status()
        assert torch.equal(nk, rk) and torch.equal(nv, rv)
        host = keys.cpu().numpy().view(np.uint32)
        order = np.argsort(host, kind="stable")
        assert np.array_equal(nv.cpu().numpy().view(np.uint32), order.astype(np.uint32))


def test_noalloc_sort_bit_range_and_limit(ctx):
    import torch

    n = 123_457
    keys = torch.randint(-(1 << 31), (1 << 31) - 1, (n,), dtype=torch.int32, device="cuda")
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    nk, nv = _noalloc_sort(ctx, keys, vals, torch, 3, 30)
    host = keys.cpu().numpy().view(np.uint32)
    order = np.argsort((host >> 3) & ((1 << 27) - 1), kind="stable")
    assert np.array_equal(nv.cpu().numpy().view(np.uint32), order.astype(np.uint32))
    # beyond the static scratch: refused with GTC_ERR_INVALID_ARG, nothing launched
    s = ctx.L.gtc_sort_pairs_u32_noalloc(ctx.h, keys.data_ptr(), vals.data_ptr(), keys.data_ptr(), vals.data_ptr(),
                                         MAX_KEYS + 1, 0, 32, None)
    assert s == 1
    assert b"limit" in ctx.L.gtc_last_error(ctx.h)
