"""The fused build's 64-bit sort plan, checked on the CPU with numpy: stable
passes over bits 23..62 only, then each run of keys equal in those bits
sorted stably by its low 23 bits, give exactly the stable sort of the whole
key (keys and payload) that 8 full passes give.  The CUDA kernels that carry
the plan out (5 onesweep passes, run_fixup_kernel) are checked against the
oracle in tests/test_gpu_pipeline.py."""
import numpy as np
import pytest

from gtc import workloads as W

LOW = 23  # the low bits the 5 onesweep passes leave to the run fixup


def plan_sort(codes):
    """The plan: stable order by the high bits, then every run of equal high
    bits stably by its low bits.  Returns the payload (original indices)."""
    high = codes >> np.uint64(LOW)
    order = np.argsort(high, kind="stable")
    h = high[order]
    edges = np.flatnonzero(np.concatenate(([True], h[1:] != h[:-1], [True])))
    low = codes[order] & np.uint64((1 << LOW) - 1)
    for a, b in zip(edges[:-1], edges[1:]):
        if b - a > 1:
            sub = np.argsort(low[a:b], kind="stable")
            order[a:b] = order[a:b][sub]
    return order


def box_points(lengths, seed):
    """Each length is one box of finest cells whose 64-bit codes agree in
    exactly bits 23..62 (free: the low 8 bits of x and y, 7 of z)."""
    g = np.random.Generator(np.random.PCG64(seed))
    bx = g.choice(1 << 13, len(lengths), replace=False)
    parts = []
    for b, n_box in enumerate(lengths):
        cells = g.choice(256 * 256 * 128, n_box, replace=False)
        c = np.stack([bx[b] * 256 + (cells & 255), (cells >> 8) & 255, 7 * 128 + (cells >> 16)], 1)
        parts.append((c.astype(np.float64) + 0.5) * (1024.0 / (1 << 21)))
    xyz = np.concatenate(parts)
    out = np.ones((xyz.shape[0], 4), np.float32)
    out[:, :3] = xyz
    return out[g.permutation(out.shape[0])]


@pytest.mark.parametrize("case", ["clustered", "dense", "boxes", "duplicates"])
def test_plan_equals_full_stable_sort(oracle, case):
    if case == "clustered":
        pts = W.gaussian_mixture_points(400_000, 32, 5.12, noise=0.02, seed=3)
    elif case == "dense":
        pts = W.gaussian_mixture_points(100_000, 1, 0.05, seed=6)
    elif case == "boxes":
        pts = box_points([2, 3, 8, 9, 31, 32, 33, 2049, 5000], seed=7)
    else:
        pts = np.repeat(W.uniform_points(20_000, seed=4), 5, axis=0)
    codes = oracle.morton(pts, 64).view(np.uint64)
    full = np.argsort(codes, kind="stable")
    got = plan_sort(codes)
    assert np.array_equal(got, full)
    assert np.array_equal(codes[got], np.sort(codes))
