"""Seeded synthetic point clouds and key sets for the five benchmark workloads.

The reference draws its points from an unseeded ``rand::thread_rng()``
(radixsort-vulkan/src/init.rs:3-23: ``rng.gen::<f32>() * range + min``, w = 1).
These generators keep that shape (float[n][4], w = 1, coordinates in
[min, min + range)) but are seeded, so that the CUDA path and the oracle
consume the identical host buffer.  Uniform draws come from SplitMix64 and are
exact float32 values ``(r >> 40) * 2^-24 * range``; Gaussian draws come from
numpy's PCG64 generator.
"""
from __future__ import annotations

import math

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)

DOMAIN_MIN = 0.0
DOMAIN_RANGE = 1024.0
_TOP = np.float32(np.nextafter(np.float32(1024.0), np.float32(0.0)))


def splitmix64(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Counter-based SplitMix64 stream: element k is the (offset+k+1)-th output."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + np.arange(offset + 1, offset + count + 1, dtype=np.uint64) * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform01_f32(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Exact float32 in [0, 1): 24 random bits times 2^-24."""
    r = splitmix64(seed, count, offset) >> np.uint64(40)
    return (r.astype(np.float32) * np.float32(2.0**-24)).astype(np.float32)


def _pack(xyz: np.ndarray) -> np.ndarray:
    n = xyz.shape[0]
    pts = np.empty((n, 4), np.float32)
    pts[:, :3] = xyz
    pts[:, 3] = 1.0
    return pts


def uniform_points(n: int, seed: int = 0, min_coord: float = DOMAIN_MIN, rng: float = DOMAIN_RANGE) -> np.ndarray:
    """n points i.i.d. uniform in [min, min + range)^3 (w = 1)."""
    u = uniform01_f32(seed, 3 * n).reshape(n, 3)
    xyz = u * np.float32(rng) + np.float32(min_coord)
    return _pack(xyz.astype(np.float32))


def _clamp(xyz: np.ndarray) -> np.ndarray:
    # The reference maps exactly range to cell 0 (quantised value 2^B wraps),
    # so points are clamped strictly below the top of the domain.
    return np.clip(xyz, np.float32(0.0), _TOP).astype(np.float32)


def gaussian_mixture_points(n: int, n_comp: int, sigma, weights=None, noise: float = 0.0, seed: int = 0,
                            centres=None, chunk: int = 1 << 22) -> np.ndarray:
    """Isotropic Gaussian mixture in [0, 1024)^3 plus a uniform-noise fraction.

    sigma is a scalar or one value per component (in domain units)."""
    g = np.random.Generator(np.random.PCG64(seed))
    if centres is None:
        centres = g.random((n_comp, 3)) * DOMAIN_RANGE
    sig = np.broadcast_to(np.asarray(sigma, np.float64), (n_comp,))
    w = np.full(n_comp, 1.0 / n_comp) if weights is None else np.asarray(weights, np.float64)
    w = w / w.sum()
    out = np.empty((n, 3), np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        k = e - s
        comp = g.choice(n_comp, size=k, p=w)
        xyz = centres[comp] + g.standard_normal((k, 3)) * sig[comp, None]
        is_noise = g.random(k) < noise
        xyz[is_noise] = g.random((int(is_noise.sum()), 3)) * DOMAIN_RANGE
        out[s:e] = _clamp(xyz.astype(np.float32))
    return _pack(out)


# ---------------------------------------------------------------- configs --

def config1_points(n: int = 1 << 20, seed: int = 0) -> np.ndarray:
    """Plain pipeline, CPU-runnable: 2^20 uniform points in [0,1024)^3, seed 0."""
    return uniform_points(n, seed)


def config2_points(n: int = 10_000_000, seed: int = 0) -> np.ndarray:
    """Plain pipeline, clustered: 32 equal-weight components, sigma = 0.5% of
    the domain, 2% uniform noise, clamped to the domain."""
    return gaussian_mixture_points(n, 32, 0.005 * DOMAIN_RANGE, noise=0.02, seed=seed)


def config3_keys(n: int, key_bits: int, and_words: int = 0, seed: int = 0) -> np.ndarray:
    """Sort sweep keys: uniform (and_words = 0) or the AND of 1..4 independent
    uniform words (bit density 2^-and_words)."""
    words = max(and_words, 1)
    off = 0
    k = None
    for _ in range(words):
        r = splitmix64(seed * 7919 + key_bits, n, off)
        off += n
        k = r if k is None else (k & r)
    if key_bits == 32:
        return (k >> np.uint64(32)).astype(np.uint32)
    return k.astype(np.uint64)


def config4_clouds(n_clouds: int = 512, seed: int = 0, lo: int = 1000, hi: int = 1_000_000):
    """Batched: n_clouds clouds with log-uniform sizes in [lo, hi]; even clouds
    uniform, odd clouds an 8-component Gaussian mixture (sigma 1% of domain).
    Returns (points float[N][4], offsets uint32[n_clouds + 1])."""
    u = uniform01_f32(seed + 101, n_clouds).astype(np.float64)
    sizes = np.floor(np.exp(math.log(lo) + u * (math.log(hi) - math.log(lo)))).astype(np.int64)
    sizes = np.clip(sizes, lo, hi)
    offsets = np.zeros(n_clouds + 1, np.int64)
    offsets[1:] = np.cumsum(sizes)
    pts = np.empty((int(offsets[-1]), 4), np.float32)
    for c in range(n_clouds):
        s, e = int(offsets[c]), int(offsets[c + 1])
        if c % 2 == 0:
            pts[s:e] = uniform_points(e - s, seed=seed * 1000003 + c)
        else:
            pts[s:e] = gaussian_mixture_points(e - s, 8, 0.01 * DOMAIN_RANGE, seed=seed * 1000003 + c)
    return pts, offsets.astype(np.uint32)


def config5_points(n: int = 64 << 20, seed: int = 0, shifted: bool = False) -> np.ndarray:
    """Learned-bucket workload: 64 components, sigma in U[0.3%, 3%] of the
    domain, Dirichlet(1) weights, 5% uniform noise.  shifted=True moves every
    centre by a seeded offset (the input that must fail the learned model's
    checks and take the onesweep path).  The mixture itself is fixed; seed
    only changes the sample, so a prior run (another seed) draws from the same
    distribution."""
    g = np.random.Generator(np.random.PCG64(10_000))
    centres = g.random((64, 3)) * DOMAIN_RANGE
    sig = g.uniform(0.003, 0.03, 64) * DOMAIN_RANGE
    w = g.exponential(1.0, 64)
    if shifted:
        centres = np.mod(centres + g.uniform(150.0, 350.0, (64, 3)), DOMAIN_RANGE)
    return gaussian_mixture_points(n, 64, sig, weights=w, noise=0.05, seed=20_000 + seed, centres=centres)
