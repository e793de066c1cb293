"""The onesweep autotuner's cache (tune.cu): record / lookup per (key width,
bits, ceil(log2 n)), text persistence, and the GTC_TUNE_CACHE file loaded on
first use.  Host logic only; the timing itself is in test_gpu_autotune.py."""
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture()
def clean(gtc_mod):
    gtc_mod.autotune_clear()
    yield gtc_mod
    gtc_mod.autotune_clear()


def test_record_and_lookup_by_size_bucket(clean):
    g = clean
    L = g.lib()
    assert g.autotune_lookup(64, 63, 10_000_000) == -1
    assert L.gtc_autotune_record(64, 63, 10_000_000, 2, 0.61) == 0
    # ceil(log2 n) buckets: 2^23 < n <= 2^24 share the entry
    assert g.autotune_lookup(64, 63, (1 << 23) + 1) == 2
    assert g.autotune_lookup(64, 63, 1 << 24) == 2
    assert g.autotune_lookup(64, 63, 1 << 23) == -1
    assert g.autotune_lookup(64, 64, 10_000_000) == -1  # another bit count
    assert g.autotune_lookup(32, 63, 10_000_000) == -1  # another key width
    assert L.gtc_autotune_entries() == 1


def test_record_rejects_bad_entries(clean):
    L = clean.lib()
    nv = L.gtc_sort_num_variants()
    assert L.gtc_autotune_record(48, 30, 100, 0, 1.0) == 1
    assert L.gtc_autotune_record(32, 33, 100, 0, 1.0) == 1
    assert L.gtc_autotune_record(32, 30, 100, nv, 1.0) == 1
    assert L.gtc_autotune_record(32, 30, 100, -1, 1.0) == 1
    assert L.gtc_autotune_entries() == 0


def test_save_load_roundtrip_and_malformed_lines(clean, tmp_path):
    g = clean
    L = g.lib()
    assert L.gtc_autotune_record(32, 30, 1 << 20, 1, 0.2) == 0
    assert L.gtc_autotune_record(64, 63, 10_000_000, 2, 0.6) == 0
    path = str(tmp_path / "tune.txt")
    g.autotune_save(path)
    g.autotune_clear()
    assert L.gtc_autotune_entries() == 0
    with open(path, "a") as f:
        f.write("garbage line\nsort 64 63 25 999 1.0\nsort 16 8 3 0 1.0\n")  # ignored
    g.autotune_load(path)
    assert L.gtc_autotune_entries() == 2
    assert g.autotune_lookup(32, 30, 1 << 20) == 1
    assert g.autotune_lookup(64, 63, 10_000_000) == 2
    with pytest.raises(g.GtcError):
        g.autotune_load(str(tmp_path / "missing.txt"))


def test_env_cache_file_is_loaded_on_first_use(tmp_path):
    path = tmp_path / "env_tune.txt"
    path.write_text("sort 64 63 24 3 0.5\n")
    code = ("import sys; sys.path.insert(0, %r); import gtc; "
            "print(gtc.autotune_lookup(64, 63, 10_000_000))" % os.path.join(REPO, "glsl-tree-construction_gb300"))
    env = dict(os.environ, GTC_TUNE_CACHE=str(path))
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "3"


def test_batched_entries_load_save_and_pin(clean, tmp_path):
    """Batched onesweep shapes share the cache file as "batched <log2n>
    <variant> <ms>" lines; a pinned variant overrides the tuned one, and out
    of range variants are refused.  Host logic only (no build runs)."""
    g = clean
    L = g.lib()
    nv = L.gtc_batched_num_variants()
    assert nv >= 2 and len(g.batched_variants()) == nv
    assert g.batched_variants()[0] == (512, 12)
    path = tmp_path / "tune.txt"
    path.write_text(f"batched 27 1 5.5\nbatched 27 {nv} 1.0\nbatched 40 0 1.0\n")  # the last two are ignored
    g.autotune_load(str(path))
    assert L.gtc_autotune_entries() == 1
    n = 83_487_470  # ceil(log2 n) = 27
    assert g.autotune_lookup_batched(n) == 1 and g.batched_get_variant(n) == 1
    assert g.autotune_lookup_batched(1 << 20) == -1 and g.batched_get_variant(1 << 20) == 0
    g.batched_set_variant(nv - 1)
    try:
        assert g.batched_get_variant(n) == nv - 1
    finally:
        g.batched_set_variant(-1)
    assert g.batched_get_variant(n) == 1
    with pytest.raises(g.GtcError):
        g.batched_set_variant(nv)
    out = str(tmp_path / "saved.txt")
    g.autotune_save(out)
    assert "batched 27 1 " in open(out).read()


def test_learned_entries_load_and_pin(clean, tmp_path):
    """Learned grouping-pass shapes: "learned <log2n> <variant> <ms>" lines,
    the pin overriding the tuned pick, range checks.  Host logic only."""
    g = clean
    L = g.lib()
    nv = L.gtc_learned_num_variants()
    assert nv >= 2 and g.learned_variants()[0] == (256, 16)
    path = tmp_path / "tune.txt"
    path.write_text(f"learned 26 2 3.1\nlearned 26 {nv} 1.0\n")
    g.autotune_load(str(path))
    assert L.gtc_autotune_entries() == 1
    assert g.autotune_lookup_learned(1 << 26) == 2 and g.learned_get_variant(1 << 26) == 2
    assert g.learned_get_variant(1 << 20) == 0
    g.learned_set_variant(1)
    try:
        assert g.learned_get_variant(1 << 26) == 1
    finally:
        g.learned_set_variant(-1)
    with pytest.raises(g.GtcError):
        g.learned_set_variant(nv)


def test_sort_entries_carry_the_digit_width(clean, tmp_path):
    """Sort entries carry the tuned digit width as a sixth field (absent: 8
    bits).  A width whose passes do not fit the bit range (6-bit digits over
    64 bits would need 11 passes) is refused on load; a pinned width overrides
    the tuned one only where it fits."""
    g = clean
    L = g.lib()
    path = tmp_path / "tune.txt"
    path.write_text("sort 32 32 24 16 0.43 7\nsort 64 40 24 0 0.40\nsort 64 64 24 2 1.0 6\n")
    g.autotune_load(str(path))
    assert L.gtc_autotune_entries() == 2
    assert g.autotune_lookup_digit_bits(32, 32, 1 << 24) == 7 and g.autotune_lookup(32, 32, 1 << 24) == 16
    assert g.autotune_lookup_digit_bits(64, 40, 1 << 24) == 8
    assert g.autotune_lookup_digit_bits(64, 64, 1 << 24) == -1
    assert L.gtc_sort_get_digit_bits(32, 32, 1 << 24) == 7
    assert L.gtc_sort_get_digit_bits(64, 64, 1 << 24) == 8
    assert L.gtc_sort_set_digit_bits(64, 6) == 0
    try:
        assert L.gtc_sort_get_digit_bits(64, 40, 1 << 24) == 6   # 7 passes: fits
        assert L.gtc_sort_get_digit_bits(64, 64, 1 << 24) == 8   # 11 passes: does not
    finally:
        L.gtc_sort_set_digit_bits(64, -1)
    assert L.gtc_sort_set_digit_bits(32, 5) != 0 and L.gtc_sort_set_digit_bits(32, 9) != 0
    out = str(tmp_path / "saved.txt")
    g.autotune_save(out)
    assert "sort 32 32 24 16 0.430000 7" in open(out).read()
