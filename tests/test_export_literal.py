"""Host-side pieces of the export and literal-mode surface (no GPU): the
little-endian dump matches numpy's byte layout for every element width and
appends in order; the literal switches round-trip and reject unknown bits."""
import os

import numpy as np
import pytest


def test_export_le_every_width(gtc_mod, tmp_path):
    rng = np.random.default_rng(3)
    for dt in ("<u1", "<u2", "<u4", "<u8", "<i4", "<f4"):
        a = rng.integers(0, 200, size=1001).astype(dt)
        p = str(tmp_path / f"a_{dt[1:]}.bin")
        gtc_mod.export_le(p, a)
        assert open(p, "rb").read() == a.tobytes()


def test_export_le_append_and_empty(gtc_mod, tmp_path):
    p = str(tmp_path / "x.bin")
    a = np.arange(10, dtype=np.uint32)
    b = np.arange(100, 105, dtype=np.uint32)
    gtc_mod.export_le(p, a)
    gtc_mod.export_le(p, b, append=True)
    assert np.array_equal(np.fromfile(p, "<u4"), np.concatenate([a, b]))
    gtc_mod.export_le(p, np.zeros(0, np.uint32))
    assert os.path.getsize(p) == 0


def test_export_le_rejects_bad_arguments(gtc_mod, tmp_path):
    L = gtc_mod.lib()
    a = np.arange(4, dtype=np.uint32)
    assert L.gtc_export_le(str(tmp_path / "y.bin").encode(), a.ctypes.data, 4, 3, 0) != 0
    assert L.gtc_export_le(None, a.ctypes.data, 4, 4, 0) != 0
    assert L.gtc_export_le(str(tmp_path / "no" / "such" / "dir.bin").encode(), a.ctypes.data, 4, 4, 0) != 0


def test_literal_switches_round_trip(gtc_mod):
    assert gtc_mod.get_literal() == 0
    try:
        gtc_mod.set_literal(gtc_mod.LITERAL_D2 | gtc_mod.LITERAL_D6)
        assert gtc_mod.get_literal() == (1 << 2) | (1 << 6)
        with pytest.raises(gtc_mod.GtcError):
            gtc_mod.set_literal(1 << 1)  # D1 races on a GPU: not offered
        assert gtc_mod.get_literal() == (1 << 2) | (1 << 6)
    finally:
        gtc_mod.set_literal(0)
    assert gtc_mod.get_literal() == 0
