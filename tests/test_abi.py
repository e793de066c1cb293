"""The C-ABI library loads and exports every entry point include/gtc.h
declares; host-side argument checking works without a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "gtc.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"GTC_API\s+[\w\s\*]+?\b(gtc_\w+)\s*\(", text)))


def test_header_declares_the_stage_surface():
    syms = declared_symbols()
    for s in ("gtc_morton32", "gtc_morton64", "gtc_global_histogram_u32", "gtc_sort_pairs_u32", "gtc_sort_pairs_u64",
              "gtc_unique_u32", "gtc_build_radix_tree_u32", "gtc_edge_count", "gtc_partial_sum_u32",
              "gtc_make_octree_u32", "gtc_link_octree_u32", "gtc_build_octree", "gtc_build_octree_host",
              "gtc_ref_compute_morton", "gtc_ref_build_octree"):
        assert s in syms, s


def test_library_exports_every_declared_symbol(gtc_mod):
    L = gtc_mod.lib()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", gtc_mod._lib.lib_path()], capture_output=True, text=True)
    exported = set(re.findall(r"\b(gtc_\w+)$", out.stdout, re.M))
    assert set(declared_symbols()) <= exported


def test_status_strings_and_version(gtc_mod):
    L = gtc_mod.lib()
    assert L.gtc_status_string(0) == b"ok"
    assert L.gtc_status_string(4).startswith(b"a bounded")
    assert b"sm_103a" in L.gtc_version()


def test_workspace_size_without_device(gtc_mod):
    L = gtc_mod.lib()
    b = ctypes.c_size_t()
    assert L.gtc_workspace_size(None, gtc_mod.OP_SORT_PAIRS, 10_000_000, 64, ctypes.byref(b)) == 0
    tiles = -(-10_000_000 // 4096)
    assert b.value >= 8 * tiles * 256 * 4
    assert L.gtc_workspace_size(None, gtc_mod.OP_BUILD_OCTREE, 1 << 20, 32, ctypes.byref(b)) == 0
    assert b.value >= (1 << 20) * 8
    assert L.gtc_workspace_size(None, gtc_mod.OP_SORT_PAIRS, 100, 48, ctypes.byref(b)) == 1  # bad key width


def test_null_context_is_rejected(gtc_mod):
    L = gtc_mod.lib()
    assert L.gtc_morton32(None, None, None, None, 0, 0.0, 1.0, None) == 1
    assert L.gtc_sort_pairs_u32(None, None, None, None, None, 10, 0, 32, None, 0, None) == 1


@pytest.mark.skipif(os.environ.get("CUDA_VISIBLE_DEVICES", None) == "" or
                    __import__("torch").cuda.is_available(), reason="checks the no-device path")
def test_create_without_device_fails_cleanly(gtc_mod):
    L = gtc_mod.lib()
    h = ctypes.c_void_p()
    assert L.gtc_create(ctypes.byref(h), 0) == 3  # GTC_ERR_CUDA, no abort
    assert not h.value


def test_batched_workspace_and_args_without_device(gtc_mod):
    L = gtc_mod.lib()
    b = ctypes.c_size_t()
    assert L.gtc_batched_workspace_size(1_000_000, 512, ctypes.byref(b)) == 0
    tiles = -(-1_000_000 // 6144) + 512  # per-cloud tiles never exceed n / tile + clouds
    assert b.value >= 4 * tiles * 256 * 4 + 3 * 1_000_000 * 4 + 512 * 4 * 256 * 4
    assert L.gtc_batched_workspace_size(1000, 0, ctypes.byref(b)) == 1  # no clouds
    assert L.gtc_batched_workspace_size(1 << 30, 4, ctypes.byref(b)) == 1  # too many points
    assert L.gtc_batched_workspace_size(1000, (1 << 20) + 1, ctypes.byref(b)) == 1  # too many clouds
    assert L.gtc_build_octree_batched(None, None, None, 1, 0, 0.0, 1.0, None, None, 0, None) == 1


def _spread3(v):
    out = np.zeros_like(v, dtype=np.uint32)
    for b in range(10):
        out |= ((v >> np.uint32(b)) & np.uint32(1)) << np.uint32(3 * b)
    return out


def test_ref_morton32_to_xyz_host_decode(gtc_mod, oracle):
    """gtc_ref_morton32_to_xyz (morton.rs:43-74, host code, no device): every
    corner of the reference fixture's octree decodes back from its code, and
    random codes under an odd min/range decode exactly as the oracle does
    (separately rounded divide, multiply and add)."""
    L = gtc_mod.lib()
    fx = np.load(os.path.join(REPO, "tests", "golden", "ref_pipeline_32.npz"))
    corners = fx["nodes"].view(np.float32)[:, 8:12]
    q = corners[:, :3].astype(np.uint32)  # min 0, range 1024: a corner is its cell coordinate
    assert np.array_equal(q.astype(np.float32), corners[:, :3])
    codes = _spread3(q[:, 0]) | (_spread3(q[:, 1]) << np.uint32(1)) | (_spread3(q[:, 2]) << np.uint32(2))
    out = np.zeros(4, np.float32)
    for c, corner in zip(codes, corners):
        L.gtc_ref_morton32_to_xyz(out.ctypes.data_as(ctypes.c_void_p), int(c), 0.0, 1024.0)
        assert out.tobytes() == corner.tobytes()
    rng = np.random.default_rng(5)
    for c in rng.integers(0, 1 << 30, 2000, dtype=np.uint32):
        for mn, rg in ((-3.7, 17.3), (0.1, 0.3), (100.0, 1024.0)):
            L.gtc_ref_morton32_to_xyz(out.ctypes.data_as(ctypes.c_void_p), int(c), mn, rg)
            assert out.tobytes() == oracle.morton_to_xyz(int(c), 32, mn, rg).tobytes()
