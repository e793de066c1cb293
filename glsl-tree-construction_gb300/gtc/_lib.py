"""ctypes binding of libgtc.so (include/gtc.h).

The library is the product; this module only declares its C signatures.
Loading fails loudly when libgtc.so is missing: there is no fallback.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

P = ctypes.c_void_p
u8p = ctypes.POINTER(ctypes.c_uint8)
u32, i32, u64, f32, i_, sz = ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_float, ctypes.c_int, ctypes.c_size_t
st = ctypes.c_int  # gtc_status


class OctreeBuffers(ctypes.Structure):
    _fields_ = [
        ("keys", P), ("idx", P), ("prefix_n", P), ("has_leaf_left", P), ("has_leaf_right", P),
        ("left_child", P), ("parent", P), ("edge_count", P), ("node_offsets", P), ("nodes", P),
        ("nodes_capacity", u32), ("counts", P),
    ]


class BatchBuffers(ctypes.Structure):
    _fields_ = [
        ("keys", P), ("idx", P), ("prefix_n", P), ("has_leaf_left", P), ("has_leaf_right", P),
        ("left_child", P), ("parent", P), ("edge_count", P), ("node_offsets", P), ("nodes", P),
        ("nodes_capacity", u32), ("key_offset", P), ("node_offset", P), ("cloud_counts", P),
    ]


SIGNATURES = {
    "gtc_create": (st, [ctypes.POINTER(P), i_]),
    "gtc_destroy": (st, [P]),
    "gtc_status_string": (ctypes.c_char_p, [st]),
    "gtc_last_error": (ctypes.c_char_p, [P]),
    "gtc_device_status": (st, [P, P]),
    "gtc_version": (ctypes.c_char_p, []),
    "gtc_set_spin_limit": (st, [P, u32]),
    "gtc_debug_skip_first_tile": (st, [P]),
    "gtc_set_profiling": (st, [P, i_]),
    "gtc_stage_times": (st, [P, P, P, i_]),
    "gtc_workspace_size": (st, [P, i_, u32, i_, ctypes.POINTER(sz)]),
    "gtc_morton32": (st, [P, P, P, P, u32, f32, f32, P]),
    "gtc_morton64": (st, [P, P, P, P, u32, f32, f32, P]),
    "gtc_global_histogram_u32": (st, [P, P, u32, i_, i_, P, P, sz, P]),
    "gtc_global_histogram_u64": (st, [P, P, u32, i_, i_, P, P, sz, P]),
    "gtc_sort_pairs_u32": (st, [P, P, P, P, P, u32, i_, i_, P, sz, P]),
    "gtc_sort_pairs_u64": (st, [P, P, P, P, P, u32, i_, i_, P, sz, P]),
    "gtc_unique_u32": (st, [P, P, P, u32, P, P, sz, P]),
    "gtc_unique_u64": (st, [P, P, P, u32, P, P, sz, P]),
    "gtc_build_radix_tree_u32": (st, [P, P, i32, P, P, P, P, P, P, P]),
    "gtc_build_radix_tree_u64": (st, [P, P, i32, P, P, P, P, P, P, P]),
    "gtc_edge_count": (st, [P, P, P, P, u32, i_, P]),
    "gtc_partial_sum_u32": (st, [P, P, u32, u32, P, P, sz, P]),
    "gtc_node_offsets": (st, [P, P, u32, P, P, P, sz, P]),
    "gtc_make_octree_u32": (st, [P, P, u32, P, P, P, P, P, f32, f32, i32, P, P, P, P]),
    "gtc_make_octree_u64": (st, [P, P, u32, P, P, P, P, P, f32, f32, i32, P, P, P, P]),
    "gtc_link_octree_u32": (st, [P, P, u32, P, P, P, P, P, i32, P, P, P, P]),
    "gtc_link_octree_u64": (st, [P, P, u32, P, P, P, P, P, i32, P, P, P, P]),
    "gtc_build_octree": (st, [P, P, u32, f32, f32, i_, ctypes.POINTER(OctreeBuffers), P, sz, P]),
    "gtc_build_octree_host": (st, [P, P, u32, f32, f32, i_, P, u32, P]),
    "gtc_build_octree_host_async": (st, [P, P, u32, f32, f32, i_, P, u32, P]),
    "gtc_build_octree_host_wait": (st, [P]),
    "gtc_host_alloc": (st, [ctypes.POINTER(P), sz]),
    "gtc_host_free": (st, [P]),
    "gtc_sort_pairs_u32_noalloc": (st, [P, P, P, P, P, u32, i_, i_, P]),
    "gtc_batched_workspace_size": (st, [u32, u32, ctypes.POINTER(sz)]),
    "gtc_build_octree_batched": (st, [P, P, P, u32, u32, f32, f32, ctypes.POINTER(BatchBuffers), P, sz, P]),
    "gtc_learned_model_create": (st, [P, i_, ctypes.POINTER(P)]),
    "gtc_learned_model_destroy": (st, [P]),
    "gtc_learned_model_params": (st, [P, ctypes.POINTER(i_), ctypes.POINTER(P), ctypes.POINTER(P)]),
    "gtc_learned_model_export": (st, [P, P, P]),
    "gtc_learned_train_u64": (st, [P, P, P, u32, u32, i_, f32, P, P]),
    "gtc_learned_gradient_u64": (st, [P, P, P, u32, u32, i_, P, P, P]),
    "gtc_learned_histogram_u64": (st, [P, P, P, u32, P, P]),
    "gtc_learned_sort_u64": (st, [P, P, P, P, P, P, u32, P, sz, P, P]),
    "gtc_sort_num_variants": (i_, []),
    "gtc_sort_variant_shape": (st, [i_, ctypes.POINTER(i_), ctypes.POINTER(i_)]),
    "gtc_sort_set_variant": (st, [i_, i_]),
    "gtc_sort_get_variant": (i_, [i_]),
    "gtc_tree_set_method": (st, [i_]),
    "gtc_tree_get_method": (i_, []),
    "gtc_set_literal": (st, [u32]),
    "gtc_get_literal": (u32, []),
    "gtc_gather_points": (st, [P, P, u32, P, u32, P, P]),
    "gtc_export_le": (st, [ctypes.c_char_p, P, sz, i_, i_]),
    "gtc_autotune_sort": (st, [P, i_, i_, i_, u32, P, i_, ctypes.POINTER(i_), P]),
    "gtc_autotune_lookup": (i_, [i_, i_, u32]),
    "gtc_autotune_sort_ex": (st, [P, i_, i_, i_, u32, P, i_, ctypes.POINTER(i_), P, ctypes.POINTER(i_), P]),
    "gtc_autotune_lookup_digit_bits": (i_, [i_, i_, u32]),
    "gtc_sort_set_digit_bits": (st, [i_, i_]),
    "gtc_sort_get_digit_bits": (i_, [i_, i_, u32]),
    "gtc_autotune_record": (st, [i_, i_, u32, i_, f32]),
    "gtc_autotune_clear": (st, []),
    "gtc_autotune_entries": (i_, []),
    "gtc_autotune_save": (st, [ctypes.c_char_p]),
    "gtc_autotune_load": (st, [ctypes.c_char_p]),
    "gtc_batched_num_variants": (i_, []),
    "gtc_batched_variant_shape": (st, [i_, ctypes.POINTER(i_), ctypes.POINTER(i_)]),
    "gtc_batched_set_variant": (st, [i_]),
    "gtc_batched_get_variant": (i_, [u32]),
    "gtc_autotune_batched": (st, [P, P, P, u32, u32, f32, f32, ctypes.POINTER(BatchBuffers), P, sz, i_,
                                  ctypes.POINTER(i_), P]),
    "gtc_autotune_lookup_batched": (i_, [u32]),
    "gtc_learned_num_variants": (i_, []),
    "gtc_learned_variant_shape": (st, [i_, ctypes.POINTER(i_), ctypes.POINTER(i_)]),
    "gtc_learned_set_variant": (st, [i_]),
    "gtc_learned_get_variant": (i_, [u32]),
    "gtc_autotune_learned": (st, [P, P, P, P, P, P, u32, P, sz, P, i_, ctypes.POINTER(i_), P]),
    "gtc_autotune_lookup_learned": (i_, [u32]),
    # reference-signature host shims
    "gtc_ref_compute_morton": (st, [P, P, u32, f32, f32, u32]),
    "gtc_ref_morton32_to_xyz": (None, [P, u32, f32, f32]),
    "gtc_ref_histogram": (st, [u32, P, P]),
    "gtc_ref_radix_sort": (st, [P, u32, P, u32]),
    "gtc_ref_unique": (u32, [P, u32]),
    "gtc_ref_build_radix_tree": (st, [i32, P, P, P, P, P, P, u32]),
    "gtc_ref_edge_count": (st, [P, P, P, u32, u32]),
    "gtc_ref_partial_sum": (st, [P, u32, u32, P]),
    "gtc_ref_build_octree": (st, [P, P, P, P, P, P, f32, f32, i32, P, P, P, u32]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = False):
    """Load libgtc.so and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(
                f"libgtc.so not found at {path}: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L
