"""Generates the committed fixtures in tests/golden/.

1. ref_global_hist.txt - the 1024 global-histogram values the reference
   recorded for its own run (radixsort-vulkan/output.txt:7684-8707, printed by
   histogram.rs:265-267 after histogram.comp ran over the keys 10,000,000..1 of
   test_radix_sort, main.rs:189-190).  Needs the reference checkout (read as
   text only); the fixture is committed so tests never read the reference.
2. ref_pipeline_{32,64}.npz - inputs and every stage output of the
   reference's own shaders (oracle/_ref/libref_shaders.so, built from the
   checkout by oracle/ref_shaders.py) driven in main.rs:60-170's order with
   the deviation patches applied: reference-derived vectors that the oracle
   and the CUDA path are checked against on machines without the checkout.
   64-bit codes are not in the reference: that fixture runs the shaders with
   64-bit codes substituted, on codes from the oracle's 64-bit encode.
3. oracle_small_{32,64}.npz - inputs and every stage output of the oracle on
   small seeded inputs, so the oracle built on another machine (the GPU host
   is aarch64) can be checked against the one that produced these.

Usage: python tests/golden/make_golden.py <path-to-reference-checkout>
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "glsl-tree-construction_gb300"))


def make_ref_hist(ref_root: str) -> None:
    path = os.path.join(ref_root, "vulkan", "radixsort-vulkan", "output.txt")
    vals = {}
    with open(path) as f:
        for line in f:
            m = re.match(r"after: b_global_hist\[(\d+)\]: (\d+)", line)
            if m:
                vals[int(m.group(1))] = int(m.group(2))
    assert sorted(vals) == list(range(1024)), "expected 1024 histogram lines"
    with open(os.path.join(HERE, "ref_global_hist.txt"), "w") as f:
        f.write("# radixsort-vulkan/output.txt:7684-8707 (b_global_hist after histogram.comp, keys 10000000..1)\n")
        for i in range(1024):
            f.write(f"{vals[i]}\n")


REF_CASES = {
    32: ("uniform 2^14 points, seed 3", lambda W: W.uniform_points(1 << 14, seed=3)),
    64: ("8-component mixture, sigma 2, 2% noise, 2^14 points, seed 5",
         lambda W: W.gaussian_mixture_points(1 << 14, 8, 2.0, noise=0.02, seed=5)),
}


def make_ref_vectors(ref_root: str) -> None:
    import oracle as O
    from oracle import ref as R
    from gtc import workloads as W

    O.build()
    R.build(ref_root)
    for kb, (what, gen) in REF_CASES.items():
        pts = gen(W)
        out = R.build_octree(pts if kb == 32 else O.morton(pts, 64), kb)
        np.savez_compressed(
            os.path.join(HERE, f"ref_pipeline_{kb}.npz"), what=np.array(what), pts=pts, keys=out["keys"],
            idx=out["idx"], prefix_n=out["prefix_n"], has_leaf_left=out["has_leaf_left"],
            has_leaf_right=out["has_leaf_right"], left_child=out["left_child"], parent=out["parent"],
            edge_count=out["edge_count"], node_offsets=out["node_offsets"],
            nodes=out["nodes"].view(np.int32).reshape(-1, 16))


def make_oracle_vectors() -> None:
    import oracle as O
    from gtc import workloads as W

    cases = {32: W.uniform_points(4096, seed=7), 64: W.gaussian_mixture_points(4096, 4, 3.0, seed=7)}
    for kb, pts in cases.items():
        out, _ = O.build_octree(pts, kb)
        np.savez_compressed(
            os.path.join(HERE, f"oracle_small_{kb}.npz"), pts=pts, keys=out["keys"], idx=out["idx"],
            prefix_n=out["prefix_n"], has_leaf_left=out["has_leaf_left"], has_leaf_right=out["has_leaf_right"],
            left_child=out["left_child"], parent=out["parent"], edge_count=out["edge_count"],
            node_offsets=out["node_offsets"], nodes=out["nodes"].view(np.int32).reshape(-1, 16))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    make_ref_hist(sys.argv[1])
    make_ref_vectors(sys.argv[1])
    make_oracle_vectors()
    print("fixtures written to", HERE)
