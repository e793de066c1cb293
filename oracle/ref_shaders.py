"""Recipe: compile the reference's own shader functions as C++ on the CPU.

TEST INFRASTRUCTURE ONLY.  This builds oracle/_ref/libref_shaders.so from the
GLSL compute shaders of the reference checkout, read where they lie
(<reference>/vulkan/radixsort-vulkan/shader/*.comp).  Nothing is copied into
the repository: the shader text is transformed in memory and written, with the
objects and the library, only under oracle/_ref/ (git-ignored).  The library
is the pin of the oracle (oracle.cpp): tests/test_oracle_ref_pin.py runs both
on the same seeded inputs and compares every stage buffer byte for byte.

The shaders' bodies are plain C-like code.  The transformation is mechanical
and keeps every function body as written:

* `#version` / `#extension` lines are dropped;
* `layout(...) buffer|uniform Name { decls };` blocks become globals (an
  unsized array `T a[]` becomes a pointer `T* a`, `T a[][k]` a pointer to
  rows), which the glue (oracle/ref_glue.cpp) points at the caller's arrays;
* `layout(local_size_x = ...) in;` is dropped;
* `inout T name` parameters become `T& name`;
* `main` is renamed by a macro; the glue runs it with one invocation and a
  stride of 1, so every grid-stride loop visits its indices in order and a
  racy write resolves to the last writer in index order.

GLSL's types and built-ins (uint, vec3/vec4, findMSB, min/max,
gl_GlobalInvocationID ...) come from the shim at the top of ref_glue.cpp.

Variants.  Each shader is compiled once per set of named patches below.  A
patch is an exact text substitution that must match the stated number of
times (the recipe fails loudly otherwise).  D-patches restore the
reference-intent semantics of one deviation row each (D1, D2, D3, D5, D6, D7,
D16); W64 patches widen the codes to the 64-bit / 21-bit-per-axis keys the
reference does not have (types and constants only).  `lit` variants apply no
D-patch, the `fix` variants all of them, and `lit_dK` all but DK, so that each
oracle switch ORC_LITERAL_DK is checked against the reference with exactly
that one deviation left in.

Usage: python oracle/ref_shaders.py <reference-checkout> [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
GEN = os.path.join(OUT, "gen")
LIB_PATH = os.path.join(OUT, "libref_shaders.so")
SHADER_DIR = os.path.join("vulkan", "radixsort-vulkan", "shader")

SHADERS = {
    "morton": "morton.comp",
    "unique": "unique.comp",
    "tree": "build_radix_tree.comp",
    "edge": "edge_count.comp",
    "psum": "partial_sum.comp",
    "octree": "octree.comp",
}

# (old text, new text, expected occurrences), grouped by patch name per stage.
PATCHES = {
    "tree": {
        # D1: the direction difference as a signed int (Karras), not uint8_t.
        "D1": [("const uint8_t direction_difference = delta_diff_right - delta_diff_left;",
                "const int direction_difference = int(delta_diff_right) - int(delta_diff_left);", 1)],
        # D16: the root covers every key, l = n_brt_nodes (= u - 1), not n - 1.
        "D16": [("l = n - 1;", "l = n;", 1)],
        "W64": [("uint codes[];", "uint64_t codes[];", 1),
                ("uint8_t delta_u32(const uint a, const uint b) {",
                 "uint8_t delta_u32(const uint64_t a, const uint64_t b) {", 1),
                ("uint val = a ^ b;", "uint64_t val = a ^ b;", 1),
                ("return uint8_t(32);", "return uint8_t(64);", 1),
                ("return uint8_t(31 - msb);", "return uint8_t(63 - msb);", 1),
                ("const uint code_i = codes[i];", "const uint64_t code_i = codes[i];", 1)],
    },
    "edge": {
        # D2: depth = (prefix_n - A) / 3, A = always-zero high bits of the word.
        "D2": [("int my_depth = prefix_n[i]/3;", "int my_depth = (prefix_n[i]-ref_unused_bits)/3;", 1),
               ("int parent_depth = prefix_n[parent[i]]/3;",
                "int parent_depth = (prefix_n[parent[i]]-ref_unused_bits)/3;", 1)],
    },
    "unique": {
        "W64": [("uint keys[];", "uint64_t keys[];", 1)],
    },
    "octree": {
        # D5 (always applied: the literal form shifts by a negative count, which
        # is undefined): cell sizes relative to the depth of the tree root.
        # REF_DEPTH follows the variant's depth rule (D2 or literal).
        "D5": [("const int root_level=rt_prefixN[i]/3;", "const int root_level=REF_DEPTH(rt_prefixN[0]);", 1)],
        "D2": [("rt_prefixN[i]/3", "REF_DEPTH(rt_prefixN[i])", 4)],
        # D3: radix node k owns slots [ps[k] - edge[k] + 1, ps[k]]; the root owns 0.
        "D3": [("int oct_idx= int(node_offsets[i]);", "int oct_idx= REF_BASE(i);", 1),
               ("const int oct_parent= int(node_offsets[rt_parent]);",
                "const int oct_parent= REF_BASE(rt_parent);", 1),
               ("int bottom_oct_idx= int(node_offsets[rt_node]);", "int bottom_oct_idx= REF_BASE(rt_node);", 2)],
        # D6: SetLeaf sets the leaf-mask bit.
        "D6": [("node.child_leaf_mask&=~(1<<which_child);", "node.child_leaf_mask|=(1<<which_child);", 1)],
        # D7 (always applied where link runs: the literal walk never ends at the
        # root): ancestor walks stop at the root.
        "D7": [("while(rt_node_counts[rt_node]==0){", "while(rt_node_counts[rt_node]==0&&rt_node!=0){", 2),
               ("while(rt_node_counts[rt_parent]==0){", "while(rt_node_counts[rt_parent]==0&&rt_parent!=0){", 1)],
        "W64": [("int codes[];", "int64_t codes[];", 1),
                ("#define morton_bits 30", "#define morton_bits 63", 1),
                ("const int node_prefix=", "const int64_t node_prefix=", 1),
                ("const int top_node_prefix=", "const int64_t top_node_prefix=", 1),
                ("int leaf_prefix=", "int64_t leaf_prefix=", 2),
                ("const int code,", "const int64_t code,", 1),
                ("void m3D_d_magicbits(const int m,", "void m3D_d_magicbits(const int64_t m,", 1),
                ("float morton3D_GetThirdBits(const int m){",
                 "float morton3D_GetThirdBits(const int64_t m){ return ref_third_bits64(m); }\n"
                 "float morton3D_GetThirdBits_w32(const int m){", 1),
                ("const float bit_scale=1024.f;", "const float bit_scale=2097152.f;", 1)],
    },
}

# variant name -> (stage, patches applied, link step run by the glue)
VARIANTS = {
    "ref_morton_lit": ("morton", [], False),
    "ref_unique_lit": ("unique", [], False),
    "ref_unique_w64": ("unique", ["W64"], False),
    "ref_tree_lit": ("tree", [], False),
    "ref_tree_fix": ("tree", ["D1", "D16"], False),
    "ref_tree_lit_d1": ("tree", ["D16"], False),
    "ref_tree_lit_d16": ("tree", ["D1"], False),
    "ref_tree_w64_fix": ("tree", ["D1", "D16", "W64"], False),
    "ref_tree_w64_lit": ("tree", ["W64"], False),
    "ref_edge_lit": ("edge", [], False),
    "ref_edge_fix": ("edge", ["D2"], False),
    "ref_psum_lit": ("psum", [], False),
    "ref_octree_fix": ("octree", ["D5", "D2", "D3", "D6", "D7"], True),
    "ref_octree_lit_d2": ("octree", ["D5", "D3", "D6", "D7"], True),
    "ref_octree_lit_d3": ("octree", ["D5", "D2", "D6", "D7"], True),
    "ref_octree_lit_d6": ("octree", ["D5", "D2", "D3", "D7"], True),
    "ref_octree_w64_fix": ("octree", ["D5", "D2", "D3", "D6", "D7", "W64"], True),
}


def default_reference_root() -> str | None:
    """The reference checkout this recipe reads: $GTC_REFERENCE_ROOT, else the
    build container's checkout at /root/reference; None where neither exists
    (the GPU host has no reference checkout)."""
    for cand in (os.environ.get("GTC_REFERENCE_ROOT"), "/root/reference"):
        if cand and os.path.isdir(os.path.join(cand, SHADER_DIR)):
            return cand
    return None


def _apply(text: str, stage: str, names: list[str]) -> str:
    for name in names:
        for old, new, count in PATCHES[stage][name]:
            got = text.count(old)
            if got != count:
                raise RuntimeError(f"patch {stage}/{name}: expected {count} occurrence(s) of {old!r}, found {got}")
            text = text.replace(old, new)
    return text


_BLOCK = re.compile(r"layout\s*\([^)]*\)\s*(?:buffer|uniform)\s+\w+\s*\{([^}]*)\}\s*;", re.S)
_DECL = re.compile(r"^\s*(\w+)\s+(\w+)\s*((?:\[\s*\d*\s*\])*)\s*$")


def _block_to_globals(m: re.Match) -> str:
    out = []
    for decl in m.group(1).split(";"):
        if not decl.strip():
            continue
        d = _DECL.match(decl)
        if not d:
            raise RuntimeError(f"unrecognised block member {decl.strip()!r}")
        ty, name, dims = d.group(1), d.group(2), re.findall(r"\[\s*(\d*)\s*\]", d.group(3))
        if not dims:
            out.append(f"{ty} {name};")
        elif dims[0] == "" and len(dims) == 1:
            out.append(f"{ty}* {name};")
        elif dims[0] == "" and len(dims) == 2 and dims[1]:
            out.append(f"{ty} (*{name})[{dims[1]}];")
        else:
            raise RuntimeError(f"unsupported block member {decl.strip()!r}")
    return "\n".join(out)


def transform(text: str) -> str:
    """GLSL compute shader text -> C++ source over the shim in ref_glue.cpp."""
    text = re.sub(r"^[ \t]*#[ \t]*(?:version|extension)\b.*$", "", text, flags=re.M)
    text = _BLOCK.sub(_block_to_globals, text)
    text = re.sub(r"layout\s*\([^)]*\)\s*in\s*;", "", text)
    text = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", text)
    return text


def _compile(sym: str, src_inc: str, stage: str, names: list[str], link: bool) -> tuple[str, str, int, str]:
    obj = os.path.join(OUT, sym + ".o")
    defs = [f"-DREF_SYM={sym}", f"-DREF_STAGE_{stage.upper()}", f'-DREF_SHADER_FILE="{src_inc}"']
    defs += [f"-DREF_PATCH_{n}" for n in names]
    if link:
        defs.append("-DREF_RUN_LINK")
    cmd = [os.environ.get("CXX", "g++"), "-O1", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
           "-fno-strict-aliasing", "-w", *defs, "-c", os.path.join(HERE, "ref_glue.cpp"), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return obj, " ".join(cmd), r.returncode, r.stdout + r.stderr


def build(reference_root: str, force: bool = False) -> str:
    """Generate the transformed shader sources and link libref_shaders.so."""
    shader_dir = os.path.join(reference_root, SHADER_DIR)
    if not os.path.isdir(shader_dir):
        raise FileNotFoundError(f"no reference shaders under {shader_dir}")
    glue = os.path.join(HERE, "ref_glue.cpp")
    sources = [os.path.join(shader_dir, f) for f in SHADERS.values()] + [glue, os.path.abspath(__file__)]
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(s) for s in sources)):
        return LIB_PATH
    os.makedirs(GEN, exist_ok=True)
    jobs = []
    for sym, (stage, names, link) in VARIANTS.items():
        with open(os.path.join(shader_dir, SHADERS[stage])) as f:
            text = f.read()
        inc = os.path.join(GEN, sym + ".inc")
        with open(inc, "w") as f:
            f.write(transform(_apply(text, stage, names)))
        jobs.append((sym, inc, stage, names, link))
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda j: _compile(*j), jobs))
    errors = [f"$ {cmd}\n{log}" for _, cmd, rc, log in results if rc != 0]
    if errors:
        raise RuntimeError("reference shader build failed:\n" + "\n".join(errors))
    cmd = [os.environ.get("CXX", "g++"), "-shared", "-o", LIB_PATH, *[o for o, _, _, _ in results]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference shader link failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if not args:
        sys.exit(__doc__)
    print(build(args[0], force="--force" in sys.argv))
